// fdtd2d: the reference program's command line, on the GB300 library.
// Usage: fdtd2d [Settings.ini] [out_dir] [gpu]
// Defaults follow the reference: Settings.ini in the working directory,
// outputs in the working directory, GPU_device from the file when no gpu
// argument is given (FDTD_2D_Full/FDTD_cuda.cu:20-30, 384-387).
#include <cstdio>
#include <cstdlib>

#include "fdtd2d.h"

int main(int argc, char** argv) {
  const char* ini = argc > 1 ? argv[1] : "Settings.ini";
  const char* out = argc > 2 ? argv[2] : "";
  const int dev = argc > 3 ? std::atoi(argv[3]) : -1;
  const int rc = fdtd2d_run_settings(ini, out, dev);
  if (rc != FDTD2D_OK) {
    std::fprintf(stderr, "fdtd2d: %s (%d)\n", fdtd2d_strerror(rc), rc);
    return 1;
  }
  return 0;
}
