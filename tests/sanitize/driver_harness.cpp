// Sanitizer harness of the drop-in driver's host code (test infrastructure,
// built by tests/test_sanitize_cpu.py): fdtd2d_run_settings end to end on a
// Settings.ini with the device entry points replaced by a host stand-in that
// checks each call's ranges and fills the read buffers with deterministic
// values (no GPU, no physics).  Exercises the parsing, the run schedule
// (slices, TOF window, S2D second shot), the trace, slice, tracker and TOF
// writers.  Prints "DRIVER OK" when the run returns 0.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/fdtd2d.h"

struct fdtd2d_ctx {
  int nx, ny, npml, n_steps, n_det, n_comp, n_rc, line_n, line_first, line_last;
  int32_t step;
};

namespace {
bool range_ok(const fdtd2d_ctx* c, int32_t n0, int32_t n1) {
  return c && n0 >= 1 && n1 >= n0 && n1 <= c->n_steps && n1 <= c->step;
}
float wave(long k) { return (float)std::sin(0.001 * (double)k) * 0.5f; }
}  // namespace

extern "C" {
int fdtd2d_create(const fdtd2d_setup* s, int, fdtd2d_ctx** out) {
  if (!s || !out || s->nx < 8 || s->ny < 8 || s->n_steps < 1) return FDTD2D_ERR_INVALID;
  *out = new fdtd2d_ctx{s->nx, s->ny, s->npml, s->n_steps, s->n_det, s->n_comp, s->n_rc,
                        s->line_n, s->line_first, s->line_last, 0};
  return FDTD2D_OK;
}
int fdtd2d_destroy(fdtd2d_ctx* c) {
  delete c;
  return FDTD2D_OK;
}
int fdtd2d_run(fdtd2d_ctx* c, int32_t n_first, int32_t n_last) {
  if (!c || n_first != c->step + 1 || n_last < n_first - 1 || n_last > c->n_steps) return FDTD2D_ERR_RANGE;
  c->step = n_last;
  return FDTD2D_OK;
}
int fdtd2d_synchronize(fdtd2d_ctx* c) { return c ? FDTD2D_OK : FDTD2D_ERR_INVALID; }
int fdtd2d_read_traces(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* det, float* cez, float* chx, float* chy) {
  if (!range_ok(c, n0, n1)) return FDTD2D_ERR_RANGE;
  const long rows = n1 - n0 + 1;
  for (long k = 0; k < rows * c->n_det; ++k)
    if (det) det[k] = wave(k);
  for (long k = 0; k < rows * c->n_comp; ++k) {
    if (cez) cez[k] = wave(k);
    if (chx) chx[k] = wave(k) / 377.f;
    if (chy) chy[k] = -wave(k) / 377.f;
  }
  return FDTD2D_OK;
}
int fdtd2d_read_rc(fdtd2d_ctx* c, int32_t n0, int32_t n1, int32_t* spd) {
  if (!range_ok(c, n0, n1) || c->n_rc <= 0 || !spd) return FDTD2D_ERR_RANGE;
  for (long t = 0; t < n1 - n0 + 1; ++t)
    for (int l = 0; l < c->n_rc; ++l) spd[t * c->n_rc + l] = 1 + (int)((t + n0 + 7 * l) % (c->ny - 3));
  return FDTD2D_OK;
}
int fdtd2d_read_line(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* out) {
  if (!c || !out || c->line_n <= 0 || n0 < c->line_first || n1 > c->line_last || n1 < n0 || n1 > c->step)
    return FDTD2D_ERR_RANGE;
  for (long k = 0; k < (long)(n1 - n0 + 1) * c->line_n; ++k) out[k] = wave(k + 3 * n0);
  return FDTD2D_OK;
}
int fdtd2d_read_field(fdtd2d_ctx* c, int which, float* host) {
  if (!c || !host) return FDTD2D_ERR_INVALID;
  long rows = c->ny, cols = c->nx;
  if (which == FDTD2D_FIELD_HX) rows = c->ny - 1;
  else if (which == FDTD2D_FIELD_HY) cols = c->nx - 1;
  else if (which != FDTD2D_FIELD_EZ && which != FDTD2D_FIELD_JZ) return FDTD2D_ERR_INVALID;
  for (long k = 0; k < rows * cols; ++k) host[k] = wave(k + c->step);
  return FDTD2D_OK;
}
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const int rc = fdtd2d_run_settings(argv[1], argv[2], 0);
  std::printf("run_settings %s: %d\n", argv[1], rc);
  if (rc != 0) return 1;
  std::printf("DRIVER OK\n");
  return 0;
}
