// One shot's device state and launch configuration (the opaque fdtd2d_ctx of
// the C ABI), shared by the single-shot entry points (api.cu) and the batch
// (batch.cu), which owns shots created on its stream and steps them with its
// own kernel.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fdtd2d.h"
#include "internal.h"

struct fdtd2d_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool batch = false;       // member of a batch: stream borrowed, stepped by the batch
  bool solo = false;        // a batch's solo member: own streams, stepped from the batch's run calls
  int nx = 0, ny = 0, pitch = 0, npml = 0, n_steps = 0;
  int n_det = 0, n_comp = 0, record = 0, medium = 0;
  bool dft = false;
  int32_t step = 0;
  int last_cuda = 0;
  int64_t launches = 0;
  fdtd2d::DevShot h{};      // host copy of the device descriptor
  fdtd2d::DevShot* d_shot = nullptr;
  int4* d_units = nullptr;
  int n_units = 0;
  int grid_warps = 0;
  int* d_flag = nullptr;
  int* d_err = nullptr;     // device error word (bounded waits)
  bool tma = false;         // shared-memory staged kernel (uniform medium)
  int tma_shape = 0;        // its launch shape (index into the compiled shapes)
  // multi-row tensor path for the interior (step_tmat.cu) beside the staged
  // kernel on the CPML bands and rows
  bool tmat = false;
  bool tb = false;            // its two-step form (field buffers h.fb[2], h.fb[3])
  int tmat_shape = 0, tmat_ctas = 0, tmat2_ctas = 0;
  int reg[4] = {0, 0, 0, 0};  // interior region [reg0, reg1) x [reg2, reg3)
  int* d_ctr = nullptr;       // the two-step kernel's unit counter
  int4* d_tunits = nullptr;   // interior units (tensor kernel)
  int n_tunits = 0;
  int n_ring = 0;             // ring units at the front of d_tunits (two-step form only)
  int4* d_eunits = nullptr;   // the rest (staged kernel)
  int n_eunits = 0;
  fdtd2d::TensorMaps maps{};
  // the per-step time of the path chosen at create, from its trials (0:
  // not timed here: forced, or the class's choice was remembered)
  float path_ms = 0.f;
  // how its kernel choices were made: 0 timed at create (or forced), 1 a
  // choice kept by this process, 2 a choice read from the persisted file,
  // 3 a default taken without timing (untimed create)
  int choice_src = 0;
  // create without timing trials: a class not timed before takes the
  // default kernel choice (a batch admitting a shot while its device work
  // is in flight)
  bool untimed = false;
  // persistent form (step_persist_kernel): many steps per cooperative
  // launch, its own units and barrier word
  bool persist = false;
  int persist_ctas = 0;
  int4* d_punits = nullptr;
  int n_punits = 0;
  unsigned* d_bar = nullptr;
  // test parameters of its grid barrier (PersistAux::wait_ns, bar_extra)
  unsigned long long wait_ns = 0;
  int bar_extra = 0;
  // the CPML-band kernel runs on a second stream beside the interior one:
  // ev_t marks the interior kernel of the last step, ev_e the CPML kernel,
  // ev_m the shot stream's work before a run
  // (two-step path: ev_t the interior kernel, ev_a the band kernel's first
  // step of the pair, ev_e its second)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_t = nullptr, ev_e = nullptr, ev_m = nullptr, ev_a = nullptr;
  char kernel_name[96] = {0};
  // event timing of the interior kernel (fdtd2d_time_step_kernel)
  bool prof = false;
  std::vector<cudaEvent_t> prof_pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_pending;
  double prof_ms = 0;
  int64_t prof_n = 0, prof_cells = 0;
  int prof_steps = 1;
  // wave-front tracker and line probe
  int n_rc = 0, rc_j_cut = 0;
  float rc_level = 0;
  int *d_rc_scan = nullptr, *d_rc_max = nullptr, *d_spd = nullptr;
  float* d_edge = nullptr;
  int line_n = 0, line_i0 = 0, line_j = 0, line_first = 0, line_last = -1;
  float* d_line = nullptr;
  std::vector<void*> allocs;
  // test parameter: the fail_alloc-th device allocation fails (0: none)
  int fail_alloc = 0, n_alloc = 0;
};

namespace fdtd2d {
// fdtd2d_create; member = true makes a shot for a batch: no launch-shape
// timing, and the batch adopts it (adopt_ctx) once its uploads are done.
// solo = true makes a batch's solo member, which runs beside the batch's
// kernel: never the persistent form, whose cooperative launch wants the
// whole GPU.  untimed = true: no create-time timing trials (a class not
// timed before takes the default kernel choice).
int create_ctx(const fdtd2d_setup* s, int device, bool member, fdtd2d_ctx** out, bool solo = false,
               bool untimed = false);
// The checks fdtd2d_create makes on a setup before it allocates anything
// (FDTD2D_OK, FDTD2D_ERR_INVALID or FDTD2D_ERR_RANGE).
int validate_setup(const fdtd2d_setup* s);
// Hand a member shot to the batch's stream: its own stream is released and
// fdtd2d_run is refused from then on (the batch steps it).
void adopt_ctx(fdtd2d_ctx* c, cudaStream_t batch_stream);
}  // namespace fdtd2d
