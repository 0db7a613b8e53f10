// Batched and continuous stepping of many shots on one GPU (fdtd2d_batch_*).
//
// The reference runs one shot per process (global state, FDTD_2D_Full/
// kernel.cu:1928-2818).  A batch owns many shots, each a full fdtd2d_ctx
// (fields, CPML state, tables, traces and DFT accumulators resident in HBM),
// and advances all of them with one persistent launch per time step of the
// staged kernel (step_tma_batch_kernel): units (shot, band, row range) of every
// unfinished shot are handed out dynamically to the resident CTAs, and each
// shot runs its own step n = global step - its admission step, so shots
// admitted at different times advance together (continuous batching).  Steps
// are issued in blocks of K launches captured once as a CUDA graph; the block
// base lives in device memory and the graph's last node advances it, so the
// same graph serves every block.  Admission is by a device-memory budget.
//
// Host-side state changes (admit, finish, remove) take effect at block
// boundaries: the unit list is rebuilt on the host and uploaded on the batch's
// stream before the next block, which the same graph then reads.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "ctx.h"

using namespace fdtd2d;

namespace {

constexpr int kMaxShots = 512;     // descriptor slots per batch
constexpr int kBlockSteps = 16;    // launches per captured step block

// Misc device words of a batch.
enum Misc : int { kNUnits = 0, kGStep = 1, kCtr0 = 2, kCtr1 = 3, kErr = 4, kMiscWords = 8 };

__global__ void advance_gstep(int* gstep, int k) { *gstep += k; }

struct Member {
  fdtd2d_ctx* ctx = nullptr;
  int64_t bytes = 0;
  int32_t base = 0;     // global steps issued before its first step
  bool live = false;
  bool done = false;    // all its steps issued
};

}  // namespace

struct fdtd2d_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t budget = 0, used = 0;
  std::vector<Member> m;
  std::vector<DevShot> h_shots;        // host copies of the slots' descriptors
  DevShot* d_shots = nullptr;          // [kMaxShots]
  DevShot* d_trial = nullptr;          // [kMaxShots] descriptors for launch-shape trials
  int4* d_units = nullptr;
  int unit_cap = 0, n_units = 0;
  int* d_misc = nullptr;               // Misc words for the real steps
  int* d_tmisc = nullptr;              // and for the trials
  int32_t g = 0;                       // global steps issued
  int shape = 0;
  bool tuned = false;
  int ctas = 0, max_pml = 1;
  bool dirty = true;
  std::map<int, cudaGraphExec_t> graphs;
  int64_t launches = 0;
  int last_cuda = 0;
  char name[64] = {0};
};

namespace {

int fail(fdtd2d_batch* b, cudaError_t e) {
  if (b) b->last_cuda = (int)e;
  return e == cudaErrorMemoryAllocation ? FDTD2D_ERR_NOMEM : FDTD2D_ERR_CUDA;
}

void drop_graphs(fdtd2d_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

// Units of one shot for band width `band` and `rows` rows per unit.
void shot_units(std::vector<int4>& u, int slot, int nx, int ny, int band, int rows) {
  const int bands = (nx + band - 1) / band;
  const int total = ny - 1;
  const int strips = std::max(1, (total + rows - 1) / rows);
  for (int s = 0; s < strips; ++s) {
    const int j0 = (int)((int64_t)total * s / strips), j1 = (int)((int64_t)total * (s + 1) / strips);
    if (j1 <= j0) continue;
    for (int c = 0; c < bands; ++c) u.push_back(make_int4(slot, c * band, j0, j1));
  }
}

// Unit list of every live shot with steps left, for launch shape `shape`:
// rows per unit chosen for about 6 units per resident CTA (16..512 rows).
std::vector<int4> build_units(const fdtd2d_batch* b, int shape, int ctas) {
  const int band = tma_band_cols(shape);
  int64_t band_rows = 0;
  for (const Member& x : b->m)
    if (x.live && !x.done) band_rows += (int64_t)((x.ctx->nx + band - 1) / band) * (x.ctx->ny - 1);
  int rows = (int)std::min<int64_t>(512, std::max<int64_t>(16, (band_rows + 6LL * ctas - 1) / (6LL * ctas)));
  std::vector<int4> u;
  for (int k = 0; k < (int)b->m.size(); ++k) {
    const Member& x = b->m[k];
    if (x.live && !x.done) shot_units(u, k, x.ctx->nx, x.ctx->ny, band, rows);
  }
  return u;
}

int upload_units(fdtd2d_batch* b, const std::vector<int4>& u, int* misc) {
  if ((int)u.size() > b->unit_cap) {
    cudaStreamSynchronize(b->stream);
    if (b->d_units) cudaFree(b->d_units);
    b->d_units = nullptr;
    const int cap = std::max<int>((int)u.size() * 2, 1024);
    cudaError_t e = cudaMalloc(&b->d_units, (size_t)cap * sizeof(int4));
    if (e != cudaSuccess) return fail(b, e);
    b->unit_cap = cap;
    drop_graphs(b);   // they hold the old pointer
  }
  static thread_local std::vector<int4> staging;
  staging = u;   // pageable source: cudaMemcpyAsync stages it before returning
  const int n = (int)u.size();
  cudaError_t e = cudaSuccess;
  if (n) e = cudaMemcpyAsync(b->d_units, staging.data(), (size_t)n * sizeof(int4), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(misc + kNUnits, &n, sizeof(int), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);   // n lives on this stack frame
  if (e != cudaSuccess) return fail(b, e);
  return FDTD2D_OK;
}

// Time every compiled launch shape on the batch's next step (traces and DFT
// off; a step reads one buffer set and overwrites the other, so re-running
// the next step leaves nothing behind) and keep the fastest.
int autotune(fdtd2d_batch* b) {
  std::vector<DevShot> t = b->h_shots;
  for (DevShot& d : t) {
    d.record = 0;
    d.dft = nullptr;
  }
  cudaError_t e = cudaMemcpyAsync(b->d_trial, t.data(), t.size() * sizeof(DevShot), cudaMemcpyHostToDevice,
                                  b->stream);
  if (e != cudaSuccess) return fail(b, e);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  int best_k = 0;
  int rc = FDTD2D_OK;
  for (int k = 0; k < tma_shape_count() && rc == FDTD2D_OK; ++k) {
    const int ctas = tma_batch_resident_ctas(k, b->max_pml, b->device);
    const std::vector<int4> u = build_units(b, k, ctas);
    rc = upload_units(b, u, b->d_tmisc);
    if (rc) break;
    const int g = b->g;
    e = cudaMemcpyAsync(b->d_tmisc + kGStep, &g, sizeof(int), cudaMemcpyHostToDevice, b->stream);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
      if (r == 1) e = cudaEventRecord(e0, b->stream);
      if (e == cudaSuccess)
        e = launch_step_tma_batch(k, b->d_trial, b->d_units, b->d_tmisc + kNUnits, b->d_tmisc + kGStep, 0,
                                  b->d_tmisc + kCtr0, b->max_pml, ctas, b->d_tmisc + kErr, b->stream);
      // the trial re-runs the same step: clear its unit counter between runs
      if (e == cudaSuccess) e = cudaMemsetAsync(b->d_tmisc + kCtr0, 0, 2 * sizeof(int), b->stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) rc = fail(b, e);
    if (rc == FDTD2D_OK && (k == 0 || ms < best)) {
      best = ms;
      best_k = k;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  int err = 0;
  e = cudaMemcpy(&err, b->d_tmisc + kErr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(b, e);
  if (err) return FDTD2D_ERR_TIMEOUT;
  b->shape = best_k;
  b->tuned = true;
  b->dirty = true;
  drop_graphs(b);
  return FDTD2D_OK;
}

cudaError_t capture_block(fdtd2d_batch* b, int K, cudaGraphExec_t* out) {
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < K && e == cudaSuccess; ++k)
    e = launch_step_tma_batch(b->shape, b->d_shots, b->d_units, b->d_misc + kNUnits, b->d_misc + kGStep, k,
                              b->d_misc + kCtr0, b->max_pml, b->ctas, b->d_misc + kErr, b->stream);
  if (e == cudaSuccess) {
    advance_gstep<<<1, 1, 0, b->stream>>>(b->d_misc + kGStep, K);
    e = cudaGetLastError();
  }
  const cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
  if (e == cudaSuccess) e = ee;
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  return e;
}

}  // namespace

extern "C" {

int fdtd2d_batch_create(int device, int64_t hbm_budget_bytes, fdtd2d_batch** out) {
  if (!out) return FDTD2D_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FDTD2D_ERR_NODEVICE;
  if (device < 0 || device >= ndev) return FDTD2D_ERR_INVALID;
  fdtd2d_batch* b = new (std::nothrow) fdtd2d_batch();
  if (!b) return FDTD2D_ERR_NOMEM;
  b->device = device;
  cudaSetDevice(device);
  if (hbm_budget_bytes <= 0) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    hbm_budget_bytes = (int64_t)(free_b * 0.9);
  }
  b->budget = hbm_budget_bytes;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_shots, kMaxShots * sizeof(DevShot));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_trial, kMaxShots * sizeof(DevShot));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_misc, 2 * kMiscWords * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(b->d_misc, 0, 2 * kMiscWords * sizeof(int));
  if (e != cudaSuccess) {
    fdtd2d_batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? FDTD2D_ERR_NOMEM : FDTD2D_ERR_CUDA;
  }
  b->d_tmisc = b->d_misc + kMiscWords;
  b->h_shots.resize(kMaxShots);
  std::memset(b->h_shots.data(), 0, kMaxShots * sizeof(DevShot));
  *out = b;
  return FDTD2D_OK;
}

int fdtd2d_batch_add(fdtd2d_batch* b, const fdtd2d_setup* s, int32_t* shot) {
  if (!b || !s || !shot) return FDTD2D_ERR_INVALID;
  *shot = -1;
  if (s->medium != FDTD2D_MEDIUM_UNIFORM || s->npml > tma_max_pml() || s->n_rc > 0 || s->line_n > 0)
    return FDTD2D_ERR_INVALID;
  const int64_t bytes = fdtd2d_device_bytes(s);
  if (bytes < 0) return FDTD2D_ERR_INVALID;
  if (b->used + bytes > b->budget) return FDTD2D_ERR_BUDGET;
  int slot = -1;
  for (int k = 0; k < (int)b->m.size(); ++k)
    if (!b->m[k].live) { slot = k; break; }
  if (slot < 0) {
    if ((int)b->m.size() >= kMaxShots) return FDTD2D_ERR_BUDGET;
    b->m.emplace_back();
    slot = (int)b->m.size() - 1;
  }
  fdtd2d_ctx* c = nullptr;
  const int rc = create_ctx(s, b->device, true, &c);   // uploads on its own stream
  if (rc) return rc;
  adopt_ctx(c, b->stream);
  Member& x = b->m[slot];
  x.ctx = c;
  x.bytes = bytes;
  x.base = b->g;
  x.live = true;
  x.done = false;
  c->h.base_n = b->g;
  b->h_shots[slot] = c->h;
  cudaSetDevice(b->device);
  cudaError_t e = cudaMemcpyAsync(b->d_shots + slot, &b->h_shots[slot], sizeof(DevShot), cudaMemcpyHostToDevice,
                                  b->stream);
  if (e != cudaSuccess) return fail(b, e);
  b->used += bytes;
  if (s->npml > b->max_pml) {
    b->max_pml = s->npml;
    drop_graphs(b);
  }
  b->dirty = true;
  *shot = slot;
  return FDTD2D_OK;
}

int fdtd2d_batch_run(fdtd2d_batch* b, int32_t n_steps) {
  if (!b || n_steps < 0) return FDTD2D_ERR_INVALID;
  cudaSetDevice(b->device);
  while (n_steps > 0) {
    bool any = false;
    for (const Member& x : b->m) any = any || (x.live && !x.done);
    if (!any) return FDTD2D_OK;
    if (!b->tuned) {
      const char* t = std::getenv("FDTD2D_TMA");
      int w = 0, st = 0;
      if (t && std::sscanf(t, "%d,%d", &w, &st) == 2 && tma_shape_find(w, st) >= 0) {
        b->shape = tma_shape_find(w, st);
        b->tuned = true;
      } else {
        const int rc = autotune(b);
        if (rc) return rc;
      }
    }
    const int ctas = tma_batch_resident_ctas(b->shape, b->max_pml, b->device);
    if (ctas != b->ctas) {
      b->ctas = ctas;
      drop_graphs(b);
    }
    if (b->dirty) {
      const std::vector<int4> u = build_units(b, b->shape, b->ctas);
      const int rc = upload_units(b, u, b->d_misc);
      if (rc) return rc;
      b->n_units = (int)u.size();
      b->dirty = false;
      // the shape's counters may hold a trial's values
      cudaError_t e = cudaMemsetAsync(b->d_misc + kCtr0, 0, 2 * sizeof(int), b->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_misc + kGStep, &b->g, sizeof(int), cudaMemcpyHostToDevice, b->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess) return fail(b, e);
    }
    const int K = std::min<int>(n_steps, kBlockSteps);
    auto it = b->graphs.find(K);
    if (it == b->graphs.end()) {
      cudaGraphExec_t ge = nullptr;
      const cudaError_t e = capture_block(b, K, &ge);
      if (e != cudaSuccess) return fail(b, e);
      it = b->graphs.emplace(K, ge).first;
    }
    const cudaError_t e = cudaGraphLaunch(it->second, b->stream);
    if (e != cudaSuccess) return fail(b, e);
    b->g += K;
    b->launches += K;
    n_steps -= K;
    for (Member& x : b->m) {
      if (!x.live) continue;
      x.ctx->step = std::min(x.ctx->n_steps, std::max(0, b->g - x.base));
      if (!x.done && x.ctx->step >= x.ctx->n_steps) {
        x.done = true;
        b->dirty = true;
      }
    }
  }
  return FDTD2D_OK;
}

int fdtd2d_batch_synchronize(fdtd2d_batch* b) {
  if (!b) return FDTD2D_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return fail(b, e);
  int err = 0;
  e = cudaMemcpy(&err, b->d_misc + kErr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(b, e);
  return err ? FDTD2D_ERR_TIMEOUT : FDTD2D_OK;
}

fdtd2d_ctx* fdtd2d_batch_shot(fdtd2d_batch* b, int32_t shot) {
  if (!b || shot < 0 || shot >= (int)b->m.size() || !b->m[shot].live) return nullptr;
  return b->m[shot].ctx;
}

int32_t fdtd2d_batch_shot_step(const fdtd2d_batch* b, int32_t shot) {
  if (!b || shot < 0 || shot >= (int)b->m.size() || !b->m[shot].live) return -1;
  return b->m[shot].ctx->step;
}

int fdtd2d_batch_remove(fdtd2d_batch* b, int32_t shot) {
  if (!b || shot < 0 || shot >= (int)b->m.size() || !b->m[shot].live) return FDTD2D_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  Member& x = b->m[shot];
  fdtd2d_destroy(x.ctx);
  b->used -= x.bytes;
  x = Member();
  b->dirty = true;
  return FDTD2D_OK;
}

int64_t fdtd2d_batch_free_bytes(const fdtd2d_batch* b) { return b ? b->budget - b->used : -1; }

int64_t fdtd2d_batch_launch_count(const fdtd2d_batch* b) { return b ? b->launches : -1; }

const char* fdtd2d_batch_kernel_name(const fdtd2d_batch* b) {
  if (!b) return "";
  int w = 0, st = 0;
  tma_shape_dims(b->shape, &w, &st);
  std::snprintf(const_cast<char*>(b->name), sizeof b->name, "step_tma_batch_kernel<%d,%d>", w, st);
  return b->name;
}

int fdtd2d_batch_destroy(fdtd2d_batch* b) {
  if (!b) return FDTD2D_ERR_INVALID;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (Member& x : b->m)
    if (x.live) fdtd2d_destroy(x.ctx);
  drop_graphs(b);
  if (b->d_units) cudaFree(b->d_units);
  if (b->d_shots) cudaFree(b->d_shots);
  if (b->d_trial) cudaFree(b->d_trial);
  if (b->d_misc) cudaFree(b->d_misc);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return FDTD2D_OK;
}

}  // extern "C"
