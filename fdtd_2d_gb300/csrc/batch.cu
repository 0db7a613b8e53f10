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
  // A solo member is a full single shot on its own streams (the tensor path:
  // two steps per pass where it wins), stepped by fdtd2d_run from the batch's
  // run calls; `ev` holds the events recorded after its recent run calls on
  // its stream, oldest first.
  bool solo = false;
  std::vector<cudaEvent_t> ev;
  int64_t seq = 0;      // admission order
};

// Solo members stepped at a time (the oldest admitted first; the others
// wait): a few two-step chains keep the GPU busy, and every extra one only
// adds streams and shares the device among more shots, which delays each.
// FDTD2D_BATCH_SOLO_ACTIVE overrides it.
int solo_active() {
  const char* v = std::getenv("FDTD2D_BATCH_SOLO_ACTIVE");
  const int k = v ? std::atoi(v) : 8;
  return k > 0 ? k : 8;
}

// Grids of at least this many cells (2^21, about 1448^2) join a batch as
// solo members (their own tensor-path launches fill the GPU); smaller ones
// share the batch kernel.  FDTD2D_BATCH_SOLO_CELLS overrides it (0: none
// solo).
int64_t solo_cells() {
  const char* v = std::getenv("FDTD2D_BATCH_SOLO_CELLS");
  return v ? std::atoll(v) : (int64_t)1 << 21;
}

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
  int64_t admitted = 0;                // admissions so far (Member::seq)
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
    if (x.live && !x.done && !x.solo) band_rows += (int64_t)((x.ctx->nx + band - 1) / band) * (x.ctx->ny - 1);
  int rows = (int)std::min<int64_t>(512, std::max<int64_t>(16, (band_rows + 6LL * ctas - 1) / (6LL * ctas)));
  std::vector<int4> u;
  for (int k = 0; k < (int)b->m.size(); ++k) {
    const Member& x = b->m[k];
    if (x.live && !x.done && !x.solo) shot_units(u, k, x.ctx->nx, x.ctx->ny, band, rows);
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

int add_solo(fdtd2d_batch* b, const fdtd2d_setup* s, int64_t bytes, int32_t* shot) {
  int slot = -1;
  for (int k = 0; k < (int)b->m.size(); ++k)
    if (!b->m[k].live) { slot = k; break; }
  if (slot < 0) {
    if ((int)b->m.size() >= kMaxShots) return FDTD2D_ERR_BUDGET;
    b->m.emplace_back();
    slot = (int)b->m.size() - 1;
  }
  // Its own streams; its kernel choice is timed at create while the batch
  // has no device work in flight.  Timing trials run beside other shots'
  // kernels measure nothing useful, and on a GB300 with some 150 shots in
  // flight a trial kernel's bounded wait ran out; such an admission takes
  // the class's stored choice or the default one.
  bool busy = cudaStreamQuery(b->stream) == cudaErrorNotReady;
  for (const Member& m : b->m)
    if (m.live && m.solo && !busy)
      busy = cudaStreamQuery(m.ctx->stream) == cudaErrorNotReady ||
             (m.ctx->side && cudaStreamQuery(m.ctx->side) == cudaErrorNotReady);
  cudaGetLastError();
  fdtd2d_ctx* c = nullptr;
  const int rc = create_ctx(s, b->device, false, &c, true, busy);
  if (rc) return rc;
  // the bytes it holds: two more field buffers on the two-step path
  if (c->tb) bytes += 2 * c->h.cells * 4 * store_bytes(c->h.store);
  Member& x = b->m[slot];
  x.ctx = c;
  x.bytes = bytes;
  x.base = b->g;
  x.live = true;
  x.done = c->n_steps <= 0;
  x.solo = true;
  x.seq = b->admitted++;
  b->used += bytes;
  *shot = slot;
  return FDTD2D_OK;
}

// Issue up to n more steps of the solo_active() oldest unfinished solo
// members on their own streams (the host does not wait), keeping at most two
// run calls of each in flight.
int run_solo(fdtd2d_batch* b, int32_t n) {
  // the solo_active() oldest unfinished solo members
  std::vector<std::pair<int64_t, int>> order;
  for (int k = 0; k < (int)b->m.size(); ++k) {
    const Member& x = b->m[k];
    if (x.live && x.solo && !x.done) order.push_back({x.seq, k});
  }
  std::sort(order.begin(), order.end());
  if ((int)order.size() > solo_active()) order.resize(solo_active());
  for (const auto& o : order) {
    Member& x = b->m[o.second];
    fdtd2d_ctx* c = x.ctx;
    while (x.ev.size() >= 2) {
      const cudaError_t e = cudaEventSynchronize(x.ev.front());
      if (e != cudaSuccess) return fail(b, e);
      cudaEventDestroy(x.ev.front());
      x.ev.erase(x.ev.begin());
    }
    const int32_t last = std::min(c->n_steps, c->step + n);
    const int64_t l0 = c->launches;
    const int rc = fdtd2d_run(c, c->step + 1, last);
    if (rc) {
      b->last_cuda = c->last_cuda;
      return rc;
    }
    b->launches += c->launches - l0;
    cudaEvent_t e = nullptr;
    cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventRecord(e, c->stream);
    if (ce != cudaSuccess) return fail(b, ce);
    x.ev.push_back(e);
    if (c->step >= c->n_steps) x.done = true;
  }
  return FDTD2D_OK;
}

// A solo member whose steps have all been issued and have completed.
bool solo_complete(const Member& x) {
  return x.solo && x.done && (x.ev.empty() || cudaEventQuery(x.ev.back()) == cudaSuccess);
}

void release_events(Member& x) {
  for (cudaEvent_t e : x.ev) cudaEventDestroy(e);
  x.ev.clear();
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
  // host descriptors first: a failure here leaves no device resource behind
  try {
    b->h_shots.resize(kMaxShots);
  } catch (...) {
    delete b;
    return FDTD2D_ERR_NOMEM;
  }
  std::memset(b->h_shots.data(), 0, kMaxShots * sizeof(DevShot));
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
  *out = b;
  return FDTD2D_OK;
}

static int fdtd2d_batch_add_body(fdtd2d_batch* b, const fdtd2d_setup* s, int32_t* shot);

// The entry point: its body, below, runs behind abi_guard.
int fdtd2d_batch_add(fdtd2d_batch* b, const fdtd2d_setup* s, int32_t* shot) {
  return abi_guard([&] { return fdtd2d_batch_add_body(b, s, shot); });
}

static int fdtd2d_batch_add_body(fdtd2d_batch* b, const fdtd2d_setup* s, int32_t* shot) {
  if (!b || !s || !shot) return FDTD2D_ERR_INVALID;
  *shot = -1;
  if (s->medium != FDTD2D_MEDIUM_UNIFORM || s->npml > tma_max_pml() || s->n_rc > 0 || s->line_n > 0)
    return FDTD2D_ERR_INVALID;
  const int64_t bytes = fdtd2d_device_bytes(s);
  if (bytes < 0) return FDTD2D_ERR_INVALID;
  if (b->used + bytes > b->budget) return FDTD2D_ERR_BUDGET;
  // A large grid goes solo when it fits with the two extra field buffers of
  // the two-step path.  The batch kernel steps FP32 fields only, so a shot
  // with 16-bit storage is a solo member whatever its size (the single-shot
  // path, 16-bit forms included), admitted once those buffers fit too.
  const int64_t field_buf = (int64_t)buffer_floats(s->nx, s->ny) * 4 * store_bytes(s->storage);
  const int64_t cells = (int64_t)s->nx * s->ny;
  const int64_t sc = solo_cells();
  const bool fits2 = b->used + bytes + 2 * field_buf <= b->budget;
  if (s->storage != FDTD2D_STORE_F32) return fits2 ? add_solo(b, s, bytes, shot) : FDTD2D_ERR_BUDGET;
  if (sc > 0 && cells >= sc && fits2) return add_solo(b, s, bytes, shot);
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

static int fdtd2d_batch_run_body(fdtd2d_batch* b, int32_t n_steps);

// The entry point: its body, below, runs behind abi_guard.
int fdtd2d_batch_run(fdtd2d_batch* b, int32_t n_steps) {
  return abi_guard([&] { return fdtd2d_batch_run_body(b, n_steps); });
}

static int fdtd2d_batch_run_body(fdtd2d_batch* b, int32_t n_steps) {
  if (!b || n_steps < 0) return FDTD2D_ERR_INVALID;
  cudaSetDevice(b->device);
  if (n_steps > 0) {
    const int rc = run_solo(b, n_steps);
    if (rc) return rc;
  }
  while (n_steps > 0) {
    bool any = false;
    for (const Member& x : b->m) any = any || (x.live && !x.done && !x.solo);
    if (!any) return FDTD2D_OK;
    if (!b->tuned) {
      const int forced = tma_shape_parse(std::getenv("FDTD2D_TMA"));
      if (forced >= 0) {
        b->shape = forced;
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
      if (!x.live || x.solo) continue;
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
  for (Member& x : b->m)
    if (x.live && x.solo) {
      const int rc = fdtd2d_synchronize(x.ctx);
      if (rc) return rc;
    }
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
  Member& x = b->m[shot];
  fdtd2d_destroy(x.ctx);   // memory released behind the queued kernels (a solo shot waits for its own)
  release_events(x);
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
    if (x.live) {
      fdtd2d_destroy(x.ctx);
      release_events(x);
    }
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

// ---- Serving loop -----------------------------------------------------------
//
// A request loop on top of a batch: shots are queued as they arrive, admitted
// in arrival order while they fit the device-memory budget, stepped together
// in blocks, and retired as soon as the block that issued their last step has
// completed on the GPU (a CUDA event per block; no device-wide wait): their
// DFT accumulators and Ez traces are copied out and their memory is released
// behind the queued kernels.  The caller drives it with fdtd2d_server_step and
// collects results with fdtd2d_server_pop.

namespace {

struct Queued {
  const fdtd2d_setup* s;
  int64_t tag;
};
struct Running {
  int32_t slot;
  int64_t tag;
  int32_t last_g;   // global step that completes the shot
};
struct Finished {
  int64_t tag;
  int32_t n_det, n_steps;
  std::vector<double> dft;    // re, im per detector
  std::vector<float> trace;   // [n_steps][n_det] Ez samples
};

}  // namespace

struct fdtd2d_server {
  fdtd2d_batch* b = nullptr;
  int32_t block = 64;
  std::vector<Queued> queue;            // FIFO (front = index 0)
  std::vector<Running> running;
  std::vector<Finished> finished;       // FIFO
  std::vector<std::pair<int32_t, cudaEvent_t>> blocks;   // (global step after the block, event)
  std::vector<cudaEvent_t> spare;
  int32_t g_complete = 0;               // global steps known complete on the GPU
};

namespace {

cudaEvent_t take_event(fdtd2d_server* s) {
  if (!s->spare.empty()) {
    cudaEvent_t e = s->spare.back();
    s->spare.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  return e;
}

// Retire every running shot whose last step has completed.
int retire(fdtd2d_server* s, int* n_done) {
  fdtd2d_batch* b = s->b;
  size_t k = 0;
  for (; k < s->blocks.size(); ++k) {
    if (cudaEventQuery(s->blocks[k].second) != cudaSuccess) break;
    s->g_complete = std::max(s->g_complete, s->blocks[k].first);
    s->spare.push_back(s->blocks[k].second);
  }
  s->blocks.erase(s->blocks.begin(), s->blocks.begin() + k);
  for (size_t r = 0; r < s->running.size();) {
    const Running x = s->running[r];
    const Member& mem = b->m[x.slot];
    if (mem.solo ? !solo_complete(mem) : x.last_g > s->g_complete) {
      ++r;
      continue;
    }
    fdtd2d_ctx* c = b->m[x.slot].ctx;
    // A shot whose kernels gave up on a bounded wait has skipped work: its
    // results are not handed out (the batch kernel's error word for its
    // members, a solo member's own one), and the call reports the timeout.
    // A solo member's word was allocated and zeroed on its own stream
    // (stream-ordered, from the pool): it is read in that stream's order,
    // which has completed.  The batch's word comes from cudaMalloc and a
    // synchronous memset; reading it does not wait for the queued blocks.
    int derr = 0;
    cudaError_t re;
    if (mem.solo) {
      re = cudaMemcpyAsync(&derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
      if (re == cudaSuccess) re = cudaStreamSynchronize(c->stream);
    } else {
      re = cudaMemcpy(&derr, b->d_misc + kErr, sizeof(int), cudaMemcpyDeviceToHost);
    }
    if (re != cudaSuccess) return fail(b, re);
    if (derr) return FDTD2D_ERR_TIMEOUT;
    Finished f;
    f.tag = x.tag;
    f.n_det = c->n_det;
    f.n_steps = c->n_steps;
    cudaError_t e = cudaSuccess;
    if (c->dft && c->n_det > 0) {
      f.dft.resize((size_t)2 * c->n_det);
      e = cudaMemcpy(f.dft.data(), c->h.dft, f.dft.size() * sizeof(double), cudaMemcpyDeviceToHost);
    }
    if (e == cudaSuccess && c->record && c->n_det > 0) {
      f.trace.resize((size_t)c->n_steps * c->n_det);
      e = cudaMemcpy(f.trace.data(), c->h.trace, f.trace.size() * sizeof(float), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return fail(b, e);
    fdtd2d_batch_remove(b, x.slot);
    s->finished.push_back(std::move(f));
    s->running.erase(s->running.begin() + r);
    ++*n_done;
  }
  return FDTD2D_OK;
}

}  // namespace

extern "C" {

int fdtd2d_server_create(int device, int64_t hbm_budget_bytes, int32_t block_steps, fdtd2d_server** out) {
  if (!out || block_steps < 1) return FDTD2D_ERR_INVALID;
  *out = nullptr;
  fdtd2d_server* s = new (std::nothrow) fdtd2d_server();
  if (!s) return FDTD2D_ERR_NOMEM;
  const int rc = fdtd2d_batch_create(device, hbm_budget_bytes, &s->b);
  if (rc) {
    delete s;
    return rc;
  }
  s->block = block_steps;
  *out = s;
  return FDTD2D_OK;
}

static int fdtd2d_server_submit_body(fdtd2d_server* s, const fdtd2d_setup* setup, int64_t tag);

// The entry point: its body, below, runs behind abi_guard.
int fdtd2d_server_submit(fdtd2d_server* s, const fdtd2d_setup* setup, int64_t tag) {
  return abi_guard([&] { return fdtd2d_server_submit_body(s, setup, tag); });
}

static int fdtd2d_server_submit_body(fdtd2d_server* s, const fdtd2d_setup* setup, int64_t tag) {
  if (!s || !setup) return FDTD2D_ERR_INVALID;
  if (setup->medium != FDTD2D_MEDIUM_UNIFORM || setup->npml > tma_max_pml() || setup->n_rc > 0 ||
      setup->line_n > 0)
    return FDTD2D_ERR_INVALID;
  // a setup fdtd2d_create would refuse is refused here, not at admission
  const int vrc = validate_setup(setup);
  if (vrc) return vrc;
  const int64_t bytes = fdtd2d_device_bytes(setup);
  if (bytes < 0) return FDTD2D_ERR_INVALID;
  // could never be admitted (a 16-bit shot also needs its two extra buffers)
  const int64_t extra = setup->storage == FDTD2D_STORE_F32
                            ? 0 : 2 * (int64_t)buffer_floats(setup->nx, setup->ny) * 4 * store_bytes(setup->storage);
  if (bytes + extra > s->b->budget) return FDTD2D_ERR_BUDGET;
  s->queue.push_back({setup, tag});
  return FDTD2D_OK;
}

static int fdtd2d_server_step_body(fdtd2d_server* s);

// The entry point: its body, below, runs behind abi_guard.
int fdtd2d_server_step(fdtd2d_server* s) {
  return abi_guard([&] { return fdtd2d_server_step_body(s); });
}

static int fdtd2d_server_step_body(fdtd2d_server* s) {
  if (!s) return FDTD2D_ERR_INVALID;
  fdtd2d_batch* b = s->b;
  cudaSetDevice(b->device);
  int n_done = 0;
  // 1. admit in arrival order while the head fits (uploads overlap the queued
  // steps).  Each shot leaves the queue as soon as it is admitted and
  // recorded, so an error on a later one returns with every earlier one
  // running exactly once; the failing shot stays at the head of the queue.
  // The running list grows before the add, so nothing can throw between a
  // successful add and its record.
  while (!s->queue.empty()) {
    s->running.reserve(s->running.size() + 1);
    const Queued head = s->queue.front();
    int32_t slot = -1;
    const int arc = fdtd2d_batch_add(b, head.s, &slot);
    if (arc == FDTD2D_ERR_BUDGET) break;
    if (arc) return arc;
    const fdtd2d_ctx* c = b->m[slot].ctx;
    s->running.push_back({slot, head.tag, b->m[slot].base + c->n_steps});
    s->queue.erase(s->queue.begin());
  }
  // 2. retire what the GPU has finished
  int rc = retire(s, &n_done);
  if (rc) return rc;
  // 3. issue one block while any shot has steps left
  bool steps_left = false, solo_left = false;
  for (const Running& x : s->running) {
    const Member& mem = b->m[x.slot];
    if (mem.solo)
      solo_left = solo_left || !mem.done;
    else
      steps_left = steps_left || x.last_g > b->g;
  }
  if (solo_left && !steps_left) {
    // only solo members have steps left: issue theirs, then wait for the
    // oldest run call of one of them instead of spinning
    rc = run_solo(b, s->block);
    if (rc) return rc;
    for (const Running& x : s->running) {
      Member& mem = b->m[x.slot];
      if (mem.solo && !mem.ev.empty()) {
        const cudaError_t we = cudaEventSynchronize(mem.ev.front());
        if (we != cudaSuccess) return fail(b, we);
        break;
      }
    }
    rc = retire(s, &n_done);
    if (rc) return rc;
  } else if (steps_left) {
    rc = fdtd2d_batch_run(b, s->block);
    if (rc) return rc;
    cudaEvent_t e = take_event(s);
    const cudaError_t ce = cudaEventRecord(e, b->stream);
    if (ce != cudaSuccess) return fail(b, ce);
    s->blocks.push_back({b->g, e});
    // keep at most two blocks ahead of the GPU
    while (s->blocks.size() > 2) {
      const cudaError_t we = cudaEventSynchronize(s->blocks.front().second);
      if (we != cudaSuccess) return fail(b, we);
      rc = retire(s, &n_done);
      if (rc) return rc;
    }
  } else if (!s->blocks.empty()) {
    // nothing more to issue: wait for the oldest block instead of spinning
    const cudaError_t we = cudaEventSynchronize(s->blocks.front().second);
    if (we != cudaSuccess) return fail(b, we);
    rc = retire(s, &n_done);
    if (rc) return rc;
  } else {
    // only solo members still running, all issued: wait for one of them
    for (const Running& x : s->running) {
      const Member& mem = b->m[x.slot];
      if (mem.solo && !mem.ev.empty()) {
        const cudaError_t we = cudaEventSynchronize(mem.ev.back());
        if (we != cudaSuccess) return fail(b, we);
        break;
      }
    }
    rc = retire(s, &n_done);
    if (rc) return rc;
  }
  int err = 0;
  if (cudaMemcpy(&err, b->d_misc + kErr, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && err)
    return FDTD2D_ERR_TIMEOUT;
  return n_done;
}

int fdtd2d_server_pop(fdtd2d_server* s, int64_t* tag, int32_t* n_det, int32_t* n_steps, double* dft,
                      int32_t max_det, float* trace, int64_t max_trace) {
  if (!s) return FDTD2D_ERR_INVALID;
  if (s->finished.empty()) return 0;
  Finished& f = s->finished.front();
  if (tag) *tag = f.tag;
  if (n_det) *n_det = f.n_det;
  if (n_steps) *n_steps = f.n_steps;
  if (dft && !f.dft.empty())
    std::memcpy(dft, f.dft.data(), std::min<size_t>(f.dft.size(), 2 * (size_t)std::max<int32_t>(0, max_det)) * 8);
  if (trace && !f.trace.empty())
    std::memcpy(trace, f.trace.data(), std::min<size_t>(f.trace.size(), (size_t)std::max<int64_t>(0, max_trace)) * 4);
  s->finished.erase(s->finished.begin());
  return 1;
}

static int fdtd2d_server_cancel_body(fdtd2d_server* s, int64_t tag);

// The entry point: its body, below, runs behind abi_guard.
int fdtd2d_server_cancel(fdtd2d_server* s, int64_t tag) {
  return abi_guard([&] { return fdtd2d_server_cancel_body(s, tag); });
}

// Queued shots of the tag leave the queue; running ones are removed from the
// batch (a batch-kernel member's memory is released behind the blocks already
// queued for it, which the batch's stream orders before any reuse, and the
// unit list is rebuilt before the next block; a solo member waits for its own
// streams); finished ones not yet popped are dropped.
static int fdtd2d_server_cancel_body(fdtd2d_server* s, int64_t tag) {
  if (!s) return FDTD2D_ERR_INVALID;
  cudaSetDevice(s->b->device);
  int n = 0;
  for (size_t q = 0; q < s->queue.size();) {
    if (s->queue[q].tag == tag) {
      s->queue.erase(s->queue.begin() + q);
      ++n;
    } else {
      ++q;
    }
  }
  for (size_t r = 0; r < s->running.size();) {
    if (s->running[r].tag != tag) {
      ++r;
      continue;
    }
    const int rc = fdtd2d_batch_remove(s->b, s->running[r].slot);
    if (rc) return rc;
    s->running.erase(s->running.begin() + r);
    ++n;
  }
  for (size_t f = 0; f < s->finished.size();) {
    if (s->finished[f].tag == tag) {
      s->finished.erase(s->finished.begin() + f);
      ++n;
    } else {
      ++f;
    }
  }
  return n;
}

int fdtd2d_server_counts(const fdtd2d_server* s, int32_t* queued, int32_t* running, int32_t* finished) {
  if (!s) return FDTD2D_ERR_INVALID;
  if (queued) *queued = (int32_t)s->queue.size();
  if (running) *running = (int32_t)s->running.size();
  if (finished) *finished = (int32_t)s->finished.size();
  return FDTD2D_OK;
}

fdtd2d_batch* fdtd2d_server_batch(fdtd2d_server* s) { return s ? s->b : nullptr; }

int fdtd2d_server_destroy(fdtd2d_server* s) {
  if (!s) return FDTD2D_ERR_INVALID;
  if (s->b) fdtd2d_batch_destroy(s->b);
  for (auto& x : s->blocks) cudaEventDestroy(x.second);
  for (cudaEvent_t e : s->spare) cudaEventDestroy(e);
  delete s;
  return FDTD2D_OK;
}

}  // extern "C"
