// C-ABI layer: one context = one shot's device state + one CUDA stream.
// Replaces DevMemoryAllocation / DevFieldCalculation / DevMemoryFree
// (FDTD_2D_Full/kernel.cu:1087-1618, 1928-2818, 2820-2987).  Unlike the
// reference, every allocation is owned by the context (no file-scope device
// globals), so independent contexts can coexist in one process.
#include "../../include/fdtd2d.h"
#include "internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

using namespace fdtd2d;

#include "ctx.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

int fail_cuda(fdtd2d_ctx* c, cudaError_t e) {
  if (c) c->last_cuda = (int)e;
  return e == cudaErrorMemoryAllocation ? FDTD2D_ERR_NOMEM : FDTD2D_ERR_CUDA;
}

// The shot's device error word, read in the order of its stream.  The word
// is allocated and zeroed on that (non-blocking) stream, and kernels on it
// set it; a plain cudaMemcpy runs on the legacy default stream, which does
// not wait for a non-blocking stream, and could read memory the pool handed
// back from a freed shot before the zeroing has run.
cudaError_t read_err(fdtd2d_ctx* c, int* err) {
  *err = 0;
  cudaError_t e = cudaMemcpyAsync(err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e;
}

// Test parameter FDTD2D_TEST_FAIL_ALLOC=k (read at create): the k-th device
// allocation a context makes reports cudaErrorMemoryAllocation without
// allocating, so a test can walk every allocation of fdtd2d_create and check
// that each failure comes back as FDTD2D_ERR_NOMEM with the context's other
// memory released, or, where the library has a smaller form to fall back to
// (the two-step path's extra buffers), that the shot still runs.  Normal runs
// leave it unset.
template <class T>
cudaError_t dalloc(fdtd2d_ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return cudaSuccess;
  if (c->fail_alloc > 0 && ++c->n_alloc == c->fail_alloc) return cudaErrorMemoryAllocation;
  void* q = nullptr;
  // Stream-ordered allocation from the device's pool: a shot's memory is
  // released with cudaFreeAsync behind its last kernel, so retiring a batch
  // member never waits for the device.
  cudaError_t e = cudaMallocAsync(&q, count * sizeof(T), c->stream);
  if (e != cudaSuccess) return e;
  c->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return cudaMemsetAsync(q, 0, count * sizeof(T), c->stream);
}

int pitch_for(int nx) { return row_pitch(nx); }

// Power-of-two scale for an array whose values reach about `m`: stored
// values then reach about 2^14, with 4x headroom below the FP16 maximum.
void pow2_scale(double m, float* sc, float* isc) {
  int k = 0;
  if (m > 0 && std::isfinite(m)) k = std::max(-100, std::min(100, (int)std::ceil(std::log2(m)) - 14));
  *sc = std::ldexp(1.f, k);
  *isc = std::ldexp(1.f, -k);
}

// Per-array scales for F16 storage (BF16 keeps FP32's exponent range: 1).
// Peaks: |Ez| from field_max, or 16 x (array elements) x (source amplitude)
// / max(2 pi f0 dt, 1e-3) (a soft source adds its sample every step, about
// 1/(2 pi f dt) steps per radian); |H| ~ |Ez|/eta0 x 4; |Jz| from the Drude
// update's steady response kp |Ez| / |1 - ja e^{-i w dt}| x 2; the drive map
// from its exact maximum.
void set_storage_scales(const fdtd2d_setup* s, double beta, DevShot* h) {
  if (h->store != FDTD2D_STORE_F16) return;
  double env = 0;
  for (int n = 0; n <= s->n_steps; ++n) env = std::max(env, (double)std::fabs(s->envelope[n]));
  const double wdt = 2 * kPi * std::max(s->f0, s->f1) * s->dt;
  double em = s->field_max;
  if (em <= 0) em = 16.0 * std::max(1, s->n_src) * std::fabs(s->src_scale) * env / std::max(wdt, 1e-3);
  double kmax = 0;
  if (s->ne)
    for (int64_t t = 0; t < (int64_t)s->nx * s->ny; ++t) kmax = std::max(kmax, beta * (double)s->ne[t]);
  const double ja = h->ja;
  const double jm = em * kmax / std::max(std::sqrt((1 - ja) * (1 - ja) + wdt * wdt), 1e-3) * 2;
  const double eta0 = 376.730313668;
  pow2_scale(em, &h->sc[0], &h->isc[0]);
  pow2_scale(em / eta0 * 4, &h->sc[1], &h->isc[1]);
  pow2_scale(em / eta0 * 4, &h->sc[2], &h->isc[2]);
  pow2_scale(jm, &h->sc[3], &h->isc[3]);
  pow2_scale(kmax, &h->sc[4], &h->isc[4]);
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on it).
PFN_cuTensorMapEncodeTiled_v12000 tensor_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Tensor maps of a shot for a tensor shape: boxes of bx columns x rows rows.
bool encode_maps(const DevShot& h, int nx, int ny, int bx, int rows, TensorMaps* m) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_encoder();
  if (!enc) return false;
  const int es = store_bytes(h.store);
  const CUtensorMapDataType dt = h.store == FDTD2D_STORE_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : h.store == FDTD2D_STORE_F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                               : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  const cuuint32_t est[3] = {1, 1, 1};
  for (int b = 0; b < 4; ++b) {
    if (!h.fb[b]) continue;
    const cuuint64_t dims3[3] = {(cuuint64_t)nx, (cuuint64_t)ny, 3};
    const cuuint64_t str3[2] = {(cuuint64_t)h.pitch * es, (cuuint64_t)h.cells * es};
    const cuuint32_t box3[3] = {(cuuint32_t)bx, (cuuint32_t)rows, 3};
    void* hx = es == 4 ? (void*)field_ptr_t<float>(h, kHx, b) : (void*)field_ptr_t<uint16_t>(h, kHx, b);
    if (enc(&m->hj[b], dt, 3, hx, dims3, str3, box3, est, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
    const cuuint64_t dims2[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
    const cuuint64_t str2[1] = {(cuuint64_t)h.pitch * es};
    const cuuint32_t box2[2] = {(cuuint32_t)bx, (cuuint32_t)rows};
    void* ez = es == 4 ? (void*)field_ptr_t<float>(h, kEz, b) : (void*)field_ptr_t<uint16_t>(h, kEz, b);
    if (enc(&m->e[b], dt, 2, ez, dims2, str2, box2, est, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  std::memset(&m->k, 0, sizeof m->k);
  if (h.kp) {
    const cuuint64_t dims2[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
    const cuuint64_t str2[1] = {(cuuint64_t)h.pitch * es};
    const cuuint32_t box2[2] = {(cuuint32_t)bx, (cuuint32_t)rows};
    if (enc(&m->k, dt, 2, const_cast<float*>(h.kp), dims2, str2, box2, est, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

// Units (0, c0, j0, j1) over columns [ca, cb) in bands of `band`, rows
// [ra, rb) in `strips` strips.
void add_units(std::vector<int4>& u, int ca, int cb, int band, int ra, int rb, int strips) {
  if (cb <= ca || rb <= ra) return;
  strips = std::max(1, std::min(strips, rb - ra));
  for (int k = 0; k < strips; ++k) {
    const int j0 = ra + (int)((int64_t)(rb - ra) * k / strips), j1 = ra + (int)((int64_t)(rb - ra) * (k + 1) / strips);
    if (j1 <= j0) continue;
    for (int c = ca; c < cb; c += band) u.push_back(make_int4(0, c, j0, j1));
  }
}

// Units of the one-row kernel on the rest of the grid beside the interior
// region [ci0, ci1) x [ri0, ri1): bands of `band` columns over [0, ci0) and
// [ci1, nx) on every row, and over [ci0, ci1) on rows [0, ri0) and [ri1,
// ny - 1).  Each band's rows are cut into strips of about equal cost (a row
// of the CPML row strips costs about 1.5 plain rows, a row of a band that
// holds an x strip about 2: with 1.3 the x-strip bands' strips finished last,
// 0.2-1.5 % slower on the 2048^2 and 8192^2 shots) so that the strips fill
// `ctas` CTAs in one wave: the band kernel's step between two interior
// passes runs alone, and its time is that of its longest CTA.
std::vector<int4> edge_units(int nx, int ny, int P, int ci0, int ci1, int ri0, int ri1, int band, int ctas) {
  struct Seg {
    int c0, j0, j1;
    double w;
  };
  std::vector<Seg> segs;
  auto xw = [&](int c) { return (c == 0 || c + band - 1 >= nx - P) ? 2.0 : 1.0; };
  for (int c = ci0; c < ci1; c += band) {
    segs.push_back({c, 0, ri0, 1.5});
    segs.push_back({c, ri1, ny - 1, 1.5});
  }
  for (int c = 0; c < ci0; c += band) segs.push_back({c, 0, ny - 1, xw(c)});
  for (int c = ci1; c < nx; c += band) segs.push_back({c, 0, ny - 1, xw(c)});
  double total = 0;
  for (const Seg& g : segs) total += std::max(0, g.j1 - g.j0) * g.w;
  const int slots = std::max(1, ctas - (int)segs.size());   // room for every band's rounding up
  // No floor above one row: at 1024^2 a floor of four rows held the whole
  // path to 72.4 Gcell/s against 81.6 with one; from 2048^2 up the floor
  // does not bind.
  const double per = std::max(1.0, total / slots);
  std::vector<int4> u;
  for (const Seg& g : segs) {
    const int r = g.j1 - g.j0;
    if (r <= 0) continue;
    const int k = std::max(1, std::min(r, (int)std::ceil(r * g.w / per)));
    for (int s = 0; s < k; ++s) {
      const int a = g.j0 + (int)((int64_t)r * s / k), b = g.j0 + (int)((int64_t)r * (s + 1) / k);
      if (b > a) u.push_back(make_int4(0, g.c0, a, b));
    }
  }
  return u;
}

// Keep freed shot memory in this process's pool of the device (default
// release threshold 0 hands it back at every synchronisation, and the next
// shot pays to map it again).  A property of this process's pool only.
void keep_pool_memory(int device) {
  static bool done[64] = {false};
  if (device < 0 || device >= 64 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[device] = true;
}

__global__ void drive_from_density(float* kp, int64_t pitch, int nx, int ny, float beta) {
  // kp = beta * ne in place over the nx x ny cells; no plasma (ne <= 0) -> 0.
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)ny * nx;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = (t / nx) * pitch + (t % nx);
    const float ne = kp[k];
    kp[k] = ne > 0.f ? beta * ne : 0.f;
  }
}

int validate(const fdtd2d_setup* s) {
  if (!s) return FDTD2D_ERR_INVALID;
  const int P = s->npml;
  if (s->nx < 8 || s->ny < 8 || P < 2) return FDTD2D_ERR_INVALID;
  if (2 * P + 2 > s->nx || 2 * P + 2 > s->ny) return FDTD2D_ERR_INVALID;
  if (s->n_steps < 1 || !(s->dt > 0) || !(s->dx > 0) || !(s->dy > 0)) return FDTD2D_ERR_INVALID;
  const float* tabs[] = {s->be_x_1, s->ce_x_1, s->be_x_2, s->ce_x_2, s->bh_x_1, s->ch_x_1,
                         s->bh_x_2, s->ch_x_2, s->be_y_1, s->ce_y_1, s->be_y_2, s->ce_y_2,
                         s->bh_y_1, s->ch_y_1, s->bh_y_2, s->ch_y_2};
  for (const float* t : tabs)
    if (!t) return FDTD2D_ERR_INVALID;
  if (!s->den_ex || !s->den_hx || !s->den_ey || !s->den_hy) return FDTD2D_ERR_INVALID;
  if (s->medium == FDTD2D_MEDIUM_MATERIAL_ID) {
    if (!s->id1 || !s->id2 || !s->id3) return FDTD2D_ERR_INVALID;
    if (s->n_materials < 2 || s->n_materials > 256) return FDTD2D_ERR_INVALID;
    if (!s->mat_ca || !s->mat_cb || !s->mat_da || !s->mat_db || !s->mat_ne) return FDTD2D_ERR_INVALID;
  } else if (s->medium != FDTD2D_MEDIUM_UNIFORM) {
    return FDTD2D_ERR_INVALID;
  }
  if (s->storage < FDTD2D_STORE_F32 || s->storage > FDTD2D_STORE_BF16) return FDTD2D_ERR_INVALID;
  // reduced storage runs on the shared-memory staged kernel only
  if (s->storage != FDTD2D_STORE_F32 && (s->medium != FDTD2D_MEDIUM_UNIFORM || s->npml > tma_max_pml()))
    return FDTD2D_ERR_INVALID;
  auto interior = [&](const fdtd2d_point& p) {
    return p.i >= 1 && p.i <= s->nx - 2 && p.j >= 1 && p.j <= s->ny - 2;
  };
  if (s->n_src < 0 || s->n_det < 0 || s->n_comp < 0) return FDTD2D_ERR_INVALID;
  if (s->n_src > 0 && (!s->src || !s->src_phase_deg || !s->envelope)) return FDTD2D_ERR_INVALID;
  if (s->n_det > 0 && !s->det) return FDTD2D_ERR_INVALID;
  if (s->n_comp > 0 && !s->comp) return FDTD2D_ERR_INVALID;
  for (int e = 0; e < s->n_src; ++e)
    if (!interior(s->src[e])) return FDTD2D_ERR_RANGE;
  for (int e = 0; e < s->n_det; ++e)
    if (!interior(s->det[e])) return FDTD2D_ERR_RANGE;
  for (int e = 0; e < s->n_comp; ++e)
    if (!interior(s->comp[e])) return FDTD2D_ERR_RANGE;
  if (s->f1 != s->f0 && !(s->t1 > 0)) return FDTD2D_ERR_INVALID;
  if (s->n_rc < 0 || (s->n_rc > 0 && (!s->rc_scan_i || !s->rc_max_i))) return FDTD2D_ERR_INVALID;
  for (int l = 0; l < s->n_rc; ++l)
    if (s->rc_scan_i[l] < 0 || s->rc_scan_i[l] >= s->nx || s->rc_max_i[l] < 0 || s->rc_max_i[l] >= s->nx)
      return FDTD2D_ERR_RANGE;
  if (s->line_n < 0) return FDTD2D_ERR_INVALID;
  if (s->line_n > 0 && (s->line_i0 < 0 || s->line_i0 + s->line_n > s->nx || s->line_j < 0 ||
                        s->line_j >= s->ny || s->line_first < 1 || s->line_last > s->n_steps ||
                        s->line_last < s->line_first))
    return FDTD2D_ERR_RANGE;
  return FDTD2D_OK;
}

// Split rows [0, ny-1) x column blocks of `cols` into at most `warps` units.
std::vector<int4> make_units(int shot, int nx, int ny, int warps, int cols = kCols, int min_rows = 8) {
  const int cb = (nx + cols - 1) / cols;
  const int rows = ny - 1;
  int strips = std::max(1, warps / cb);
  strips = std::min(strips, std::max(1, rows / min_rows));
  std::vector<int4> u;
  u.reserve((size_t)cb * strips);
  for (int s = 0; s < strips; ++s) {
    const int j0 = (int)((int64_t)rows * s / strips);
    const int j1 = (int)((int64_t)rows * (s + 1) / strips);
    if (j1 <= j0) continue;
    for (int c = 0; c < cb; ++c) u.push_back(make_int4(shot, c * cols, j0, j1));
  }
  return u;
}

}  // namespace

extern "C" {

int fdtd2d_abi_version(void) { return FDTD2D_ABI_VERSION; }

const char* fdtd2d_strerror(int status) {
  switch (status) {
    case FDTD2D_OK: return "ok";
    case FDTD2D_ERR_INVALID: return "invalid argument or setup";
    case FDTD2D_ERR_NOMEM: return "out of memory";
    case FDTD2D_ERR_CUDA: return "CUDA runtime error";
    case FDTD2D_ERR_NONFINITE: return "non-finite value in the fields";
    case FDTD2D_ERR_RANGE: return "index or step out of range";
    case FDTD2D_ERR_IO: return "file I/O error";
    case FDTD2D_ERR_CONFIG: return "configuration error";
    case FDTD2D_ERR_STATE: return "call not valid in this state";
    case FDTD2D_ERR_BUDGET: return "request exceeds the memory budget";
    case FDTD2D_ERR_NODEVICE: return "no CUDA device";
    case FDTD2D_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    default: return "unknown error";
  }
}

int64_t fdtd2d_device_bytes(const fdtd2d_setup* s) {
  if (!s) return -1;
  const int64_t pitch = pitch_for(s->nx);
  const int64_t cells = buffer_floats(s->nx, s->ny);
  const int64_t P = s->npml;
  const int64_t es = (s->storage == FDTD2D_STORE_F16 || s->storage == FDTD2D_STORE_BF16) ? 2 : 4;
  int64_t b = cells * es * 8;                                      // 4 fields x 2
  b += (s->medium == FDTD2D_MEDIUM_UNIFORM) ? (s->ne ? cells * es : 0) : cells * 3;
  b += 2 * 4 * (2 * (P - 1) * pitch + 2 * P * pitch + 2 * s->ny * P * 2);
  b += 4 * (int64_t)s->n_steps * (s->record_traces ? (s->n_det + 3 * s->n_comp) : 0);
  b += 4 * (int64_t)(s->n_steps + 1) + 16 * (int64_t)s->n_det + (1 << 20);
  return b;
}

int fdtd2d_create(const fdtd2d_setup* s, int device, fdtd2d_ctx** out) {
  return abi_guard([&] { return fdtd2d::create_ctx(s, device, false, out); });
}

}  // extern "C"

namespace {

// Field-buffer slots a and b of a descriptor and its tensor maps traded.
void swap_slots(DevShot& h, TensorMaps& m, int a, int b) {
  std::swap(h.fb[a], h.fb[b]);
  std::swap(m.hj[a], m.hj[b]);
  std::swap(m.e[a], m.e[b]);
}

// Interior-kernel timing (fdtd2d_time_step_kernel): an event pair around a
// launch on the shot stream.  Pending pairs are folded into the totals when
// read, or when many have piled up.
cudaEvent_t prof_event(fdtd2d_ctx* c) {
  if (!c->prof_pool.empty()) {
    cudaEvent_t e = c->prof_pool.back();
    c->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
}

cudaError_t prof_fold(fdtd2d_ctx* c) {
  cudaError_t r = cudaSuccess;
  for (auto& pr : c->prof_pending) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(pr.second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, pr.first, pr.second);
    if (e == cudaSuccess) {
      c->prof_ms += ms;
      ++c->prof_n;
    } else {
      r = e;
    }
    c->prof_pool.push_back(pr.first);
    c->prof_pool.push_back(pr.second);
  }
  c->prof_pending.clear();
  return r;
}

// Start (e0 = nullptr) or end a timed launch; returns the start event.
cudaEvent_t prof_mark(fdtd2d_ctx* c, cudaEvent_t e0, int64_t cells, int steps) {
  if (!c->prof) return nullptr;
  if (!e0) {
    cudaEvent_t e = prof_event(c);
    if (e) cudaEventRecord(e, c->stream);
    return e;
  }
  cudaEvent_t e1 = prof_event(c);
  if (!e1) return nullptr;
  cudaEventRecord(e1, c->stream);
  c->prof_pending.emplace_back(e0, e1);
  c->prof_cells = cells;
  c->prof_steps = steps;
  if (c->prof_pending.size() >= 4096) prof_fold(c);
  return nullptr;
}

// What one two-step pair launches: the interior kernel's shape, units and
// CTAs, the CPML-band kernel's, and the interior region.
struct PairPlan {
  int k, tctas, ntu;
  const int4* tu;
  int q, ectas, neu;
  const int4* eu;
  int ci0, ci1, ri0, ri1;
};

// Steps n and n+1 on the two-step path.  Shot stream: the interior kernel
// (both steps of R), then, once the CPML-band kernel's step n is done, the
// frame kernel (step n+1 of the 2-cell frame around R: all that the next
// interior pass reads outside R).  Side stream: the band kernel's step n,
// then, once the interior kernel is done, its step n+1, which so runs beside
// the next pair's interior kernel.  Slots: state n-1 in a = (n-1)&1, state n
// (band cells, and R's edge cells from the interior kernel's ring units)
// into b = n&1, state n+1 into slot 2; slot 3 holds
// the previous pair's state-n buffer, which that pair's band step n+1 may
// still be reading.  h and m come back with state n+1 in slot a (= (n+1)&1),
// the next pair's state-n buffer in slot b, the old state n-1 buffer in slot
// 2 and this pair's state-n buffer in slot 3.  Every buffer a kernel here
// overwrites was last read by work the stream order or these waits put
// before it (the interior kernel's output by the band kernel's step n of the
// previous pair, waited for by that pair's frame kernel).
cudaError_t issue_pair(fdtd2d_ctx* c, const PairPlan& p, DevShot& h, TensorMaps& m, int n) {
  const int a = (n - 1) & 1, b = n & 1;
  DevShot ti = h;
  TensorMaps tm = m;
  ti.fb[0] = h.fb[a];
  ti.fb[1] = h.fb[b];
  tm.hj[0] = m.hj[a];
  tm.e[0] = m.e[a];
  DevShot t2 = h;          // step n+1: reads slot b, writes slot a = the state n+1 buffer
  t2.fb[a] = h.fb[2];
  cudaError_t x = cudaStreamWaitEvent(c->side, c->ev_t, 0);
  cudaEvent_t p0 = prof_mark(c, nullptr, 0, 2);
  if (x == cudaSuccess)
    x = launch_step_tmat2(p.k, ti, tm, p.tu, p.ntu, n, make_int4(p.ci0, p.ci1, p.ri0, p.ri1), p.tctas, c->d_ctr,
                          c->d_err, c->stream);
  if (p0) prof_mark(c, p0, (int64_t)(p.ci1 - p.ci0) * (p.ri1 - p.ri0), 2);
  if (x == cudaSuccess) x = cudaEventRecord(c->ev_t, c->stream);
  if (x == cudaSuccess) x = launch_step_tma(p.q, h, p.eu, p.neu, n, p.ectas, c->d_err, c->side);
  if (x == cudaSuccess) x = cudaEventRecord(c->ev_a, c->side);
  if (x == cudaSuccess) x = cudaStreamWaitEvent(c->stream, c->ev_a, 0);
  if (x == cudaSuccess) x = launch_frame(t2, p.ci0, p.ci1, p.ri0, p.ri1, n + 1, c->d_ctr, c->stream);
  if (x == cudaSuccess) x = cudaStreamWaitEvent(c->side, c->ev_t, 0);
  if (x == cudaSuccess) x = launch_step_tma(p.q, t2, p.eu, p.neu, n + 1, p.ectas, c->d_err, c->side);
  if (x == cudaSuccess) x = cudaEventRecord(c->ev_e, c->side);
  swap_slots(h, m, a, 2);
  swap_slots(h, m, b, 3);
  return x;
}

// Kernel choices found by the create-time timing, per shot class (device,
// grid size class, CPML depth in steps of 16, storage, drive map, the
// FDTD2D_* overrides):
// later shots of the same class take the stored choice without timing.  The
// size class of a side n is ceil(log2 n) and, within it, the half it falls
// in, so that shots of similar grids share one timing.  `k` is the tensor
// shape (-1: the one-row kernel alone), `q` the one-row shape, `lv` the
// tensor path's steps per pass.
struct KernelChoice {
  int k = -1, q = 0, lv = 1;
  bool from_file = false;   // read from the persisted choices, not timed in this process
};
using ChoiceKey = std::tuple<int, int, int, int, int, int, std::string>;
std::mutex g_choice_mu;
std::map<ChoiceKey, KernelChoice> g_choice;

ChoiceKey choice_key(const fdtd2d_ctx* c, int device, const char* what) {
  std::string env = what;
  for (const char* v : {"FDTD2D_TMAT", "FDTD2D_TB", "FDTD2D_TMA", "FDTD2D_TMA_AUTOTUNE", "FDTD2D_TMAT_AUTOTUNE",
                        "FDTD2D_KERNEL", "FDTD2D_PERSIST"}) {
    const char* x = std::getenv(v);
    env += '|';
    env += x ? x : "-";
  }
  auto cls = [](int n) {
    int b = 0;
    while ((1 << b) < n) ++b;                      // n in (2^(b-1), 2^b]
    return 2 * b + (n > 3 * (1 << b) / 4 ? 1 : 0);   // upper or lower half of that range
  };
  return ChoiceKey{device, cls(c->nx), cls(c->ny), (c->npml + 15) / 16, c->h.store, c->h.kp != nullptr, env};
}

// ---- persisted choices -------------------------------------------------------
// The choices are also kept in a small JSON file, so that a new process skips
// the timing of the classes an earlier one timed (0.31 s at 8192^2): the file
// $FDTD2D_TUNE_CACHE, else $XDG_CACHE_HOME/fdtd2d/kernel_choices.json, else
// $HOME/.cache/fdtd2d/kernel_choices.json; FDTD2D_TUNE_CACHE=0 (or empty)
// keeps the choices in memory only.  An entry is keyed by the device's name,
// SM count and compute capability (not its index) and the shot class.  The
// file is read once per device, at its first lookup, and rewritten whole
// (temporary file, then rename) when a choice is added.  A file that cannot
// be read or written only costs the timing.
std::map<std::string, KernelChoice> g_file;   // every entry of the file, all devices
bool g_file_loaded[64] = {};

std::string clean(const std::string& t) {
  std::string o = t;
  for (char& ch : o)
    if (ch == '"' || ch == '\\' || ch < 32) ch = '_';
  return o;
}

std::string cache_path() {
  if (const char* v = std::getenv("FDTD2D_TUNE_CACHE")) return (std::strcmp(v, "0") == 0) ? std::string() : v;
  if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x) return std::string(x) + "/fdtd2d/kernel_choices.json";
  if (const char* h = std::getenv("HOME"); h && *h) return std::string(h) + "/.cache/fdtd2d/kernel_choices.json";
  return std::string();
}

std::string device_ident(int device) {
  static std::string ident[64];
  if (device < 0 || device >= 64) return std::string();
  if (ident[device].empty()) {
    cudaDeviceProp pr{};
    if (cudaGetDeviceProperties(&pr, device) != cudaSuccess) return std::string();
    char b[320];
    std::snprintf(b, sizeof b, "%s|%d|%d.%d", pr.name, pr.multiProcessorCount, pr.major, pr.minor);
    ident[device] = clean(b);
  }
  return ident[device];
}

// "<device>|<class fields>|<what and overrides>" (the last part holds '|'s)
// The version of the timing that made a choice: a file entry of another
// version is not used (choices made by an earlier candidate set or trial
// method are timed again).
constexpr int kChoiceVersion = 2;

std::string key_text(const ChoiceKey& k) {
  char b[112];
  std::snprintf(b, sizeof b, "|v%d|%d|%d|%d|%d|%d|", kChoiceVersion, std::get<1>(k), std::get<2>(k), std::get<3>(k),
                std::get<4>(k), std::get<5>(k));
  return device_ident(std::get<0>(k)) + b + clean(std::get<6>(k));
}

void load_choices(int device) {   // g_choice_mu held
  if (device < 0 || device >= 64 || g_file_loaded[device]) return;
  g_file_loaded[device] = true;
  const std::string path = cache_path();
  const std::string id = device_ident(device);
  if (path.empty() || id.empty()) return;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[1024];
  while (std::fgets(line, sizeof line, f)) {
    // one entry per line:  "key": [k, q, lv],
    const char* a = std::strchr(line, '"');
    const char* z = a ? std::strchr(a + 1, '"') : nullptr;
    if (!z) continue;
    const std::string key(a + 1, z);
    KernelChoice ch;
    if (std::sscanf(z + 1, " : [ %d , %d , %d ]", &ch.k, &ch.q, &ch.lv) != 3) continue;
    ch.from_file = true;
    if (!g_file.count(key)) g_file[key] = ch;
    // entries of this device go to the lookup table
    if (key.compare(0, id.size() + 1, id + "|") != 0) continue;
    int ver, f1, f2, f3, f4, f5, used = 0;
    if (std::sscanf(key.c_str() + id.size(), "|v%d|%d|%d|%d|%d|%d|%n", &ver, &f1, &f2, &f3, &f4, &f5, &used) != 6 ||
        !used || ver != kChoiceVersion)
      continue;
    const ChoiceKey ck{device, f1, f2, f3, f4, f5, key.substr(id.size() + used)};
    if (!g_choice.count(ck)) g_choice[ck] = ch;
  }
  std::fclose(f);
}

void save_choices() {   // g_choice_mu held
  const std::string path = cache_path();
  if (path.empty()) return;
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0) {
    // make the directories of the path (one level at a time)
    for (size_t p = path.find('/', 1); p != std::string::npos && p <= slash; p = path.find('/', p + 1))
      mkdir(path.substr(0, p).c_str(), 0755);
  }
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return;
  std::fprintf(f, "{\n \"fdtd2d_kernel_choices\": 1,\n \"choices\": {\n");
  size_t n = 0;
  for (const auto& kv : g_file)
    std::fprintf(f, "  \"%s\": [%d, %d, %d]%s\n", kv.first.c_str(), kv.second.k, kv.second.q, kv.second.lv,
                 ++n < g_file.size() ? "," : "");
  std::fprintf(f, " }\n}\n");
  const bool ok = std::fclose(f) == 0;
  if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

bool find_choice(const ChoiceKey& key, KernelChoice* out) {
  std::lock_guard<std::mutex> lock(g_choice_mu);
  load_choices(std::get<0>(key));
  auto it = g_choice.find(key);
  if (it == g_choice.end()) return false;
  *out = it->second;
  return true;
}

void keep_choice(const ChoiceKey& key, const KernelChoice& ch) {
  std::lock_guard<std::mutex> lock(g_choice_mu);
  KernelChoice c = ch;
  c.from_file = false;
  g_choice[key] = c;
  const std::string kt = key_text(key);
  if (device_ident(std::get<0>(key)).empty()) return;
  g_file[kt] = c;
  save_choices();
}

// How the choices of a create were made (fdtd2d_kernel_choice_source).
void note_choice(fdtd2d_ctx* c, bool have, const KernelChoice& known) {
  if (have) c->choice_src = std::max(c->choice_src, known.from_file ? 2 : 1);
}

// A material-ID medium that the uniform medium represents exactly: every
// cell inside the reference's launch coverage, no PEC cell (Ez material 1),
// one (CA, CB) over the materials of the Ez map and one (DA, DB) over those
// of the Hx and Hy maps (bit for bit: the reference's vacuum and plasma
// levels all share them).  Then the shot is stepped as the uniform medium
// with a drive map holding each Ez cell's material drive, the float the
// material kernel reads, so the staged and tensor kernels give it the
// material kernel's bits.  kp stays empty when no cell has plasma.
bool material_as_uniform(const fdtd2d_setup* s, double beta, float* ca, float* cb, float* da, float* db,
                         std::vector<float>* kp) {
  const int64_t n = (int64_t)s->nx * s->ny;
  // reference thread indices each update kernel needs for every cell (its
  // largest index + 1): Hx, Hx y strips, Hy, Hy x strips, Jz, Ez, Ez x
  // strips, Ez y strips
  const int64_t X = s->nx, Y = s->ny, Q = s->npml - 1;
  const int64_t need[8] = {(Y - 1) * (X - 1), Q * (X - 1), Y * (X - 1), Y * Q,
                           (Y - 2) * (X - 2), (Y - 2) * (X - 2), (Y - 2) * Q, Q * (X - 2)};
  for (int k = 0; k < 8; ++k)
    if (s->cover[k] != 0 && s->cover[k] < need[k]) return false;
  const int nm = s->n_materials;
  std::vector<char> used_e(nm, 0), used_h(nm, 0);
  for (int64_t t = 0; t < n; ++t) {
    const int32_t a = s->id1[t], b = s->id2[t], e = s->id3[t];
    if (a < 0 || a >= nm || b < 0 || b >= nm || e < 0 || e >= nm) return false;
    used_h[a] = used_h[b] = 1;
    used_e[e] = 1;
  }
  if (nm > 1 && used_e[1]) return false;
  auto same = [](float x, float y) { return std::memcmp(&x, &y, sizeof(float)) == 0; };
  int fe = -1, fh = -1;
  for (int m = 0; m < nm; ++m) {
    if (used_e[m]) {
      if (fe < 0) fe = m;
      else if (!same(s->mat_ca[m], s->mat_ca[fe]) || !same(s->mat_cb[m], s->mat_cb[fe])) return false;
    }
    if (used_h[m]) {
      if (fh < 0) fh = m;
      else if (!same(s->mat_da[m], s->mat_da[fh]) || !same(s->mat_db[m], s->mat_db[fh])) return false;
    }
  }
  if (fe < 0 || fh < 0) return false;
  *ca = s->mat_ca[fe];
  *cb = s->mat_cb[fe];
  *da = s->mat_da[fh];
  *db = s->mat_db[fh];
  std::vector<float> drive(nm, 0.f);
  bool any = false;
  for (int m = 0; m < nm; ++m) {
    const double ne = s->mat_ne[m];
    drive[m] = ne > 0 ? (float)(beta * ne) : 0.f;   // the material table's value
    any = any || (used_e[m] && drive[m] != 0.f);
  }
  kp->clear();
  if (any) {
    kp->resize((size_t)n);
    for (int64_t t = 0; t < n; ++t) (*kp)[(size_t)t] = drive[s->id3[t]];
  }
  return true;
}

// Multi-row tensor path (step_tmat.cu) for the interior of the shot, beside
// the staged kernel on the CPML bands and rows.  Times every tensor shape that
// fits the grid (tensor kernel on the interior units + staged kernel on the
// rest, issued as fdtd2d_run issues them, traces and DFT off, re-run
// idempotently) against the staged kernel alone, and keeps the fastest per
// step.  Each tensor shape is tried in its one-step form and in its two-step
// form (two time steps per pass over the fields; two more field buffers).
// The trials cover the shapes that win on GB300 (three tensor shapes, three
// one-row shapes for the CPML bands) unless FDTD2D_TMAT_AUTOTUNE=full asks
// for every compiled pair; a shot of a class timed before takes the stored
// choice.  FDTD2D_TMAT=0 leaves the tensor path off, FDTD2D_TMAT=W,R,ST
// forces a shape; FDTD2D_TB=0 leaves the two-step form out, FDTD2D_TB=1
// keeps only it.
// Grids up to this many cells are tried on the persistent kernel: there a
// step's fields stay in L2 and the per-launch gaps, not bytes, set the
// step time.
constexpr int64_t kPersistMaxCells = int64_t(1) << 22;
// Steps per persistent launch (a launch of a few tens of ms at most).
constexpr int kPersistSteps = 4096;

// Persistent launches of every shot of this process on a device run one at a
// time: each waits for the previous one (on whichever stream it ran) and
// leaves an event for the next.  Two cooperative grids that each fill the
// GPU then never wait on each other's CTAs.
std::mutex g_persist_mu;
cudaEvent_t g_persist_last[64] = {};

cudaError_t launch_persist_ordered(fdtd2d_ctx* c, const DevShot& t, int32_t n, int32_t m, int repeat,
                                   const PersistAux& A) {
  if (c->device < 0 || c->device >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_persist_mu);
  cudaEvent_t& last = g_persist_last[c->device];
  cudaError_t e = cudaSuccess;
  if (!last) {
    e = cudaEventCreateWithFlags(&last, cudaEventDisableTiming);
  } else {
    e = cudaStreamWaitEvent(c->stream, last, 0);
  }
  if (e == cudaSuccess)
    e = launch_step_persist(t, c->d_punits, c->n_punits, n, m, repeat, A, c->medium, c->persist_ctas, c->d_bar,
                            c->d_err, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(last, c->stream);
  return e;
}

// The persistent form: FP32 single shots of at most kPersistMaxCells cells
// whose path at create was timed (path_ms) or whose class chose it before.
// Trial: one launch that repeats step 1 sixteen times with traces and the
// DFT off (each repeat reads the same buffers and writes the same values),
// against the chosen path's per-step time; kept when at least 10 % faster.
// FDTD2D_PERSIST=0 never, =1 always (where it can run); not tried when
// FDTD2D_TMA, FDTD2D_TMAT or FDTD2D_TB names a staged path.
int setup_persist(fdtd2d_ctx* c, int device) {
  const char* env = std::getenv("FDTD2D_PERSIST");
  const int mode = env ? std::atoi(env) : -1;
  DevShot& h = c->h;
  if (mode == 0 || h.store != FDTD2D_STORE_F32 || c->n_steps < 2) return FDTD2D_OK;
  if (mode < 0 && (int64_t)c->nx * c->ny > kPersistMaxCells) return FDTD2D_OK;
  // a staged path forced by name is kept
  if (mode < 0 && (std::getenv("FDTD2D_TMA") || std::getenv("FDTD2D_TMAT") || std::getenv("FDTD2D_TB")))
    return FDTD2D_OK;
  const int ctas = persist_resident_ctas(c->medium, device);
  const int work = ctas * (kThreads / 32) - c->n_rc - (c->line_n > 0 ? 1 : 0);
  if (ctas <= 0 || work < 1) return FDTD2D_OK;
  const ChoiceKey key = choice_key(c, device, c->medium == FDTD2D_MEDIUM_UNIFORM ? "persist0" : "persist1");
  KernelChoice known;
  const bool have = mode < 0 && find_choice(key, &known);
  note_choice(c, have, known);
  if (have && known.k != 1) return FDTD2D_OK;
  if (mode < 0 && !have && c->path_ms <= 0.f && c->tma) return FDTD2D_OK;   // nothing to compare with
  // units down to one row: a step's time is the longest warp's chain of
  // dependent loads, which grows with its rows (512^2: 6.8 against 12.7 us
  // per step with two-row units)
  const std::vector<int4> units = make_units(0, c->nx, c->ny, work, kCols, 1);
  cudaError_t e = dalloc(c, &c->d_punits, units.size());
  if (e == cudaSuccess) e = dalloc(c, &c->d_bar, 1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_punits, units.data(), units.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return fail_cuda(c, e);
  c->n_punits = (int)units.size();
  c->persist_ctas = ctas;
  bool use = mode == 1 || have;
  if (!use) {
    DevShot t = h;
    t.record = 0;
    t.dft = nullptr;
    const int n1 = t.base_n + 1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float path = c->path_ms, ms = -1.f;
    if (e == cudaSuccess && !c->tma) {
      // the streaming kernel's step (never timed at create)
      for (int r = 0; r < 4 && e == cudaSuccess; ++r) {
        if (r == 1) e = cudaEventRecord(e0, c->stream);
        if (e == cudaSuccess) e = launch_step(t, c->d_units, c->n_units, n1, c->medium, c->grid_warps, c->stream);
      }
      if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&path, e0, e1);
      path /= 3;
    }
    const PersistAux none{};
    if (e == cudaSuccess) e = launch_persist_ordered(c, t, n1, n1, 4, none);
    if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
    if (e == cudaSuccess) e = launch_persist_ordered(c, t, n1, n1, 16, none);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return fail_cuda(c, e);
    int derr = 0;
    if (read_err(c, &derr) != cudaSuccess) return FDTD2D_ERR_CUDA;
    if (derr != kErrNone) return FDTD2D_ERR_TIMEOUT;
    use = ms / 16 < 0.9f * path;
    if (mode < 0) {
      KernelChoice ch;
      ch.k = use ? 1 : 0;
      keep_choice(key, ch);
    }
  }
  if (use) {
    c->persist = true;
    std::snprintf(c->kernel_name, sizeof c->kernel_name, "step_persist_kernel<%d>",
                  c->medium == FDTD2D_MEDIUM_UNIFORM ? 0 : 1);
  }
  return FDTD2D_OK;
}

int setup_tmat(fdtd2d_ctx* c, int device) {
  const char* env = std::getenv("FDTD2D_TMAT");
  if (env && std::strcmp(env, "0") == 0) return FDTD2D_OK;
  if (!tensor_encoder()) return FDTD2D_OK;
  int forced = -1;
  if (env) {
    int w = 0, r = 0, st = 0;
    if (std::sscanf(env, "%d,%d,%d", &w, &r, &st) == 3)
      for (int k = 0; k < tmat_shape_count(); ++k) {
        int a, b, d;
        tmat_shape_dims(k, &a, &b, &d);
        if (a == w && b == r && d == st) forced = k;
      }
  }
  const char* tbe = std::getenv("FDTD2D_TB");
  int tb_mode = tbe ? std::atoi(tbe) : -1;   // -1 both forms, 0 one-step only, 1 two-step only
  const ChoiceKey key = choice_key(c, device, "tmat");
  KernelChoice known;
  bool have = find_choice(key, &known);
  note_choice(c, have, known);
  if (!have && c->untimed && forced < 0 && tb_mode != 0) {
    // no timing: the shapes the timing keeps most often on GB300 (two steps
    // per pass; 4 warps x 2 rows x 2 stages in FP32, 4 x 4 x 2 with 16-bit
    // storage; 2-warp, 2-stage one-row shape on the CPML bands), not stored
    known.k = c->h.store == FDTD2D_STORE_F32 ? tmat_shape_find(4, 2, 2) : tmat_shape_find(4, 4, 2);
    known.q = tma_shape_find(2, 2);
    known.lv = 2;
    have = known.k >= 0 && known.q >= 0;
    if (have) c->choice_src = std::max(c->choice_src, 3);
  }
  if (have && known.k < 0) return FDTD2D_OK;   // the one-row kernel alone won for this class
  if (have) {
    forced = known.k;
    tb_mode = known.lv == 2 ? 1 : 0;
  }
  const char* full_env = std::getenv("FDTD2D_TMAT_AUTOTUNE");
  const bool full = full_env && std::strcmp(full_env, "full") == 0;
  DevShot& h = c->h;
  const int nx = c->nx, ny = c->ny, P = c->npml;
  if (!c->side) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_t, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_e, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_m, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail_cuda(c, e);
  }
  // Two-step form: two more field buffers, copies of the first (cells that
  // no kernel writes keep their values in every buffer), its unit counter,
  // and a scratch psi slab for the trials (a trial pair's second step writes
  // psi buffer 0).
  // (the two-step kernel takes the interior denominators as constants)
  bool try2 = tb_mode != 0 && c->n_steps >= 2 && ny - 2 * P - 4 >= 8 && h.den_uniform;
  float* psi_trial = nullptr;
  const size_t psi_floats = (size_t)h.psi_buf * 2 + 1024;
  auto give_back = [&](float*& p) {
    if (!p) return;
    cudaFreeAsync(p, c->stream);
    auto it = std::find(c->allocs.begin(), c->allocs.end(), (void*)p);
    if (it != c->allocs.end()) c->allocs.erase(it);
    p = nullptr;
  };
  if (try2) {
    const size_t fbytes = (size_t)h.cells * 4 * store_bytes(h.store);
    cudaError_t e = dalloc(c, &h.fb[2], fbytes / 4);
    if (e == cudaSuccess) e = dalloc(c, &h.fb[3], fbytes / 4);
    if (e == cudaSuccess && !c->d_ctr) e = dalloc(c, &c->d_ctr, 1);
    if (e == cudaSuccess) e = cudaMallocAsync(&psi_trial, psi_floats * 4, c->stream);
    if (e == cudaErrorMemoryAllocation) {
      // no room for the two-step form's buffers: the one-step forms only
      cudaGetLastError();
      give_back(h.fb[2]);
      give_back(h.fb[3]);
      if (psi_trial) cudaFreeAsync(psi_trial, c->stream);
      psi_trial = nullptr;
      try2 = false;
      if (tb_mode == 1) return FDTD2D_OK;   // only the two-step form was asked for: the one-row kernel
      e = cudaSuccess;
    } else {
      if (e == cudaSuccess) e = cudaMemcpyAsync(h.fb[2], h.fb[0], fbytes, cudaMemcpyDeviceToDevice, c->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h.fb[3], h.fb[0], fbytes, cudaMemcpyDeviceToDevice, c->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(psi_trial, h.psi, psi_floats * 4, cudaMemcpyDeviceToDevice, c->stream);
    }
    if (e != cudaSuccess) {
      if (psi_trial) cudaFreeAsync(psi_trial, c->stream);
      return fail_cuda(c, e);
    }
  }
  DevShot t = h;
  t.record = 0;
  t.dft = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    if (psi_trial) cudaFreeAsync(psi_trial, c->stream);
    return FDTD2D_ERR_CUDA;
  }
  // Trials time `reps` steps (pairs: reps pairs, halved), about 0.6 ms of
  // work at ~200 Gcell/s and at least 3: at 2048^2 three pairs (~0.1 ms)
  // picked the one-step form for F16 at 155 Gcell/s where two steps per
  // pass run at 179.
  const int reps = (int)std::max<int64_t>(3, std::min<int64_t>(24, (int64_t)(0.6e-3 / (5e-12 * (double)nx * ny)) + 1));
  auto timed = [&](auto&& step) -> float {
    cudaError_t e = step();
    if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = step();
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = -1.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    return e == cudaSuccess ? ms : -1.f;
  };
  // a pair trial: pairs issued back to back (the band kernel's second step
  // of one beside the next one's interior kernel), timed to the last kernel
  auto timed2 = [&](auto&& pair) -> float {
    cudaError_t e = pair();
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
    if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = pair();
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = -1.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    return e == cudaSuccess ? ms : -1.f;
  };
  const int n1 = t.base_n + 1;
  float best = 1e30f;   // per step
  if (!have && forced < 0 && tb_mode != 1) {
    best = timed([&] { return launch_step_tma(c->tma_shape, t, c->d_units, c->n_units, n1, c->grid_warps, c->d_err,
                                              c->stream); });
    if (best < 0) best = 1e30f;
  }
  int best_k = -1, best_q = -1, best_ectas = 0, best_l = 1;
  std::vector<int4> best_t, best_e;
  int best_nring = 0;
  TensorMaps best_m{};
  const int quick_q[3] = {tma_shape_find(2, 2), tma_shape_find(4, 2), tma_shape_find(4, 3)};
  for (int k = 0; k < tmat_shape_count(); ++k) {
    if (forced >= 0 && k != forced) continue;
    if (forced < 0 && !full && k >= 2 && k != tmat_shape_find(4, 2, 2)) continue;   // the shapes that win
    const int bt = tmat_band_cols(k), R = tmat_rows(k);
    TensorMaps maps{};
    if (ny - 2 * P < 4 * R + 2 || !encode_maps(h, nx, ny, tmat_box_cols(k), R, &maps)) continue;
    // every one-row shape is a candidate for the CPML bands and rows
    // (FDTD2D_TMA=W,ST forces one)
    const int q_forced = have ? known.q : tma_shape_parse(std::getenv("FDTD2D_TMA"));
    // both forms' launch attributes are set here: the two-step path also
    // runs single steps (an odd step, a step the line probe reads)
    const int tctas1 = tmat_resident_ctas(k, h.store, device);
    const int tctas2 = try2 ? tmat2_resident_ctas(k, h.store, device) : 0;
    for (int lv = 1; lv <= 2; ++lv) {
      if ((lv == 2 && !try2) || (lv == 1 && tb_mode == 1)) continue;
      // Where two steps per pass can run, the quick search times only that
      // form: forced runs of every tensor shape at 1024^2-3072^2, FP32 and
      // F16, found it 5-60 % faster than one step per pass, and short trials
      // of both forms picked the one-step form at 1024^2 and 2048^2.
      if (lv == 1 && try2 && tb_mode < 0 && !full) continue;
      const int tctas = lv == 1 ? tctas1 : tctas2;
      // interior region: rows [ri0, ri1), columns [ci0, ci1) with ci0 the
      // first multiple of the one-row band at or past the CPML (two-step
      // form: two cells further in on every side, so that the frame kernel's
      // cells and their neighbours have no CPML), then whole tensor bands
      // (two-step form: whole one-row bands; the first tensor unit of a row
      // range then starts `lead` columns left of ci0, and its warps there
      // idle)
      const int ri0 = lv == 1 ? P : P + 2, ri1 = ny - ri0;
      for (int q = 0; q < tma_shape_count(); ++q) {
        if (q_forced >= 0 && q != q_forced) continue;
        if (q_forced < 0 && !full && q != quick_q[0] && q != quick_q[1] && q != quick_q[2]) continue;
        const int b1 = tma_band_cols(q);
        const int gran = lv == 1 ? bt : b1;
        const int ci0 = (ri0 + b1 - 1) / b1 * b1;
        const int ci1 = ci0 + std::max(0, (nx - ri0 - ci0) / gran) * gran;
        if (ci1 - ci0 < bt) continue;
        const int ectas = tma_resident_ctas(q, P, h.store, device);
        std::vector<int4> tu, eu;
        const int nbt = (ci1 - ci0 + bt - 1) / bt;
        const int lead = nbt * bt - (ci1 - ci0);   // a multiple of kCols below bt
        // (two-step form: about three units per CTA, taken in turn)
        add_units(tu, ci0 - lead, ci1, bt, ri0, ri1,
                  std::min((lv == 1 ? 1 : 3) * std::max(1, tctas / nbt), (ri1 - ri0) / (2 * R)));
        if (lv == 2)
          for (int4& u : tu)
            u.x = (h.store == FDTD2D_STORE_F32
                       ? (u.z == ri0 ? kRingTop : 0) | (u.w == ri1 ? kRingBottom : 0) |
                             (u.y == ci0 - lead ? kRingLeft : 0) | (u.y + bt == ci1 ? kRingRight : 0)
                       : 0) |
                  (u.y == ci0 - lead ? (lead / kCols) << 4 : 0);
        int nring = 0;
        if (lv == 2 && h.store != FDTD2D_STORE_F32) {
          // 16-bit storage: ring units first, step n of R's edge cells, 4 per thread
          const int cells = 2 * (ci1 - ci0) + 2 * std::max(0, ri1 - ri0 - 2);
          std::vector<int4> ru;
          for (int t = 0; t < cells; t += 4 * kCols) ru.push_back(make_int4(kUnitRing, t, std::min(cells, t + 4 * kCols), 0));
          nring = (int)ru.size();
          tu.insert(tu.begin(), ru.begin(), ru.end());
        }
        eu = edge_units(nx, ny, P, ci0, ci1, ri0, ri1, b1, ectas);
        int4 *dt = nullptr, *de = nullptr;
        cudaError_t e = cudaMallocAsync(&dt, tu.size() * sizeof(int4), c->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&de, eu.size() * sizeof(int4), c->stream);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(dt, tu.data(), tu.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(de, eu.data(), eu.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
        float ms = -1.f;
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_m, c->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_m, 0);
        // one trial step (pair) as fdtd2d_run issues it: the two kernels on two streams
        if (e == cudaSuccess && have) {
          ms = 0.f;   // the stored choice
        } else if (e == cudaSuccess && lv == 1) {
          ms = timed([&] {
            cudaError_t x = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
            if (x == cudaSuccess) x = launch_step_tmat(k, t, maps, dt, (int)tu.size(), n1, tctas, c->d_err, c->stream);
            if (x == cudaSuccess) x = cudaStreamWaitEvent(c->side, c->ev_t, 0);
            if (x == cudaSuccess) x = cudaEventRecord(c->ev_t, c->stream);
            if (x == cudaSuccess) x = launch_step_tma(q, t, de, (int)eu.size(), n1, ectas, c->d_err, c->side);
            if (x == cudaSuccess) x = cudaEventRecord(c->ev_e, c->side);
            if (x == cudaSuccess) x = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
            return x;
          });
        } else if (e == cudaSuccess) {
          // pairs as the run issues them, the field slots rotating from pair
          // to pair (all at step n1: the values are not used), psi into the
          // scratch slab; the shot's buffers are zeroed again after the trials
          // (a trial that kept reading one slot and writing another measured
          // within ~10 % of the run, enough to pick the wrong shape)
          const PairPlan pl{k, tctas, (int)tu.size(), dt, q, ectas, (int)eu.size(), de, ci0, ci1, ri0, ri1};
          DevShot t2 = t;
          t2.psi = psi_trial;
          TensorMaps m2 = maps;
          ms = timed2([&] { return issue_pair(c, pl, t2, m2, n1); });
          if (ms >= 0) ms *= 0.5f;
        }
        if (dt) cudaFreeAsync(dt, c->stream);
        if (de) cudaFreeAsync(de, c->stream);
        if (ms >= 0 && ms < best) {
          best = ms;
          best_k = k;
          best_q = q;
          best_l = lv;
          best_ectas = ectas;
          best_t = tu;
          best_nring = nring;
          best_e = eu;
          best_m = maps;
          c->tmat_ctas = tctas1;
          c->tmat2_ctas = tctas2;
          c->reg[0] = ci0;
          c->reg[1] = ci1;
          c->reg[2] = ri0;
          c->reg[3] = ri1;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (psi_trial) cudaFreeAsync(psi_trial, c->stream);
  if (!have && best > 0.f && best < 1e29f) c->path_ms = best / reps;   // trials time `reps` steps
  // the trials wrote the shot's field buffers and psi: back to their state
  // at create, all zero
  if (!have) {
    const size_t fbytes = (size_t)h.cells * 4 * store_bytes(h.store);
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 4 && e == cudaSuccess; ++b)
      if (h.fb[b]) e = cudaMemsetAsync(h.fb[b], 0, fbytes, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h.psi, 0, ((size_t)h.psi_buf * 2 + 1024) * sizeof(float), c->stream);
    if (e != cudaSuccess) return fail_cuda(c, e);
  }
  if (h.fb[2] && !(best_k >= 0 && best_l == 2)) {
    // the two-step form lost: give its buffers back
    for (int b = 2; b < 4; ++b) {
      give_back(h.fb[b]);
      std::memset(&best_m.hj[b], 0, sizeof best_m.hj[b]);
      std::memset(&best_m.e[b], 0, sizeof best_m.e[b]);
    }
  }
  int derr = 0;
  if (read_err(c, &derr) != cudaSuccess) return FDTD2D_ERR_CUDA;
  if (derr != kErrNone) return FDTD2D_ERR_TIMEOUT;
  if (!have) {
    KernelChoice ch;
    ch.k = best_k;
    ch.q = best_q;
    ch.lv = best_l;
    keep_choice(key, ch);
  }
  if (best_k < 0) return FDTD2D_OK;
  cudaError_t e = dalloc(c, &c->d_tunits, best_t.size());
  if (e == cudaSuccess) e = dalloc(c, &c->d_eunits, best_e.size());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_tunits, best_t.data(), best_t.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_eunits, best_e.data(), best_e.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail_cuda(c, e);
  c->tmat = true;
  c->tb = best_l == 2;
  c->tmat_shape = best_k;
  c->tma_shape = best_q;          // the one-row kernel's shape on the CPML bands and rows
  c->grid_warps = best_ectas;
  c->n_tunits = (int)best_t.size();
  c->n_ring = best_nring;
  c->n_eunits = (int)best_e.size();
  c->maps = best_m;
  int w, r, st;
  tmat_shape_dims(best_k, &w, &r, &st);
  char one[48];
  tma_shape_name(c->tma_shape, "step_tma_kernel", one, sizeof one);
  std::snprintf(c->kernel_name, sizeof c->kernel_name, "%s<%d,%d,%d>+%s", c->tb ? "step_tmat2_kernel" : "step_tmat_kernel",
                w, r, st, one);
  return FDTD2D_OK;
}

}  // namespace

int fdtd2d::validate_setup(const fdtd2d_setup* s) { return validate(s); }

void fdtd2d::adopt_ctx(fdtd2d_ctx* c, cudaStream_t batch_stream) {
  cudaSetDevice(c->device);
  if (c->stream && !c->batch) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  for (cudaEvent_t ev : {c->ev_t, c->ev_e, c->ev_m, c->ev_a})
    if (ev) cudaEventDestroy(ev);
  c->stream = batch_stream;
  c->batch = true;
}

int fdtd2d::create_ctx(const fdtd2d_setup* s, int device, bool member, fdtd2d_ctx** out, bool solo,
                       bool untimed) {
  if (!out) return FDTD2D_ERR_INVALID;
  *out = nullptr;
  int rc = validate(s);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FDTD2D_ERR_NODEVICE;
  if (device < 0 || device >= ndev) return FDTD2D_ERR_INVALID;

  fdtd2d_ctx* c = new (std::nothrow) fdtd2d_ctx();
  if (!c) return FDTD2D_ERR_NOMEM;
  c->device = device;
  c->solo = solo;
  c->untimed = untimed;
  if (const char* v = std::getenv("FDTD2D_TEST_FAIL_ALLOC")) c->fail_alloc = std::atoi(v);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) keep_pool_memory(device);
  if (e != cudaSuccess) {
    rc = fail_cuda(c, e);
    fdtd2d_destroy(c);
    return rc;
  }
  const int nx = s->nx, ny = s->ny, P = s->npml;
  const int pitch = pitch_for(nx);
  const int64_t cells = buffer_floats(nx, ny);
  c->nx = nx; c->ny = ny; c->pitch = pitch; c->npml = P; c->n_steps = s->n_steps;
  c->n_det = s->n_det; c->n_comp = s->n_comp; c->record = s->record_traces ? 1 : 0;
  c->medium = s->medium;
  c->dft = s->dft_freq > 0 && s->n_det > 0;
  // Test parameters of the persistent kernel's grid barrier (the test that
  // makes a wait run out): its bound in ns and a count added to its target.
  if (const char* v = std::getenv("FDTD2D_WAIT_NS")) c->wait_ns = std::strtoull(v, nullptr, 10);
  if (const char* v = std::getenv("FDTD2D_TEST_BARRIER_EXTRA")) c->bar_extra = std::max(0, std::atoi(v));

  DevShot& h = c->h;
  h.nx = nx; h.ny = ny; h.pitch = pitch; h.npml = P; h.n_steps = s->n_steps; h.base_n = 0;
  const double nudt = 0.5 * s->nu * s->dt;
  h.ja = (float)((1.0 - nudt) / (1.0 + nudt));
  const double beta = s->jz_coef * s->dt / (1.0 + nudt);
  h.dx = (float)s->dx; h.dy = (float)s->dy;
  // a material medium the uniform one represents exactly runs as uniform
  // (FDTD2D_MATERIAL_AS_UNIFORM=0 keeps the material kernel)
  bool as_uniform = false;
  float u_ca = 0.f, u_cb = 0.f, u_da = 0.f, u_db = 0.f;
  std::vector<float> u_kp;
  if (s->medium == FDTD2D_MEDIUM_MATERIAL_ID && s->storage == FDTD2D_STORE_F32) {
    const char* v = std::getenv("FDTD2D_MATERIAL_AS_UNIFORM");
    if (!(v && std::strcmp(v, "0") == 0)) as_uniform = material_as_uniform(s, beta, &u_ca, &u_cb, &u_da, &u_db, &u_kp);
  }
  if (as_uniform) c->medium = FDTD2D_MEDIUM_UNIFORM;

#define CK(expr)                     \
  do {                               \
    cudaError_t _e = (expr);         \
    if (_e != cudaSuccess) {         \
      rc = fail_cuda(c, _e);         \
      fdtd2d_destroy(c);             \
      return rc;                     \
    }                                \
  } while (0)
#define CK_RC(expr)                  \
  do {                               \
    rc = (expr);                     \
    if (rc != FDTD2D_OK) {           \
      fdtd2d_destroy(c);             \
      return rc;                     \
    }                                \
  } while (0)

  h.cells = cells;
  h.store = s->storage;
  for (int a = 0; a < 5; ++a) h.sc[a] = h.isc[a] = 1.f;
  const int es = store_bytes(h.store);
  {
    float* slab = nullptr;
    CK(dalloc(c, &slab, (size_t)cells * 8 * es / 4));
    h.fb[0] = slab;
    h.fb[1] = reinterpret_cast<float*>(reinterpret_cast<char*>(slab) + (size_t)cells * 4 * es);
  }
  h.o_ezy = (int64_t)2 * (P - 1) * pitch;
  h.o_hyx = h.o_ezy + (int64_t)2 * P * pitch;
  h.o_ezx = h.o_hyx + (int64_t)2 * ny * P;
  h.psi_buf = h.o_ezx + (int64_t)2 * ny * P;
  // + slack for the staged kernel's whole-band copies of the last psi_Ezy row
  // and the 16-byte round-up of its x-strip row copies
  CK(dalloc(c, &h.psi, (size_t)h.psi_buf * 2 + 1024));

  // medium
  if (as_uniform) {
    h.ca = u_ca; h.cb = u_cb; h.da = u_da; h.db = u_db;
    if (!u_kp.empty()) {
      float* kp_buf = nullptr;
      CK(dalloc(c, &kp_buf, cells));
      CK(cudaMemcpy2DAsync(kp_buf + kMargin, pitch * sizeof(float), u_kp.data(), nx * sizeof(float),
                           nx * sizeof(float), ny, cudaMemcpyHostToDevice, c->stream));
      CK(cudaStreamSynchronize(c->stream));   // u_kp is released when create returns
      h.kp = kp_buf + kMargin;
    }
  } else if (s->medium == FDTD2D_MEDIUM_UNIFORM) {
    h.ca = s->ca; h.cb = s->cb; h.da = s->da; h.db = s->db;
    if (h.store != FDTD2D_STORE_F32) set_storage_scales(s, beta, &h);
    if (s->ne) {
      float* kp_buf = nullptr;
      if (h.store == FDTD2D_STORE_F32) {
        CK(dalloc(c, &kp_buf, cells));
      } else {
        CK(cudaMallocAsync(&kp_buf, (size_t)cells * sizeof(float), c->stream));   // FP32 staging
        CK(cudaMemsetAsync(kp_buf, 0, (size_t)cells * sizeof(float), c->stream));
      }
      float* kp = kp_buf + kMargin;
      CK(cudaMemcpy2DAsync(kp, pitch * sizeof(float), s->ne, nx * sizeof(float), nx * sizeof(float),
                           ny, cudaMemcpyHostToDevice, c->stream));
      drive_from_density<<<1024, 256, 0, c->stream>>>(kp, pitch, nx, ny, (float)beta);
      ++c->launches;
      CK(cudaGetLastError());
      if (h.store == FDTD2D_STORE_F32) {
        h.kp = kp;
      } else {
        uint16_t* kp16 = nullptr;
        CK(dalloc(c, &kp16, (size_t)cells));
        CK(launch_to_storage(kp_buf, kp16, cells, h.store, h.isc[4], c->stream));
        ++c->launches;
        CK(cudaFreeAsync(kp_buf, c->stream));
        h.kp = reinterpret_cast<const float*>(kp16 + kMargin);   // elements of the storage type
      }
    }
  } else {
    std::vector<uint8_t> ids((size_t)cells * 3, 0);
    const int32_t* src[3] = {s->id1, s->id2, s->id3};
    for (int m = 0; m < 3; ++m) {
      for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
          const int32_t v = src[m][(int64_t)j * nx + i];
          if (v < 0 || v >= s->n_materials) {
            fdtd2d_destroy(c);
            return FDTD2D_ERR_RANGE;
          }
          ids[(size_t)m * cells + kMargin + (size_t)j * pitch + i] = (uint8_t)v;
        }
      }
    }
    uint8_t* d_ids = nullptr;
    CK(dalloc(c, &d_ids, ids.size()));
    CK(cudaMemcpyAsync(d_ids, ids.data(), ids.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    h.id1 = d_ids + kMargin; h.id2 = d_ids + cells + kMargin; h.id3 = d_ids + 2 * cells + kMargin;
    std::vector<MatE> me(256);
    std::vector<MatH> mh(256);
    for (int m = 0; m < 256; ++m) {
      me[m] = MatE{0.f, 0.f, 0.f, m == 1 ? 1.f : 0.f};
      mh[m] = MatH{0.f, 0.f};
      if (m < s->n_materials) {
        const double ne = s->mat_ne[m];
        me[m].ca = s->mat_ca[m];
        me[m].cb = s->mat_cb[m];
        me[m].kp = ne > 0 ? (float)(beta * ne) : 0.f;
        mh[m].da = s->mat_da[m];
        mh[m].db = s->mat_db[m];
      }
    }
    MatE* d_me = nullptr;
    MatH* d_mh = nullptr;
    CK(dalloc(c, &d_me, 256));
    CK(dalloc(c, &d_mh, 256));
    CK(cudaMemcpyAsync(d_me, me.data(), 256 * sizeof(MatE), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_mh, mh.data(), 256 * sizeof(MatH), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    h.mat_e = d_me; h.mat_h = d_mh;
  }

  // CPML and denominator tables
  {
    std::vector<float> tab((size_t)kCpmlRows * P, 0.f);
    const float* rows[kCpmlRows] = {s->be_x_1, s->ce_x_1, s->be_x_2, s->ce_x_2, s->bh_x_1, s->ch_x_1,
                                    s->bh_x_2, s->ch_x_2, s->be_y_1, s->ce_y_1, s->be_y_2, s->ce_y_2,
                                    s->bh_y_1, s->ch_y_1, s->bh_y_2, s->ch_y_2};
    // b rows as given; c rows hold c/d (d = dx for the x strips, dy for the
    // y strips), so the kernels multiply instead of dividing.
    for (int r = 0; r < kCpmlRows; ++r) {
      const bool hrow = (r % 8) >= 4;
      const int len = hrow ? P - 1 : P;
      const bool crow = (r % 2) == 1;
      const double d = r < 8 ? (double)s->dx : (double)s->dy;
      for (int k = 0; k < len; ++k)
        tab[(size_t)r * P + k] = crow ? (float)((double)rows[r][k] / d) : rows[r][k];
    }
    std::vector<float> dex(pitch, 0.f), dhx(pitch, 0.f), dey(ny, 0.f), dhy(ny, 0.f);
    for (int i = 0; i < nx - 1; ++i) { dex[i] = s->den_ex[i]; dhx[i] = s->den_hx[i]; }
    for (int j = 0; j < ny - 1; ++j) { dey[j] = s->den_ey[j]; dhy[j] = s->den_hy[j]; }
    // each table constant over the CPML-free columns / rows (bitwise)?
    auto constant = [](const std::vector<float>& v, int a, int b, float* out) {
      if (b < a) return false;
      for (int k = a + 1; k <= b; ++k)
        if (std::memcmp(&v[k], &v[a], sizeof(float)) != 0) return false;
      *out = v[a];
      return true;
    };
    h.den_uniform = constant(dex, P, nx - P - 1, &h.den_c[0]) && constant(dhx, P, nx - P - 1, &h.den_c[1]) &&
                    constant(dey, P, ny - P - 1, &h.den_c[2]) && constant(dhy, P, ny - P - 1, &h.den_c[3]);
    float *d_tab, *d_dex, *d_dhx, *d_dey, *d_dhy;
    CK(dalloc(c, &d_tab, tab.size()));
    CK(dalloc(c, &d_dex, (size_t)pitch));
    CK(dalloc(c, &d_dhx, (size_t)pitch));
    CK(dalloc(c, &d_dey, (size_t)ny));
    CK(dalloc(c, &d_dhy, (size_t)ny));
    CK(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_dex, dex.data(), pitch * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_dhx, dhx.data(), pitch * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_dey, dey.data(), ny * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_dhy, dhy.data(), ny * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    h.cpml = d_tab; h.den_ex = d_dex; h.den_hx = d_dhx; h.den_ey = d_dey; h.den_hy = d_dhy;
  }

  // points by row: sources, Ez detectors, component detectors
  {
    struct Pt { int j, kind, i, idx; };
    std::vector<Pt> pts;
    for (int e = 0; e < s->n_src; ++e) pts.push_back({s->src[e].j, kPointSource, s->src[e].i, e});
    for (int e = 0; e < s->n_det; ++e) pts.push_back({s->det[e].j, kPointDetEz, s->det[e].i, e});
    for (int e = 0; e < s->n_comp; ++e) pts.push_back({s->comp[e].j, kPointDetComp, s->comp[e].i, e});
    std::stable_sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& b) {
      if (a.j != b.j) return a.j < b.j;
      if (a.kind != b.kind) return a.kind < b.kind;
      return a.i < b.i;
    });
    std::vector<int> row_start(ny + 1, 0);
    for (const Pt& p : pts) row_start[p.j + 1]++;
    for (int j = 0; j < ny; ++j) row_start[j + 1] += row_start[j];
    std::vector<int4> dp(std::max<size_t>(1, pts.size()));
    for (size_t q = 0; q < pts.size(); ++q) dp[q] = make_int4(pts[q].i, pts[q].kind, pts[q].idx, 0);
    int* d_rs;
    int4* d_pts;
    CK(dalloc(c, &d_rs, row_start.size()));
    CK(dalloc(c, &d_pts, dp.size()));
    CK(cudaMemcpyAsync(d_rs, row_start.data(), row_start.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_pts, dp.data(), dp.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    h.row_start = d_rs;
    h.pts = d_pts;
  }

  // source waveform and DFT twiddle tables (FP64 on the device, once)
  {
    std::vector<float> env(s->n_steps + 1, 0.f);
    const int nsrc = std::max(1, s->n_src);
    std::vector<double> ph(nsrc, 0.0);
    if (s->n_src > 0) {
      for (int n = 0; n <= s->n_steps; ++n) env[n] = s->envelope[n];
      for (int e = 0; e < s->n_src; ++e) ph[e] = s->src_phase_deg[e] / 360.0;
    }
    float* d_env;
    double* d_ph;
    float* d_val;
    double2* d_tw = nullptr;
    CK(dalloc(c, &d_env, env.size()));
    CK(dalloc(c, &d_ph, ph.size()));
    CK(dalloc(c, &d_val, (size_t)(s->n_steps + 1) * nsrc));
    if (c->dft) CK(dalloc(c, &d_tw, (size_t)(s->n_steps + 1)));
    CK(cudaMemcpyAsync(d_env, env.data(), env.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_ph, ph.data(), ph.size() * 8, cudaMemcpyHostToDevice, c->stream));
    const double beta_half = (s->f1 != s->f0) ? 0.5 * (s->f1 - s->f0) / s->t1 : 0.0;
    const double src_pi = s->src_pi > 0 ? s->src_pi : kPi;
    CK(build_source_tables(d_val, d_tw, d_env, d_ph, nsrc, s->n_steps, s->dt, s->src_scale, s->f0,
                           beta_half, src_pi, s->dft_freq * s->dt, c->stream));
    ++c->launches;
    CK(cudaStreamSynchronize(c->stream));
    h.src_val = d_val;
    h.twiddle = d_tw;
    h.n_src = nsrc;
  }

  // detector outputs
  h.n_det = s->n_det;
  h.n_comp = s->n_comp;
  h.record = c->record;
  if (c->record) {
    CK(dalloc(c, &h.trace, (size_t)s->n_steps * std::max(1, s->n_det)));
    CK(dalloc(c, &h.ctrace, (size_t)s->n_steps * std::max(1, s->n_comp) * 3));
  }
  if (c->dft) CK(dalloc(c, &h.dft, (size_t)s->n_det));

  for (int k = 0; k < 8; ++k) {
    const int64_t v = s->cover[k];
    h.cov[k] = (s->medium != FDTD2D_MEDIUM_MATERIAL_ID || as_uniform || v == 0) ? INT64_MAX : (v < 0 ? 0 : v);
  }

  // wave-front tracker and line probe
  if (s->n_rc > 0) {
    c->n_rc = s->n_rc;
    c->rc_j_cut = s->rc_j_cut;
    c->rc_level = s->rc_level;
    CK(dalloc(c, &c->d_rc_scan, (size_t)s->n_rc));
    CK(dalloc(c, &c->d_rc_max, (size_t)s->n_rc));
    CK(dalloc(c, &c->d_edge, (size_t)s->n_rc));
    CK(dalloc(c, &c->d_spd, (size_t)s->n_steps * s->n_rc));
    std::vector<float> e0(s->n_rc, s->rc_edge0);
    CK(cudaMemcpyAsync(c->d_rc_scan, s->rc_scan_i, s->n_rc * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_rc_max, s->rc_max_i, s->n_rc * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_edge, e0.data(), s->n_rc * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (s->line_n > 0) {
    c->line_n = s->line_n; c->line_i0 = s->line_i0; c->line_j = s->line_j;
    c->line_first = s->line_first; c->line_last = s->line_last;
    CK(dalloc(c, &c->d_line, (size_t)(s->line_last - s->line_first + 1) * s->line_n));
  }

  CK(dalloc(c, &c->d_shot, 1));
  CK(cudaMemcpyAsync(c->d_shot, &h, sizeof(DevShot), cudaMemcpyHostToDevice, c->stream));
  // Kernel: the shared-memory staged step for the uniform medium with a CPML
  // of at most tma_max_pml() cells, unless FDTD2D_KERNEL=stream selects the
  // register-streaming one; the material-ID medium (Settings.ini path) and
  // deeper CPMLs always stream.
  {
    const char* k = std::getenv("FDTD2D_KERNEL");
    c->tma = (c->medium == FDTD2D_MEDIUM_UNIFORM) && P <= tma_max_pml() &&
             (h.store != FDTD2D_STORE_F32 || !(k && std::strcmp(k, "stream") == 0));
  }
  CK(dalloc(c, &c->d_err, 1));
  std::vector<int4> units;
  if (c->tma) {
    // FDTD2D_TMA="W,ST" picks a compiled launch shape (W warps, ST stages);
    // otherwise the shapes are timed on this shot and the fastest is kept,
    // unless FDTD2D_TMA_AUTOTUNE=0 (then shape 0).
    const int forced = tma_shape_parse(std::getenv("FDTD2D_TMA"));
    const char* at = std::getenv("FDTD2D_TMA_AUTOTUNE");
    KernelChoice known;
    if (member) {
      // batch members are stepped by the batch's kernel
    } else if (forced >= 0) {
      c->tma_shape = forced;
    } else if (!(at && std::strcmp(at, "0") == 0) && c->n_steps >= 1 &&
               find_choice(choice_key(c, device, "tma"), &known)) {
      c->tma_shape = known.q;   // timed for a shot of this class before
      note_choice(c, true, known);
    } else if (c->untimed) {
      // no timing: the compiled default shape
    } else if (!(at && std::strcmp(at, "0") == 0) && c->n_steps >= 1) {
      // Each trial re-runs step 1 with traces and the DFT switched off: a
      // step reads one buffer set and overwrites the other with values that
      // depend on the first alone, so the trials leave nothing behind once
      // step 1 runs for real.
      DevShot t = h;
      t.record = 0;
      t.dft = nullptr;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      float best = 0.f;
      int best_k = 0;
      for (int k = 0; k < tma_shape_count(); ++k) {
        const int ctas = tma_resident_ctas(k, P, h.store, device);
        const std::vector<int4> u = make_units(0, nx, ny, ctas, tma_band_cols(k));
        int4* du = nullptr;
        cudaError_t e = cudaMalloc(&du, u.size() * sizeof(int4));
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(du, u.data(), u.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
        for (int r = 0; r < 4 && e == cudaSuccess; ++r) {
          if (r == 1) e = cudaEventRecord(e0, c->stream);
          if (e == cudaSuccess) e = launch_step_tma(k, t, du, (int)u.size(), t.base_n + 1, ctas, c->d_err, c->stream);
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (du) cudaFree(du);
        if (e != cudaSuccess) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          rc = fail_cuda(c, e);
          fdtd2d_destroy(c);
          return rc;
        }
        if (k == 0 || ms < best) { best = ms; best_k = k; }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      int derr = 0;
      CK(read_err(c, &derr));
      if (derr != kErrNone) {
        fdtd2d_destroy(c);
        return FDTD2D_ERR_TIMEOUT;
      }
      c->tma_shape = best_k;
      c->path_ms = best / 3;   // three timed launches
      KernelChoice ch;
      ch.q = best_k;
      keep_choice(choice_key(c, device, "tma"), ch);
    }
    c->grid_warps = tma_resident_ctas(c->tma_shape, P, h.store, device);  // CTAs for this path
    units = make_units(0, nx, ny, c->grid_warps, tma_band_cols(c->tma_shape));
    tma_shape_name(c->tma_shape, "step_tma_kernel", c->kernel_name, sizeof c->kernel_name);
  } else {
    c->grid_warps = resident_warps(c->medium, device);
    // one warp per unit, units of at least 2 rows: a narrow grid (a few
    // 128-column blocks) still fills the resident warps in one wave
    units = make_units(0, nx, ny, c->grid_warps, kCols, 2);
    std::snprintf(c->kernel_name, sizeof c->kernel_name, "step_stream_kernel<%d>", c->medium == FDTD2D_MEDIUM_UNIFORM ? 0 : 1);
  }
  c->n_units = (int)units.size();
  CK(dalloc(c, &c->d_units, units.size()));
  CK(cudaMemcpyAsync(c->d_units, units.data(), units.size() * sizeof(int4), cudaMemcpyHostToDevice,
                     c->stream));
  if (c->tma && !member) CK_RC(setup_tmat(c, device));
  if (!member && !solo) CK_RC(setup_persist(c, device));
  CK(dalloc(c, &c->d_flag, 1));
  CK(cudaStreamSynchronize(c->stream));
#undef CK
#undef CK_RC
  *out = c;
  return FDTD2D_OK;
}

extern "C" {

static int run_body(fdtd2d_ctx* c, int32_t n_first, int32_t n_last);

// The entry point: its body (which may grow the event-timing lists) runs
// behind abi_guard.
int fdtd2d_run(fdtd2d_ctx* c, int32_t n_first, int32_t n_last) {
  return abi_guard([&] { return run_body(c, n_first, n_last); });
}

static int run_body(fdtd2d_ctx* c, int32_t n_first, int32_t n_last) {
  if (!c) return FDTD2D_ERR_INVALID;
  if (c->batch) return FDTD2D_ERR_STATE;   // stepped by its batch
  if (n_first != c->step + 1 || n_last < n_first - 1 || n_last > c->n_steps) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  if (c->tmat && n_first <= n_last) {
    // the side stream starts after the shot stream's earlier work (uploads, writes)
    cudaError_t e = cudaEventRecord(c->ev_m, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_m, 0);
    if (e != cudaSuccess) return fail_cuda(c, e);
  }
  if (c->persist) {
    // all the steps in persistent launches, the tracker and the line probe
    // on their service warps
    PersistAux A{};
    A.wait_ns = c->wait_ns;
    A.bar_extra = c->bar_extra;
    if (c->n_rc > 0) {
      A.n_rc = c->n_rc;
      A.scan_i = c->d_rc_scan;
      A.max_i = c->d_rc_max;
      A.j_cut = c->rc_j_cut;
      A.level = c->rc_level;
      A.edge = c->d_edge;
      A.spd = c->d_spd;
    }
    if (c->line_n > 0) {
      A.line_n = c->line_n;
      A.line_j = c->line_j;
      A.line_i0 = c->line_i0;
      A.line_first = c->line_first;
      A.line_last = c->line_last;
      A.line = c->d_line;
    }
    for (int32_t n = n_first; n <= n_last;) {
      const int32_t m = (int32_t)std::min<int64_t>(n_last, (int64_t)n + kPersistSteps - 1);
      cudaEvent_t p0 = prof_mark(c, nullptr, 0, m - n + 1);
      const cudaError_t e = launch_persist_ordered(c, c->h, n, m, 0, A);
      if (p0) prof_mark(c, p0, (int64_t)c->nx * c->ny, m - n + 1);
      if (e != cudaSuccess) return fail_cuda(c, e);
      ++c->launches;
      c->step = m;
      n = m + 1;
    }
    return FDTD2D_OK;
  }
  bool paired = false;   // the last iteration issued a pair
  for (int32_t n = n_first; n <= n_last; ++n) {
    cudaError_t e;
    // Two steps per pass where nothing reads the fields between them (the
    // tracker and the line probe read every step's Ez).
    if (c->tb && n < n_last && c->n_rc == 0 &&
        !(c->line_n > 0 && n + 1 >= c->line_first && n <= c->line_last)) {
      const PairPlan pl{c->tmat_shape, c->tmat2_ctas, c->n_tunits, c->d_tunits, c->tma_shape, c->grid_warps,
                        c->n_eunits, c->d_eunits, c->reg[0], c->reg[1], c->reg[2], c->reg[3]};
      // after single steps the interior kernel waits for their band kernel
      e = paired ? cudaSuccess : cudaStreamWaitEvent(c->stream, c->ev_e, 0);
      if (e == cudaSuccess) e = issue_pair(c, pl, c->h, c->maps, n);
      if (e == cudaSuccess && n + 1 == n_last) e = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
      if (e != cudaSuccess) return fail_cuda(c, e);
      c->launches += 4;
      c->step = ++n;
      paired = true;
      continue;
    }
    paired = false;
    if (c->tmat) {
      // Interior on the multi-row tensor kernel (shot stream), CPML bands and
      // rows on the staged kernel (side stream), both kernels of a step at
      // once.  Each waits for the other's kernel of the previous step: it
      // overwrites the buffer that kernel read.
      e = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
      cudaEvent_t p0 = c->tb ? nullptr : prof_mark(c, nullptr, 0, 1);
      if (e == cudaSuccess)
        e = launch_step_tmat(c->tmat_shape, c->h, c->maps, c->d_tunits + c->n_ring, c->n_tunits - c->n_ring, n,
                             c->tmat_ctas, c->d_err, c->stream);
      if (p0) prof_mark(c, p0, (int64_t)(c->reg[1] - c->reg[0]) * (c->reg[3] - c->reg[2]), 1);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_t, 0);
      if (e == cudaSuccess) e = cudaEventRecord(c->ev_t, c->stream);
      if (e == cudaSuccess) {
        ++c->launches;
        e = launch_step_tma(c->tma_shape, c->h, c->d_eunits, c->n_eunits, n, c->grid_warps, c->d_err, c->side);
      }
      if (e == cudaSuccess) e = cudaEventRecord(c->ev_e, c->side);
      // what follows on the shot stream (tracker, line probe, reads) sees the whole step
      if (e == cudaSuccess && (c->n_rc > 0 || c->line_n > 0 || n == n_last))
        e = cudaStreamWaitEvent(c->stream, c->ev_e, 0);
    } else {
      cudaEvent_t p0 = prof_mark(c, nullptr, 0, 1);
      e = c->tma ? launch_step_tma(c->tma_shape, c->h, c->d_units, c->n_units, n, c->grid_warps, c->d_err, c->stream)
                 : launch_step(c->h, c->d_units, c->n_units, n, c->medium, c->grid_warps, c->stream);
      if (p0) prof_mark(c, p0, (int64_t)c->nx * c->ny, 1);
    }
    if (e != cudaSuccess) return fail_cuda(c, e);
    ++c->launches;
    const float* ez_now = field_ptr(c->h, kEz, n & 1);
    if (c->n_rc > 0) {
      e = launch_rc(ez_now, c->pitch, c->ny, c->n_rc, c->d_rc_scan, c->d_rc_max, c->rc_j_cut,
                    c->rc_level, c->d_edge, c->d_spd + (size_t)(n - 1) * c->n_rc, c->stream);
      if (e != cudaSuccess) return fail_cuda(c, e);
      ++c->launches;
    }
    if (c->line_n > 0 && n >= c->line_first && n <= c->line_last) {
      e = launch_line(ez_now, c->pitch, c->line_j, c->line_i0, c->line_n,
                      c->d_line + (size_t)(n - c->line_first) * c->line_n, c->stream);
      if (e != cudaSuccess) return fail_cuda(c, e);
      ++c->launches;
    }
    c->step = n;
  }
  return FDTD2D_OK;
}

int fdtd2d_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int fdtd2d_run_timed(fdtd2d_ctx* c, int32_t n_first, int32_t n_last, float* elapsed_ms) {
  if (!c || !elapsed_ms) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaEvent_t a, b;
  cudaError_t e = cudaEventCreate(&a);
  if (e != cudaSuccess) return fail_cuda(c, e);
  e = cudaEventCreate(&b);
  if (e != cudaSuccess) {
    cudaEventDestroy(a);
    return fail_cuda(c, e);
  }
  e = cudaEventRecord(a, c->stream);
  int rc = (e == cudaSuccess) ? fdtd2d_run(c, n_first, n_last) : fail_cuda(c, e);
  if (rc == FDTD2D_OK) {
    e = cudaEventRecord(b, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(elapsed_ms, a, b);
    if (e != cudaSuccess) rc = fail_cuda(c, e);
  }
  if (rc == FDTD2D_OK) rc = fdtd2d_synchronize(c);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

void fdtd2d_clear_kernel_choices(void) {
  std::lock_guard<std::mutex> lock(g_choice_mu);
  g_choice.clear();
}

int fdtd2d_time_step_kernel(fdtd2d_ctx* c, int on) {
  if (!c) return FDTD2D_ERR_INVALID;
  if (c->batch) return FDTD2D_ERR_STATE;
  cudaSetDevice(c->device);
  cudaError_t e = prof_fold(c);
  c->prof = on != 0;
  c->prof_ms = 0;
  c->prof_n = 0;
  return e == cudaSuccess ? FDTD2D_OK : fail_cuda(c, e);
}

int fdtd2d_step_kernel_time(fdtd2d_ctx* c, double* ms, int64_t* launches, int64_t* cells, int32_t* steps) {
  if (!c || !ms || !launches || !cells || !steps) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaError_t e = prof_fold(c);
  if (e != cudaSuccess) return fail_cuda(c, e);
  *ms = c->prof_ms;
  *launches = c->prof_n;
  *cells = c->prof_cells;
  *steps = c->prof_steps;
  return FDTD2D_OK;
}

double fdtd2d_stability(const fdtd2d_setup* s) {
  if (!s || !(s->dx > 0) || !(s->dy > 0)) return -1;
  const double c0 = 2.99792458E8;
  const double eps = 1.0 / (c0 * c0 * 4.0 * 3.14159265358979 * 1.0E-7);
  double ne_max = 0;
  if (s->medium == FDTD2D_MEDIUM_UNIFORM) {
    if (s->ne)
      for (int64_t k = 0; k < (int64_t)s->nx * s->ny; ++k) ne_max = std::max(ne_max, (double)s->ne[k]);
  } else if (s->mat_ne) {
    for (int m = 0; m < s->n_materials; ++m) ne_max = std::max(ne_max, (double)s->mat_ne[m]);
  }
  const double wp2 = s->jz_coef * ne_max / eps;
  const double cdt = c0 * s->dt;
  return cdt * cdt * (1.0 / (s->dx * s->dx) + 1.0 / (s->dy * s->dy)) + wp2 * s->dt * s->dt / 4.0;
}

int fdtd2d_synchronize(fdtd2d_ctx* c) {
  if (!c) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  int err = 0;
  cudaError_t e = read_err(c, &err);
  if (e != cudaSuccess) return fail_cuda(c, e);
  return err == kErrWaitTimeout ? FDTD2D_ERR_TIMEOUT : (err ? FDTD2D_ERR_CUDA : FDTD2D_OK);
}

int fdtd2d_current_step(const fdtd2d_ctx* c, int32_t* n) {
  if (!c || !n) return FDTD2D_ERR_INVALID;
  *n = c->step;
  return FDTD2D_OK;
}

static int read_traces_body(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* det_ez, float* comp_ez, float* comp_hx,
                            float* comp_hy);

// The entry points below whose bodies allocate host buffers run them behind
// abi_guard: a failed allocation is FDTD2D_ERR_NOMEM, not an exception.
int fdtd2d_read_traces(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* det_ez, float* comp_ez,
                       float* comp_hx, float* comp_hy) {
  return abi_guard([&] { return read_traces_body(c, n0, n1, det_ez, comp_ez, comp_hx, comp_hy); });
}

static int read_traces_body(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* det_ez, float* comp_ez, float* comp_hx,
                            float* comp_hy) {
  if (!c) return FDTD2D_ERR_INVALID;
  if (!c->record) return FDTD2D_ERR_STATE;
  if (n0 < 1 || n1 < n0 || n1 > c->n_steps) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail_cuda(c, e);
  const size_t rows = (size_t)(n1 - n0 + 1);
  if (det_ez && c->n_det > 0) {
    e = cudaMemcpy(det_ez, c->h.trace + (size_t)(n0 - 1) * c->n_det, rows * c->n_det * 4,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail_cuda(c, e);
  }
  if ((comp_ez || comp_hx || comp_hy) && c->n_comp > 0) {
    std::vector<float> buf(rows * c->n_comp * 3);
    e = cudaMemcpy(buf.data(), c->h.ctrace + (size_t)(n0 - 1) * c->n_comp * 3, buf.size() * 4,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail_cuda(c, e);
    for (size_t r = 0; r < rows * c->n_comp; ++r) {
      if (comp_ez) comp_ez[r] = buf[r * 3 + 0];
      if (comp_hx) comp_hx[r] = buf[r * 3 + 1];
      if (comp_hy) comp_hy[r] = buf[r * 3 + 2];
    }
  }
  return FDTD2D_OK;
}

static int read_dft_body(fdtd2d_ctx* c, double* re, double* im);

int fdtd2d_read_dft(fdtd2d_ctx* c, double* re, double* im) {
  return abi_guard([&] { return read_dft_body(c, re, im); });
}

static int read_dft_body(fdtd2d_ctx* c, double* re, double* im) {
  if (!c || !re || !im) return FDTD2D_ERR_INVALID;
  if (!c->dft) return FDTD2D_ERR_STATE;
  cudaSetDevice(c->device);
  std::vector<double2> buf(c->n_det);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(buf.data(), c->h.dft, c->n_det * sizeof(double2), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(c, e);
  for (int k = 0; k < c->n_det; ++k) {
    re[k] = buf[k].x;
    im[k] = buf[k].y;
  }
  return FDTD2D_OK;
}

int fdtd2d_read_rc(fdtd2d_ctx* c, int32_t n0, int32_t n1, int32_t* spd) {
  if (!c || !spd) return FDTD2D_ERR_INVALID;
  if (c->n_rc <= 0) return FDTD2D_ERR_STATE;
  if (n0 < 1 || n1 < n0 || n1 > c->n_steps) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(spd, c->d_spd + (size_t)(n0 - 1) * c->n_rc, (size_t)(n1 - n0 + 1) * c->n_rc * 4,
                   cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(c, e);
  return FDTD2D_OK;
}

int fdtd2d_read_line(fdtd2d_ctx* c, int32_t n0, int32_t n1, float* out) {
  if (!c || !out) return FDTD2D_ERR_INVALID;
  if (c->line_n <= 0) return FDTD2D_ERR_STATE;
  if (n0 < c->line_first || n1 < n0 || n1 > c->line_last) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(out, c->d_line + (size_t)(n0 - c->line_first) * c->line_n,
                   (size_t)(n1 - n0 + 1) * c->line_n * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(c, e);
  return FDTD2D_OK;
}

namespace {

// Device pointer + geometry of a field in the reference layout.
struct FieldView {
  float* base;          // device
  int64_t dpitch;       // elements
  int rows, cols;       // reference layout
  int64_t hpitch;       // host row stride (elements)
};

bool field_view(fdtd2d_ctx* c, int which, int buf, FieldView* v) {
  const int nx = c->nx, ny = c->ny, P = c->npml;
  const int64_t pitch = c->pitch;
  const DevShot& h = c->h;
  switch (which) {
    case FDTD2D_FIELD_EZ: *v = {field_ptr(h, kEz, buf), pitch, ny, nx, nx}; return true;
    case FDTD2D_FIELD_JZ: *v = {field_ptr(h, kJz, buf), pitch, ny, nx, nx}; return true;
    case FDTD2D_FIELD_HX: *v = {field_ptr(h, kHx, buf), pitch, ny - 1, nx, nx}; return true;
    case FDTD2D_FIELD_HY: *v = {field_ptr(h, kHy, buf), pitch, ny, nx - 1, nx - 1}; return true;
    default: break;
  }
  float* ps = h.psi + buf * h.psi_buf;
  switch (which) {
    case FDTD2D_FIELD_PSI_EZX_1: *v = {ps + h.o_ezx, P, ny, P, P}; return true;
    case FDTD2D_FIELD_PSI_EZX_2: *v = {ps + h.o_ezx + (int64_t)ny * P, P, ny, P, P}; return true;
    case FDTD2D_FIELD_PSI_HYX_1: *v = {ps + h.o_hyx, P, ny, P - 1, P - 1}; return true;
    case FDTD2D_FIELD_PSI_HYX_2: *v = {ps + h.o_hyx + (int64_t)ny * P, P, ny, P - 1, P - 1}; return true;
    case FDTD2D_FIELD_PSI_EZY_1: *v = {ps + h.o_ezy, pitch, P, nx, nx}; return true;
    case FDTD2D_FIELD_PSI_EZY_2: *v = {ps + h.o_ezy + (int64_t)P * pitch, pitch, P, nx, nx}; return true;
    case FDTD2D_FIELD_PSI_HXY_1: *v = {ps, pitch, P - 1, nx, nx}; return true;
    case FDTD2D_FIELD_PSI_HXY_2: *v = {ps + (int64_t)(P - 1) * pitch, pitch, P - 1, nx, nx}; return true;
    default: return false;
  }
}

// The four physical fields in 16-bit storage: rows of the reference layout,
// converted with the array's scale on the host.
struct View16 {
  const uint16_t* base;  // device, column 0 of row 0 of buffer b
  int rows, cols;
  float sc, isc;
};

bool view16(fdtd2d_ctx* c, int which, int b, View16* v) {
  const DevShot& h = c->h;
  const int nx = c->nx, ny = c->ny;
  int f = -1, rows = ny, cols = nx;
  switch (which) {
    case FDTD2D_FIELD_EZ: f = kEz; break;
    case FDTD2D_FIELD_JZ: f = kJz; break;
    case FDTD2D_FIELD_HX: f = kHx; rows = ny - 1; break;
    case FDTD2D_FIELD_HY: f = kHy; cols = nx - 1; break;
    default: return false;
  }
  *v = {field_ptr_t<uint16_t>(h, f, b), rows, cols, h.sc[f], h.isc[f]};
  return true;
}

float from16(uint16_t u, int store) {
  if (store == FDTD2D_STORE_F16) {
    __half x;
    std::memcpy(&x, &u, 2);
    return __half2float(x);
  }
  __nv_bfloat16 x;
  std::memcpy(&x, &u, 2);
  return __bfloat162float(x);
}

uint16_t to16(float f, int store) {
  uint16_t u;
  if (store == FDTD2D_STORE_F16) {
    const __half x = __float2half_rn(f);
    std::memcpy(&u, &x, 2);
  } else {
    const __nv_bfloat16 x = __float2bfloat16_rn(f);
    std::memcpy(&u, &x, 2);
  }
  return u;
}

int read_field16(fdtd2d_ctx* c, int which, float* host) {
  View16 v;
  if (!view16(c, which, c->step & 1, &v)) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  std::vector<uint16_t> buf((size_t)v.rows * v.cols);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy2D(buf.data(), (size_t)v.cols * 2, v.base, (size_t)c->pitch * 2, (size_t)v.cols * 2, v.rows,
                     cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(c, e);
  for (size_t t = 0; t < buf.size(); ++t) host[t] = from16(buf[t], c->h.store) * v.sc;
  return FDTD2D_OK;
}

int write_field16(fdtd2d_ctx* c, int which, const float* host) {
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  for (int b = 0; b < 4 && e == cudaSuccess; ++b) {
    if (!c->h.fb[b]) continue;
    View16 v;
    if (!view16(c, which, b, &v)) return FDTD2D_ERR_INVALID;
    std::vector<uint16_t> buf((size_t)v.rows * v.cols);
    for (size_t t = 0; t < buf.size(); ++t) buf[t] = to16(host[t] * v.isc, c->h.store);
    // in the shot stream's order, finished before the host buffer goes away
    e = cudaMemcpy2DAsync(const_cast<uint16_t*>(v.base), (size_t)c->pitch * 2, buf.data(), (size_t)v.cols * 2,
                          (size_t)v.cols * 2, v.rows, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  if (e != cudaSuccess) return fail_cuda(c, e);
  return FDTD2D_OK;
}

}  // namespace

int fdtd2d_read_field(fdtd2d_ctx* c, int which, float* host) {
  if (!c || !host) return FDTD2D_ERR_INVALID;
  if (c->h.store != FDTD2D_STORE_F32 && which <= FDTD2D_FIELD_JZ)
    return abi_guard([&] { return read_field16(c, which, host); });
  FieldView v;
  if (!field_view(c, which, c->step & 1, &v)) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy2D(host, v.hpitch * 4, v.base, v.dpitch * 4, (size_t)v.cols * 4, v.rows,
                     cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(c, e);
  return FDTD2D_OK;
}

int fdtd2d_write_field(fdtd2d_ctx* c, int which, const float* host) {
  if (!c || !host) return FDTD2D_ERR_INVALID;
  if (c->h.store != FDTD2D_STORE_F32 && which <= FDTD2D_FIELD_JZ)
    return abi_guard([&] { return write_field16(c, which, host); });
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  for (int b = 0; b < 4 && e == cudaSuccess; ++b) {
    if (which <= FDTD2D_FIELD_JZ && !c->h.fb[b]) continue;
    if (which > FDTD2D_FIELD_JZ && b >= 2) break;   // psi: two buffers
    FieldView v;
    if (!field_view(c, which, b, &v)) return FDTD2D_ERR_INVALID;
    // In the shot stream's order: a plain cudaMemcpy2D from pageable memory
    // may return before its DMA has landed, and the shot's kernels run on a
    // non-blocking stream that would not wait for it.
    e = cudaMemcpy2DAsync(v.base, v.dpitch * 4, host, v.hpitch * 4, (size_t)v.cols * 4, v.rows,
                          cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  if (e != cudaSuccess) return fail_cuda(c, e);
  return FDTD2D_OK;
}

// ---- Snapshot and restore of a shot's state ----------------------------------
//
// Host image layout: a StateHeader, then the twelve field arrays of
// fdtd2d_read_field in FDTD2D_FIELD_* order (reference layouts, FP32 values;
// 16-bit storage round-trips exactly, every stored value being an FP32 value
// times a power of two), then the FP64 DFT sums (re, im per detector), the
// detector traces of every step ([n_steps][n_det] and [n_steps][n_comp][3]),
// the wave-front tracker's edge levels and rows ([n_rc], [n_steps][n_rc]) and
// the line-probe rows, each present when the setup has it.

namespace {

struct StateHeader {
  uint32_t magic, version;
  int32_t nx, ny, npml, n_steps, store, step;
  int32_t n_det, n_comp, record, dft, n_rc, line_n, line_first, line_last;
  int64_t bytes;
};
constexpr uint32_t kStateMagic = 0x31534446u;   // "FDS1"

int64_t field_count(const fdtd2d_ctx* c, int which) {
  const int64_t nx = c->nx, ny = c->ny, P = c->npml;
  switch (which) {
    case FDTD2D_FIELD_EZ: case FDTD2D_FIELD_JZ: return nx * ny;
    case FDTD2D_FIELD_HX: return (ny - 1) * nx;
    case FDTD2D_FIELD_HY: return ny * (nx - 1);
    case FDTD2D_FIELD_PSI_EZX_1: case FDTD2D_FIELD_PSI_EZX_2: return ny * P;
    case FDTD2D_FIELD_PSI_EZY_1: case FDTD2D_FIELD_PSI_EZY_2: return P * nx;
    case FDTD2D_FIELD_PSI_HYX_1: case FDTD2D_FIELD_PSI_HYX_2: return ny * (P - 1);
    default: return (P - 1) * nx;   // FDTD2D_FIELD_PSI_HXY_1/_2
  }
}

// The device arrays after the fields, as (device pointer, bytes) in image order.
std::vector<std::pair<void*, size_t>> state_blocks(fdtd2d_ctx* c) {
  std::vector<std::pair<void*, size_t>> b;
  if (c->dft) b.push_back({c->h.dft, (size_t)c->n_det * sizeof(double2)});
  if (c->record) {
    b.push_back({c->h.trace, (size_t)c->n_steps * c->n_det * sizeof(float)});
    b.push_back({c->h.ctrace, (size_t)c->n_steps * c->n_comp * 3 * sizeof(float)});
  }
  if (c->n_rc > 0) {
    b.push_back({c->d_edge, (size_t)c->n_rc * sizeof(float)});
    b.push_back({c->d_spd, (size_t)c->n_steps * c->n_rc * sizeof(int)});
  }
  if (c->line_n > 0)
    b.push_back({c->d_line, (size_t)(c->line_last - c->line_first + 1) * c->line_n * sizeof(float)});
  return b;
}

StateHeader state_header(fdtd2d_ctx* c) {
  StateHeader h{};
  h.magic = kStateMagic;
  h.version = 1;
  h.nx = c->nx; h.ny = c->ny; h.npml = c->npml; h.n_steps = c->n_steps; h.store = c->h.store;
  h.step = c->step;
  h.n_det = c->n_det; h.n_comp = c->n_comp; h.record = c->record; h.dft = c->dft ? 1 : 0;
  h.n_rc = c->n_rc; h.line_n = c->line_n; h.line_first = c->line_first; h.line_last = c->line_last;
  int64_t n = sizeof(StateHeader);
  for (int w = 0; w <= FDTD2D_FIELD_PSI_HXY_2; ++w) n += field_count(c, w) * 4;
  for (const auto& blk : state_blocks(c)) n += (int64_t)blk.second;
  h.bytes = n;
  return h;
}

// Every kernel of the shot, on both of its streams, has finished.
cudaError_t quiesce(fdtd2d_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess && c->side) e = cudaStreamSynchronize(c->side);
  return e;
}

int save_state_body(fdtd2d_ctx* c, void* buf, int64_t bytes) {
  if (!c || !buf) return FDTD2D_ERR_INVALID;
  const StateHeader h = state_header(c);
  if (bytes < h.bytes) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  cudaError_t e = quiesce(c);
  if (e != cudaSuccess) return fail_cuda(c, e);
  char* p = static_cast<char*>(buf);
  std::memcpy(p, &h, sizeof h);
  p += sizeof h;
  for (int w = 0; w <= FDTD2D_FIELD_PSI_HXY_2; ++w) {
    const int rc = fdtd2d_read_field(c, w, reinterpret_cast<float*>(p));
    if (rc) return rc;
    p += field_count(c, w) * 4;
  }
  for (const auto& blk : state_blocks(c)) {
    e = cudaMemcpyAsync(p, blk.first, blk.second, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cuda(c, e);
    p += blk.second;
  }
  return FDTD2D_OK;
}

int load_state_body(fdtd2d_ctx* c, const void* buf, int64_t bytes) {
  if (!c || !buf) return FDTD2D_ERR_INVALID;
  if (c->batch || c->solo) return FDTD2D_ERR_STATE;   // a batch member's step is the batch's
  const StateHeader want = state_header(c);
  StateHeader h;
  if (bytes < (int64_t)sizeof h) return FDTD2D_ERR_RANGE;
  std::memcpy(&h, buf, sizeof h);
  if (h.magic != kStateMagic || h.version != 1) return FDTD2D_ERR_INVALID;
  // the same shot geometry, storage, detectors and probes, a step it can be at
  if (h.nx != want.nx || h.ny != want.ny || h.npml != want.npml || h.n_steps != want.n_steps ||
      h.store != want.store || h.n_det != want.n_det || h.n_comp != want.n_comp || h.record != want.record ||
      h.dft != want.dft || h.n_rc != want.n_rc || h.line_n != want.line_n || h.line_first != want.line_first ||
      h.line_last != want.line_last || h.bytes != want.bytes || h.step < 0 || h.step > h.n_steps)
    return FDTD2D_ERR_INVALID;
  if (bytes < h.bytes) return FDTD2D_ERR_RANGE;
  cudaSetDevice(c->device);
  cudaError_t e = quiesce(c);
  if (e != cudaSuccess) return fail_cuda(c, e);
  // the fields go into every buffer of the shot (fdtd2d_write_field), so the
  // state is in place whatever slot the next step reads
  c->step = h.step;
  const char* p = static_cast<const char*>(buf) + sizeof h;
  for (int w = 0; w <= FDTD2D_FIELD_PSI_HXY_2; ++w) {
    const int rc = fdtd2d_write_field(c, w, reinterpret_cast<const float*>(p));
    if (rc) return rc;
    p += field_count(c, w) * 4;
  }
  for (const auto& blk : state_blocks(c)) {
    e = cudaMemcpyAsync(blk.first, p, blk.second, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cuda(c, e);
    p += blk.second;
  }
  return FDTD2D_OK;
}

}  // namespace

int64_t fdtd2d_state_bytes(fdtd2d_ctx* c) {
  if (!c) return FDTD2D_ERR_INVALID;
  return state_header(c).bytes;
}

int fdtd2d_save_state(fdtd2d_ctx* c, void* buf, int64_t bytes) {
  return abi_guard([&] { return save_state_body(c, buf, bytes); });
}

int fdtd2d_load_state(fdtd2d_ctx* c, const void* buf, int64_t bytes) {
  return abi_guard([&] { return load_state_body(c, buf, bytes); });
}

int fdtd2d_check_finite(fdtd2d_ctx* c) {
  if (!c) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  const int b = c->step & 1;
  const int64_t cells = c->h.cells;  // whole buffers, margins included (they stay 0)
  cudaError_t e = cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
    if (c->h.store == FDTD2D_STORE_F32)
      e = launch_nonfinite(field_ptr(c->h, k, b) - kMargin, cells, c->d_flag, c->stream);
    else
      e = launch_nonfinite16(field_ptr_t<uint16_t>(c->h, k, b) - kMargin, cells,
                             c->h.store == FDTD2D_STORE_BF16, c->d_flag, c->stream);
    ++c->launches;
  }
  int flag = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail_cuda(c, e);
  return flag ? FDTD2D_ERR_NONFINITE : FDTD2D_OK;
}

int fdtd2d_destroy(fdtd2d_ctx* c) {
  if (!c) return FDTD2D_ERR_INVALID;
  cudaSetDevice(c->device);
  // A batch member's memory is freed behind the batch's queued kernels (no
  // wait); a single shot waits for its stream and releases it.
  if (c->stream) {
    if (c->side) cudaStreamWaitEvent(c->stream, c->ev_e, 0);   // the side stream's last kernel
    for (void* p : c->allocs) cudaFreeAsync(p, c->stream);
  }
  if (c->stream && !c->batch) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  for (cudaEvent_t ev : {c->ev_t, c->ev_e, c->ev_m, c->ev_a})
    if (ev) cudaEventDestroy(ev);
  for (auto& pr : c->prof_pending) c->prof_pool.insert(c->prof_pool.end(), {pr.first, pr.second});
  for (cudaEvent_t ev : c->prof_pool) cudaEventDestroy(ev);
  delete c;
  return FDTD2D_OK;
}

int64_t fdtd2d_launch_count(const fdtd2d_ctx* c) { return c ? c->launches : -1; }

const char* fdtd2d_kernel_name(const fdtd2d_ctx* c) {
  if (!c) return "";
  return c->kernel_name;
}

int fdtd2d_last_cuda_error(const fdtd2d_ctx* c) { return c ? c->last_cuda : -1; }

int fdtd2d_kernel_choice_source(const fdtd2d_ctx* c) { return c ? c->choice_src : FDTD2D_ERR_INVALID; }

}  // extern "C"
