// Fused TMz step for the interior of a shot, staged R rows at a time with
// tensor copies (cp.async.bulk.tensor, TMA tiles).
//
// The one-row-per-stage kernel (step_tma.cu) spends most of its producer
// thread's row time inside its 5-7 cp.async.bulk instructions: each costs the
// issuing thread a few hundred cycles whatever its size.  Here one stage
// holds R rows of a band, fetched with one rank-3 tensor copy per box for
// Hx, Hy and Jz together (column x row x field), one rank-2 copy per box for
// Ez (rows j+1..j+R) and one for the plasma drive: 3 x boxes instructions
// per R rows instead of 5 per row.  The units it takes have no CPML work (the
// band and its Hy halo column lie outside the x strips, the rows inside
// [npml, ny - npml)), so the band loop has no CPML code and no per-column
// predicates; the CPML bands and rows run on step_tma.cu's kernel in the
// same time step.  The arithmetic is the same, operation for operation, as
// that kernel's, so either kernel gives a cell the same bits.
//
// Every wait is bounded as in step_tma.cu (1 s without progress: the error
// word is set, the copies in flight are waited for, the kernel returns).
#include "internal.h"
#include "step_common.cuh"
#include "tma_common.cuh"

namespace fdtd2d {

namespace {

// W warps (band of 128*W columns), R rows per stage, ST stages, storage T.
template <int W, int R, int ST, class T>
struct TCfg {
  using Elem = T;
  static constexpr int kWarps = W;
  static constexpr int kThreads = W * 32;
  static constexpr int kRows = R;
  static constexpr int kStages = ST;
  static constexpr int kBand = W * kCols;
  static constexpr int kHalo = 8;                        // elements staged on each side
  static constexpr int kSpan = kBand + 2 * kHalo;        // staged columns
  static constexpr int kBoxes = (kSpan + 255) / 256;     // tensor boxes across the span
  static constexpr int kBX = kSpan / kBoxes;             // columns per box
  static constexpr uint32_t pad128(uint32_t b) { return (b + 127) / 128 * 128; }
  static constexpr uint32_t kHJBytes = pad128(kBX * R * 3 * sizeof(T));   // [3 fields][R][kBX]
  static constexpr uint32_t kEBytes = pad128(kBX * R * sizeof(T));        // [R][kBX]
  static constexpr uint32_t kHJOff = 0;
  static constexpr uint32_t kEOff = kBoxes * kHJBytes;
  static constexpr uint32_t kKOff = kEOff + kBoxes * kEBytes;
  static constexpr uint32_t kStageBytes = kKOff + kBoxes * kEBytes;
  static constexpr size_t kSmem = (size_t)ST * kStageBytes;
  static constexpr int kMinBlocks = W <= 2 ? 6 : (W <= 4 ? 4 : 2);
  static_assert(kSpan % kBoxes == 0 && kBX % 8 == 0 && kBX <= 256, "box tiling of the staged span");
};

__device__ __forceinline__ void tensor3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tensor2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

struct TRing {
  unsigned char* stage;
  uint64_t* full;
  uint64_t* empty;
  uint32_t issued = 0;   // stages issued (producer thread)
  uint32_t used = 0;     // stages consumed (every thread)
};

// Producer: copy rows [jr, jr + R) of the band at c0 (Ez rows jr+1..jr+R)
// into the next stage.
template <class C>
__device__ bool issue_stage(TRing& R, const TensorMaps& M, int par, int c0, int jr, bool has_kp) {
  using T = typename C::Elem;
  const uint32_t g = R.issued++;
  const int s = g % C::kStages;
  if (g >= (uint32_t)C::kStages && !mbar_wait(&R.empty[s], ((g / C::kStages) - 1) & 1)) return false;
  unsigned char* dst = R.stage + s * C::kStageBytes;
  const uint32_t box = C::kBX * C::kRows * sizeof(T);
  mbar_expect_tx(&R.full[s], C::kBoxes * (box * 3 + box + (has_kp ? box : 0)));
#pragma unroll
  for (int b = 0; b < C::kBoxes; ++b) {
    const int x = c0 - C::kHalo + b * C::kBX;
    tensor3d(dst + C::kHJOff + b * C::kHJBytes, &M.hj[par], x, jr, 0, &R.full[s]);
    tensor2d(dst + C::kEOff + b * C::kEBytes, &M.e[par], x, jr + 1, &R.full[s]);
    if (has_kp) tensor2d(dst + C::kKOff + b * C::kEBytes, &M.k, x, jr, &R.full[s]);
  }
  return true;
}

template <class C>
__device__ void tdrain(TRing& R) {
  for (uint32_t g = R.used; g < R.issued; ++g) mbar_wait(&R.full[g % C::kStages], (g / C::kStages) & 1);
}

// Staged element (array a: 0 Hx, 1 Hy, 2 Jz in the HJ box; 3 Ez; 4 drive) at
// staged column xr (0 = c0 - kHalo) of stage row r.
template <class C>
__device__ __forceinline__ const typename C::Elem* at(const unsigned char* st, int a, int r, int xr) {
  using T = typename C::Elem;
  const int b = xr / C::kBX, cb = xr - b * C::kBX;
  if (a < 3)
    return reinterpret_cast<const T*>(st + C::kHJOff + b * C::kHJBytes) + (a * C::kRows + r) * C::kBX + cb;
  const uint32_t off = (a == 3 ? C::kEOff : C::kKOff) + b * C::kEBytes;
  return reinterpret_cast<const T*>(st + off) + r * C::kBX + cb;
}

template <class C>
__device__ void tband(const DevShot& S, const TensorMaps& M, TRing& R, int c0, int j0, int j1, int n, int* err) {
  using T = typename C::Elem;
  using St = Sto<T>;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t pitch = S.pitch;
  const int par = (n - 1) & 1;
  const bool has_kp = S.kp != nullptr;
  const T* __restrict__ ezo = field_ptr_t<T>(S, kEz, par);
  const T* __restrict__ hxo_p = field_ptr_t<T>(S, kHx, par);
  T* __restrict__ ezw = field_ptr_t<T>(S, kEz, par ^ 1);
  T* __restrict__ hxw = field_ptr_t<T>(S, kHx, par ^ 1);
  T* __restrict__ hyw = field_ptr_t<T>(S, kHy, par ^ 1);
  T* __restrict__ jzw = field_ptr_t<T>(S, kJz, par ^ 1);
  const float sE = S.sc[0], sHx = S.sc[1], sHy = S.sc[2], sJ = S.sc[3], sK = S.sc[4];

  const int i0 = c0 + warp * kCols;            // this warp's first column
  const int i = i0 + 4 * lane;                 // this lane's first column (all interior)
  const int xr = C::kHalo + warp * kCols + 4 * lane;   // its staged column
  const int xl = C::kHalo + warp * kCols - 1;          // Ez/Hy (i0 - 1)
  const int xe = C::kHalo + warp * kCols + kCols;      // Ez (i0 + 128)
  const int nst = (j1 - j0 + C::kRows - 1) / C::kRows;
  const bool producer = tid == 0;
  R.issued = R.used;

  if (producer) {
    for (int k = 0; k < nst && k < C::kStages; ++k)
      if (!issue_stage<C>(R, M, par, c0, j0 + k * C::kRows, has_kp)) {
        atomicExch(err, kErrWaitTimeout);
        tdrain<C>(R);
        return;
      }
  }

  MediumRow<0> m;
  m.init(S);
  float dex[4], dhx[4];
  ld4(dex, S.den_ex + i);
  ld4(dhx, S.den_hx + i);
  const float dhx_left = __ldg(S.den_hx + i0 - 1);

  // Row j0 state: Ez(j0), the warp-edge Ez values, and Hx_new(j0 - 1)
  // recomputed from the old buffers (row j0 - 1 >= npml - 1 has no CPML).
  float ezc[4], hxp[4];
  St::ldg4(ezc, ezo + (int64_t)j0 * pitch + i, sE);
  float ezl = lane == 0 ? St::ldg1(ezo + (int64_t)j0 * pitch + i0 - 1, sE) : 0.f;
  float ezr = lane == 31 ? St::ldg1(ezo + (int64_t)j0 * pitch + i0 + kCols, sE) : 0.f;
  {
    float ezp[4], hxo[4];
    St::ldg4(ezp, ezo + (int64_t)(j0 - 1) * pitch + i, sE);
    St::ldg4(hxo, hxo_p + (int64_t)(j0 - 1) * pitch + i, sHx);
    hx_row<0>(S, m, par, i, j0 - 1, ezp, ezc, hxo, hxp, false);
  }

  float dhy = __ldg(S.den_hy + j0), dey = __ldg(S.den_ey + j0);
  int p0 = __ldg(S.row_start + j0), p1 = __ldg(S.row_start + j0 + 1);

  for (int k = 0; k < nst; ++k) {
    const uint32_t g = R.used;
    const int s = g % C::kStages;
    if (!mbar_wait(&R.full[s], (g / C::kStages) & 1)) {
      atomicExch(err, kErrWaitTimeout);
      if (producer) tdrain<C>(R);
      return;
    }
    const unsigned char* st = R.stage + s * C::kStageBytes;
    const int jr = j0 + k * C::kRows;
    const int rows_here = min(C::kRows, j1 - jr);
    for (int r = 0; r < rows_here; ++r) {
      const int j = jr + r;
      const int jn = j + 1 < j1 ? j + 1 : j;
      const float dhy_n = __ldg(S.den_hy + jn), dey_n = __ldg(S.den_ey + jn);
      const int p1_n = __ldg(S.row_start + jn + 1);

      float ezn[4], hxo[4], hyo[4], jzo[4];
      St::lds4(ezn, at<C>(st, 3, r, xr), sE);
      St::lds4(hxo, at<C>(st, 0, r, xr), sHx);
      St::lds4(hyo, at<C>(st, 1, r, xr), sHy);
      St::lds4(jzo, at<C>(st, 2, r, xr), sJ);
      if (has_kp) {
        St::lds4(m.kp, at<C>(st, 4, r, xr), sK);
      } else {
        zero4(m.kp);
      }
      const float ezl_next = St::ld1(at<C>(st, 3, r, xl), sE);
      const float ezr_next = St::ld1(at<C>(st, 3, r, xe), sE);
      const float hyo_left = St::ld1(at<C>(st, 1, r, xl), sHy);

      // ---- H update (no CPML in these units)
      float hxn[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) hxn[q] = upd_h(S.da, hxo[q], S.db, ezc[q], ezn[q], dhy);
      float ezr_k = __shfl_down_sync(0xffffffffu, ezc[0], 1);
      if (lane == 31) ezr_k = ezr;
      const float ezr4[4] = {ezc[1], ezc[2], ezc[3], ezr_k};
      float hyn[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) hyn[q] = upd_h(m.day(q), hyo[q], m.dby(q), ezr4[q], ezc[q], dhx[q]);
      float hyl = __shfl_up_sync(0xffffffffu, hyn[3], 1);
      if (lane == 0) hyl = upd_h(S.da, hyo_left, S.db, ezc[0], ezl, dhx_left);

      // ---- Jz, Ez
      const float hyl4[4] = {hyl, hyn[0], hyn[1], hyn[2]};
      float ezw4[4], jzw4[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        jzw4[q] = upd_j(S.ja, jzo[q], m.kp[q], ezc[q]);
        ezw4[q] = upd_e(S.ca, ezc[q], S.cb, __fsub_rn(hyn[q], hyl4[q]), dex[q], __fsub_rn(hxp[q], hxn[q]), dey,
                        jzw4[q]);
      }

      // ---- sources, then detectors, of this row
      for (int p = p0; p < p1; ++p) {
        const int4 pt = __ldg(S.pts + p);
        const int kk = pt.x - i;
        if (kk < 0 || kk > 3) continue;
        float e = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) if (q == kk) e = ezw4[q];
        if (pt.y == kPointSource) {
          e = __fsub_rn(e, __ldg(S.src_val + (int64_t)n * S.n_src + pt.z));
#pragma unroll
          for (int q = 0; q < 4; ++q) if (q == kk) ezw4[q] = e;
        } else if (pt.y == kPointDetEz) {
          if (S.record) S.trace[(int64_t)(n - 1) * S.n_det + pt.z] = e;
          if (S.dft) {
            const double2 tw = __ldg(S.twiddle + n);
            double2 acc = S.dft[pt.z];
            acc.x = fma((double)e, tw.x, acc.x);
            acc.y = fma(-(double)e, tw.y, acc.y);
            S.dft[pt.z] = acc;
          }
        } else {
          float hxv = 0.f, hyv = 0.f;
#pragma unroll
          for (int q = 0; q < 4; ++q) if (q == kk) { hxv = hxn[q]; hyv = hyn[q]; }
          if (S.record) {
            float* dst = S.ctrace + ((int64_t)(n - 1) * S.n_comp + pt.z) * 3;
            dst[0] = e; dst[1] = hxv; dst[2] = hyv;
          }
        }
      }

      const int64_t o = (int64_t)j * pitch + i;
      St::stcs4(hxw + o, hxn, S.isc[1]);
      St::stcs4(hyw + o, hyn, S.isc[2]);
      St::stcs4(ezw + o, ezw4, S.isc[0]);
      St::stcs4(jzw + o, jzw4, S.isc[3]);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        hxp[q] = hxn[q];
        ezc[q] = ezn[q];
      }
      ezl = ezl_next;
      ezr = ezr_next;
      dhy = dhy_n;
      dey = dey_n;
      p0 = p1;
      p1 = p1_n;
    }
    // every read of this stage is done: release it, then refill it
    __syncwarp();
    if (lane == 0) mbar_arrive(&R.empty[s]);
    R.used++;
    if (producer && k + C::kStages < nst) {
      if (!issue_stage<C>(R, M, par, c0, j0 + (k + C::kStages) * C::kRows, has_kp)) {
        atomicExch(err, kErrWaitTimeout);
        tdrain<C>(R);
        return;
      }
    }
  }
}

template <class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks)
step_tmat_kernel(const __grid_constant__ DevShot S, const __grid_constant__ TensorMaps M,
                 const int4* __restrict__ units, int n_units, int n_global, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[C::kStages], empty[C::kStages];
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  TRing R;
  R.stage = smem;
  R.full = full;
  R.empty = empty;
  const int n = n_global - S.base_n;
  if (n < 1 || n > S.n_steps) return;
  for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
    const int4 ud = __ldg(units + u);
    tband<C>(S, M, R, ud.y, ud.z, ud.w, n, err);
    if (*(volatile int*)err) return;
  }
}

using TKernelFn = void (*)(DevShot, TensorMaps, const int4*, int, int, int*);

struct TShape {
  int warps, rows, stages;
  TKernelFn fn[3];
  size_t smem[3];
  int bx;
};

template <int W, int R, int ST>
constexpr TShape tentry() {
  using C32 = TCfg<W, R, ST, float>;
  using C16 = TCfg<W, R, ST, __half>;
  using CB16 = TCfg<W, R, ST, __nv_bfloat16>;
  return {W, R, ST, {step_tmat_kernel<C32>, step_tmat_kernel<C16>, step_tmat_kernel<CB16>},
          {C32::kSmem, C16::kSmem, CB16::kSmem}, C32::kBX};
}

// Compiled shapes (warps, rows per stage, stages); the first is the default.
const TShape kTShapes[] = {tentry<4, 4, 2>(), tentry<4, 2, 3>(), tentry<4, 4, 3>(), tentry<2, 8, 2>(),
                           tentry<4, 8, 2>(), tentry<8, 2, 2>()};
constexpr int kNumTShapes = sizeof(kTShapes) / sizeof(kTShapes[0]);

}  // namespace

int tmat_shape_count() { return kNumTShapes; }

void tmat_shape_dims(int shape, int* warps, int* rows, int* stages) {
  *warps = kTShapes[shape].warps;
  *rows = kTShapes[shape].rows;
  *stages = kTShapes[shape].stages;
}

int tmat_band_cols(int shape) { return kTShapes[shape].warps * kCols; }

int tmat_box_cols(int shape) { return kTShapes[shape].bx; }

int tmat_rows(int shape) { return kTShapes[shape].rows; }

cudaError_t launch_step_tmat(int shape, const DevShot& shot, const TensorMaps& maps, const int4* units,
                             int n_units, int n_global, int max_ctas, int* err, cudaStream_t stream) {
  const TShape& e = kTShapes[shape];
  const int ctas = max_ctas < n_units ? max_ctas : n_units;
  if (ctas <= 0) return cudaSuccess;
  const int st = shot.store;
  e.fn[st]<<<ctas, e.warps * 32, e.smem[st], stream>>>(shot, maps, units, n_units, n_global, err);
  return cudaGetLastError();
}

int tmat_resident_ctas(int shape, int store, int device) {
  const TShape& e = kTShapes[shape];
  cudaFuncSetAttribute(e.fn[store], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem[store]);
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e.fn[store], e.warps * 32, e.smem[store]);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fdtd2d
