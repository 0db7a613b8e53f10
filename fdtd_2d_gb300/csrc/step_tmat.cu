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
// step_tmat2_kernel is the two-step form: one pass over state n-1 gives
// state n+1 of the interior (each warp recomputes step n one column beyond
// its sides, each unit one row beyond its ends), so the fields are read and
// written once for two time steps; frame_kernel steps the 2-cell frame the
// next pass reads beyond the interior.
//
// Every wait is bounded as in step_tma.cu (1 s without progress: the error
// word is set, the copies in flight are waited for, the kernel returns).
#include <algorithm>

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
  // two-step form: more registers; 4 CTAs (128 registers, no spills in
  // F32) where shared memory lets four fit, 3 otherwise (16-bit storage:
  // its conversions spill at 128)
  static constexpr int kMinBlocks2 =
      W <= 2 ? 5 : (W <= 4 ? ((sizeof(T) == 4 && kSmem <= 56 * 1024) ? 4 : 3) : 1);
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
__device__ void tband(const DevShot& S, const TensorMaps& M, TRing& R, int c0, int j0, int j1, int idle, int n,
                      int* err) {
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

  // The first `idle` warps lie left of the region (a two-step unit list
  // stepped once): they only follow the stages, and their few preamble
  // loads address the first working warp's columns.
  const bool act = warp >= idle;
  const int wl = act ? warp : idle;
  const int i0 = c0 + wl * kCols;              // this warp's first column
  const int i = i0 + 4 * lane;                 // this lane's first column (all interior)
  const int xr = C::kHalo + wl * kCols + 4 * lane;     // its staged column
  const int xl = C::kHalo + wl * kCols - 1;            // Ez/Hy (i0 - 1)
  const int xe = C::kHalo + wl * kCols + kCols;        // Ez (i0 + 128)
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
    const int rows_here = act ? min(C::kRows, j1 - jr) : 0;
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

// Sources of step n, then its detectors when `rec`, on the cells i..i+3 of
// one row (the point loop of tband), plus the sources at column xc, which
// are applied to ezx: the edge column a two-step unit recomputes.  The
// fields are in stored units (Ez/sE, H/sH): a source sample enters as
// sample/sE, a detector records the field times its scale, both exact
// (kScaled false: FP32 storage, unit scales).
template <bool kScaled>
__device__ __forceinline__ float upd_e2(float ca, float e, float cb, float dhy, float dex, float dhx, float dey,
                                        float jz, float rj) {
  if constexpr (kScaled) return upd_es(ca, e, cb, dhy, dex, dhx, dey, jz, rj);
  else return upd_e(ca, e, cb, dhy, dex, dhx, dey, jz);
}

template <bool kScaled>
__device__ __forceinline__ void pts2(const DevShot& S, int p0, int p1, int i, int n, bool rec, float (&ez)[4],
                                     const float (&hx)[4], const float (&hy)[4], int xc, float& ezx) {
  // value of a source sample in stored units, of a stored field in FP32 units
  auto src = [&](int z, int m) {
    const float v = __ldg(S.src_val + (int64_t)m * S.n_src + z);
    return kScaled ? __fmul_rn(v, S.isc[0]) : v;
  };
  auto unit = [&](float v, int f) { return kScaled ? __fmul_rn(v, S.sc[f]) : v; };
  for (int p = p0; p < p1; ++p) {
    const int4 pt = __ldg(S.pts + p);
    if (pt.y == kPointSource && pt.x == xc)
      ezx = __fsub_rn(ezx, src(pt.z, n));
    const int kk = pt.x - i;
    if (kk < 0 || kk > 3) continue;
    float e = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) if (q == kk) e = ez[q];
    if (pt.y == kPointSource) {
      e = __fsub_rn(e, src(pt.z, n));
#pragma unroll
      for (int q = 0; q < 4; ++q) if (q == kk) ez[q] = e;
    } else if (!rec) {
      continue;
    } else if (pt.y == kPointDetEz) {
      e = unit(e, 0);
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
      for (int q = 0; q < 4; ++q) if (q == kk) { hxv = hx[q]; hyv = hy[q]; }
      if (S.record) {
        float* dst = S.ctrace + ((int64_t)(n - 1) * S.n_comp + pt.z) * 3;
        dst[0] = unit(e, 0); dst[1] = unit(hxv, 1); dst[2] = unit(hyv, 2);
      }
    }
  }
}

// Two time steps of one unit (flags, c0, j0, j1) in one pass over state n-1
// (slot 0).  Step n runs over rows j0-1 .. j1 and, per warp, one column
// beyond each side of its 128 (lane 0 the left one, lane 31 the right one),
// so that step n+1 over the warp's cells [i0, i0+128) x [j0, j1) needs
// nothing from other warps or units; step n+1 of row j-1 follows step n of
// row j.  Step-n values reach step n+1 as a store and reload would give
// them (Sto::rt*), and every update is the one-step kernel's, operation for
// operation, so the two steps give the bits of two one-step launches.
// State n+1 goes to slot 2, and state n of R's edge rows and columns, which
// the CPML-band kernel's step n+1 reads, to slot 1: with FP32 storage from
// here (ring flags), with 16-bit storage from the ring units (ring_unit),
// because stores of it in the unrolled 16-bit row loop, even when seldom
// taken, slowed that form 13 %.
template <class C>
__device__ void tband2(const DevShot& S, const TensorMaps& M, TRing& R, const int4 ud, int n, int* err) {
  using T = typename C::Elem;
  using St = Sto<T>;
  const int c0 = ud.y, j0 = ud.z, j1 = ud.w;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t pitch = S.pitch;
  const bool has_kp = S.kp != nullptr;
  const T* __restrict__ ezo = field_ptr_t<T>(S, kEz, 0);
  const T* __restrict__ hxo_p = field_ptr_t<T>(S, kHx, 0);
  T* __restrict__ ezm = field_ptr_t<T>(S, kEz, 1);
  T* __restrict__ hxm = field_ptr_t<T>(S, kHx, 1);
  T* __restrict__ hym = field_ptr_t<T>(S, kHy, 1);
  T* __restrict__ jzm = field_ptr_t<T>(S, kJz, 1);
  T* __restrict__ ezw = field_ptr_t<T>(S, kEz, 2);
  T* __restrict__ hxw = field_ptr_t<T>(S, kHx, 2);
  T* __restrict__ hyw = field_ptr_t<T>(S, kHy, 2);
  T* __restrict__ jzw = field_ptr_t<T>(S, kJz, 2);
  // Arithmetic in stored units (Ez/sE, Hx/sH, Hy/sH, Jz/sJ): loads and
  // stores convert without a scale, and the power-of-two scales are folded
  // into db, cb, the drive map and the Jz term of the curl (upd_es), so
  // every stored value keeps the bits of the FP32-unit update.  Hx and Hy
  // share one scale (checked at launch).  FP32 storage has unit scales.
  constexpr bool kScaled = sizeof(T) == 2;
  const float sE = kScaled ? S.sc[0] : 1.f, sH = kScaled ? S.sc[1] : 1.f, iH = kScaled ? S.isc[1] : 1.f;
  const float da = S.da, ca = S.ca, ja = S.ja;
  const float db = kScaled ? __fmul_rn(__fmul_rn(S.db, sE), iH) : S.db;           // db sE/sH
  const float cb = kScaled ? __fmul_rn(__fmul_rn(S.cb, sH), S.isc[0]) : S.cb;      // cb sH/sE
  const float rj = kScaled ? __fmul_rn(S.sc[3], iH) : 1.f;                         // sJ/sH
  const float rk = kScaled ? __fmul_rn(__fmul_rn(S.sc[4], sE), S.isc[3]) : 1.f;    // sK sE/sJ

  // The first `idle` warps of a unit (bits 4-6 of its flags) lie left of
  // R: a region that is not a whole number of units wide starts with a unit
  // whose leading columns belong to the CPML-band kernel.  Those warps only
  // follow the stages (barrier waits and arrivals); their few preamble
  // loads read the first working warp's columns, which are in bounds.
  const int idle = (ud.x >> 4) & 7;
  const bool act = warp >= idle;
  const int wl = act ? warp : idle;            // the warp whose columns this one addresses
  const int i0 = c0 + wl * kCols;              // this warp's first column
  const int i = i0 + 4 * lane;                 // this lane's first column
  const int xr = C::kHalo + wl * kCols + 4 * lane;     // its staged column
  // the warp's edge column: lane 0 the one left of the warp, the other lanes
  // (for use: lane 31) the one right of it
  const int xc = lane == 0 ? i0 - 1 : i0 + kCols;
  const int sx = C::kHalo + (xc - c0);         // its staged column
  const int jb = j0 - 1;                       // first step-n row
  const int rows_n = j1 - j0 + 2;              // step-n rows jb .. j1
  const int nst = (rows_n + C::kRows - 1) / C::kRows;
  const bool producer = tid == 0;
  R.issued = R.used;

  if (producer) {
    for (int k = 0; k < nst && k < C::kStages; ++k)
      if (!issue_stage<C>(R, M, 0, c0, jb + k * C::kRows, has_kp)) {
        atomicExch(err, kErrWaitTimeout);
        tdrain<C>(R);
        return;
      }
  }

  // Every cell the unit steps, edge columns and their neighbours included,
  // lies in the CPML-free part of the grid, where each denominator table
  // holds one value (den_c; checked at create): the same floats as the
  // tables' entries there.
  const float dex = S.den_c[0], dhx = S.den_c[1], dey = S.den_c[2], dhy = S.den_c[3];

  // Row jb state: Ez_{n-1}(jb) here and at the edge column and its
  // neighbours, Hx_n(jb - 1) recomputed (row jb - 1 >= npml - 1: no CPML).
  float ezc[4], hxp[4];
  St::ldg4(ezc, ezo + (int64_t)jb * pitch + i);
  float e_m = St::ldg1(ezo + (int64_t)jb * pitch + xc - 1);
  float e_0 = St::ldg1(ezo + (int64_t)jb * pitch + xc);
  float e_p = St::ldg1(ezo + (int64_t)jb * pitch + xc + 1);
  float hxe_p;                                 // Hx_n(xc, j - 1)
  {
    float ezp[4], hxo[4];
    const int64_t o = (int64_t)(jb - 1) * pitch;
    St::ldg4(ezp, ezo + o + i);
    St::ldg4(hxo, hxo_p + o + i);
#pragma unroll
    for (int q = 0; q < 4; ++q) hxp[q] = upd_h(da, hxo[q], db, ezp[q], ezc[q], dhy);
    hxe_p = upd_h(da, St::ldg1(hxo_p + o + xc), db, St::ldg1(ezo + o + xc), e_0, dhy);
  }

  // state n of the previous row as stored, for step n+1
  float ez1[4], hx1[4], hy1[4], jz1[4], kp1[4], hx2p[4];
  float eze1 = 0.f, hye1 = 0.f;                // Ez_n(xc, j-1), Hy_n(xc, j-1) as stored
#pragma unroll
  for (int q = 0; q < 4; ++q) ez1[q] = hx1[q] = hy1[q] = jz1[q] = kp1[q] = hx2p[q] = 0.f;
  int q0 = 0, q1 = 0;
  int p0 = __ldg(S.row_start + jb), p1 = __ldg(S.row_start + jb + 1);

  for (int k = 0; k < nst; ++k) {
    const uint32_t g = R.used;
    const int s = g % C::kStages;
    if (!mbar_wait(&R.full[s], (g / C::kStages) & 1)) {
      atomicExch(err, kErrWaitTimeout);
      if (producer) tdrain<C>(R);
      return;
    }
    const unsigned char* st = R.stage + s * C::kStageBytes;
    const int jr = jb + k * C::kRows;
    const int rows_here = act ? min(C::kRows, jb + rows_n - jr) : 0;
    // The row body, inlined.  With 16-bit storage a full stage's rows are
    // unrolled, so the row state handed from one row to the next is renamed
    // instead of moved and the staged offsets of each row are constants:
    // 15 % fewer instructions per launch, and the issue-bound 16-bit kernel
    // runs 3 % faster (8192^2, GB300).  The FP32 kernel, bound by DRAM,
    // measured 1 % slower unrolled and keeps the loop.
    auto row = [&](const int r) {
      const int j = jr + r;
      const int jn = j + 1 <= j1 ? j + 1 : j;
      const int p1_n = __ldg(S.row_start + jn + 1);

      // ---- staged state n-1: row j (Ez row j+1)
      float ezn[4], hxo[4], hyo[4], jzo[4], kp[4];
      St::lds4(ezn, at<C>(st, 3, r, xr));
      St::lds4(hxo, at<C>(st, 0, r, xr));
      St::lds4(hyo, at<C>(st, 1, r, xr));
      St::lds4(jzo, at<C>(st, 2, r, xr));
      if (has_kp) {
        St::lds4(kp, at<C>(st, 4, r, xr), rk);
      } else {
        zero4(kp);
      }
      const float f_m = St::ld1(at<C>(st, 3, r, sx - 1));
      const float f_0 = St::ld1(at<C>(st, 3, r, sx));
      const float f_p = St::ld1(at<C>(st, 3, r, sx + 1));
      const float hyoA = St::ld1(at<C>(st, 1, r, sx - 1));
      const float hyoB = St::ld1(at<C>(st, 1, r, sx));
      const float hxoE = St::ld1(at<C>(st, 0, r, sx));
      const float jzoE = St::ld1(at<C>(st, 2, r, sx));
      const float kpE = !has_kp ? 0.f : kScaled ? __fmul_rn(St::ld1(at<C>(st, 4, r, sx)), rk) : St::ld1(at<C>(st, 4, r, sx));

      // ---- step n, row j
      float hxn[4], hyn[4], jzn[4], ezs_n[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) hxn[q] = upd_h(da, hxo[q], db, ezc[q], ezn[q], dhy);
      float ezr_k = __shfl_down_sync(0xffffffffu, ezc[0], 1);
      if (lane == 31) ezr_k = e_0;
      const float ezr4[4] = {ezc[1], ezc[2], ezc[3], ezr_k};
#pragma unroll
      for (int q = 0; q < 4; ++q) hyn[q] = upd_h(da, hyo[q], db, ezr4[q], ezc[q], dhx);
      // edge column: Hy at xc-1 and xc, then Hx, Jz, Ez at xc
      const float hyA = upd_h(da, hyoA, db, e_0, e_m, dhx);
      const float hyB = upd_h(da, hyoB, db, e_p, e_0, dhx);
      float hyl = __shfl_up_sync(0xffffffffu, hyn[3], 1);
      if (lane == 0) hyl = hyB;
      const float hxE = upd_h(da, hxoE, db, e_0, f_0, dhy);
      const float jzE = upd_j(ja, jzoE, kpE, e_0);
      float ezE = upd_e2<kScaled>(ca, e_0, cb, __fsub_rn(hyB, hyA), dex, __fsub_rn(hxe_p, hxE), dey, jzE, rj);
      const float hyl4[4] = {hyl, hyn[0], hyn[1], hyn[2]};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        jzn[q] = upd_j(ja, jzo[q], kp[q], ezc[q]);
        ezs_n[q] = upd_e2<kScaled>(ca, ezc[q], cb, __fsub_rn(hyn[q], hyl4[q]), dex, __fsub_rn(hxp[q], hxn[q]), dey, jzn[q], rj);
      }
      const bool own = j >= j0 && j < j1;
      pts2<kScaled>(S, p0, p1, i, n, own, ezs_n, hxn, hyn, xc, ezE);
      if constexpr (!kScaled) {
        // FP32: state n of R's edge rows and columns (flags kRing*) to slot
        // 1 from here; the 16-bit forms take it from the ring units
        if (own) {
          const int64_t o = (int64_t)j * pitch + i;
          if (((ud.x & kRingTop) && j == j0) || ((ud.x & kRingBottom) && j == j1 - 1)) {
            St::stcs4(ezm + o, ezs_n);
            St::stcs4(hxm + o, hxn);
            St::stcs4(hym + o, hyn);
            St::stcs4(jzm + o, jzn);
          } else if ((ud.x & kRingLeft) && warp == idle && lane == 0) {
            St::st1(ezm + o, ezs_n[0]);
            St::st1(hxm + o, hxn[0]);
            St::st1(hym + o, hyn[0]);
            St::st1(jzm + o, jzn[0]);
          } else if ((ud.x & kRingRight) && warp == C::kWarps - 1 && lane == 31) {
            St::st1(ezm + o + 3, ezs_n[3]);
            St::st1(hxm + o + 3, hxn[3]);
            St::st1(hym + o + 3, hyn[3]);
            St::st1(jzm + o + 3, jzn[3]);
          }
        }
      }

      // ---- step n+1, row j-1 (row jb: its Hx only)
      float ezs[4], hxs[4], hys[4], jzs[4];       // state n of row j as stored
      St::rt4(ezs, ezs_n);
      St::rt4(hxs, hxn);
      St::rt4(hys, hyn);
      St::rt4(jzs, jzn);
      if (j > jb) {
        float hx2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) hx2[q] = upd_h(da, hx1[q], db, ez1[q], ezs[q], dhy);
        if (j > j0) {
          float rk = __shfl_down_sync(0xffffffffu, ez1[0], 1);
          if (lane == 31) rk = eze1;
          const float er4[4] = {ez1[1], ez1[2], ez1[3], rk};
          float hy2[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) hy2[q] = upd_h(da, hy1[q], db, er4[q], ez1[q], dhx);
          float hl = __shfl_up_sync(0xffffffffu, hy2[3], 1);
          if (lane == 0) hl = upd_h(da, hye1, db, ez1[0], eze1, dhx);
          const float hl4[4] = {hl, hy2[0], hy2[1], hy2[2]};
          float ez2[4], jz2[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            jz2[q] = upd_j(ja, jz1[q], kp1[q], ez1[q]);
            ez2[q] = upd_e2<kScaled>(ca, ez1[q], cb, __fsub_rn(hy2[q], hl4[q]), dex, __fsub_rn(hx2p[q], hx2[q]), dey,
                            jz2[q], rj);
          }
          float unused = 0.f;
          pts2<kScaled>(S, q0, q1, i, n + 1, true, ez2, hx2, hy2, -1, unused);
          const int64_t o = (int64_t)(j - 1) * pitch + i;
          St::stcs4(hxw + o, hx2);
          St::stcs4(hyw + o, hy2);
          St::stcs4(ezw + o, ez2);
          St::stcs4(jzw + o, jz2);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) hx2p[q] = hx2[q];
      }

#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ez1[q] = ezs[q];
        hx1[q] = hxs[q];
        hy1[q] = hys[q];
        jz1[q] = jzs[q];
        kp1[q] = kp[q];
        hxp[q] = hxn[q];
        ezc[q] = ezn[q];
      }
      eze1 = St::rt1(ezE);
      hye1 = St::rt1(hyB);
      hxe_p = hxE;
      e_m = f_m;
      e_0 = f_0;
      e_p = f_p;
      q0 = p0;
      q1 = p1;
      p0 = p1;
      p1 = p1_n;
    };
    if constexpr (kScaled) {
      if (rows_here == C::kRows) {
#pragma unroll
        for (int r = 0; r < C::kRows; ++r) row(r);
      } else {
        for (int r = 0; r < rows_here; ++r) row(r);
      }
    } else {
#pragma unroll 1
      for (int r = 0; r < rows_here; ++r) row(r);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&R.empty[s]);
    R.used++;
    if (producer && k + C::kStages < nst) {
      if (!issue_stage<C>(R, M, 0, c0, jb + (k + C::kStages) * C::kRows, has_kp)) {
        atomicExch(err, kErrWaitTimeout);
        tdrain<C>(R);
        return;
      }
    }
  }
}

// One cell (i, j) of step n outside the CPML: the one-step kernels' updates
// of Hx, Hy (and the Hx, Hy the Ez update takes from the cells above and to
// the left), Jz and Ez, operation for operation, from state n-1 in slot rd
// into slot wr, sources applied.
template <class T>
__device__ __forceinline__ void frame_cell(const DevShot& S, int i, int j, int n, int rd, int wr) {
  using St = Sto<T>;
  const int64_t p = S.pitch, o = (int64_t)j * p + i;
  const float sE = S.sc[0], sHx = S.sc[1], sHy = S.sc[2], sJ = S.sc[3], sK = S.sc[4];
  const T* ez = field_ptr_t<T>(S, kEz, rd);
  const T* hx = field_ptr_t<T>(S, kHx, rd);
  const T* hy = field_ptr_t<T>(S, kHy, rd);
  const T* jz = field_ptr_t<T>(S, kJz, rd);
  const float e_c = St::ldg1(ez + o, sE), e_r = St::ldg1(ez + o + 1, sE), e_l = St::ldg1(ez + o - 1, sE);
  const float e_d = St::ldg1(ez + o + p, sE), e_u = St::ldg1(ez + o - p, sE);
  const float da = S.da, db = S.db;
  const float hx_c = upd_h(da, St::ldg1(hx + o, sHx), db, e_c, e_d, __ldg(S.den_hy + j));
  const float hx_u = upd_h(da, St::ldg1(hx + o - p, sHx), db, e_u, e_c, __ldg(S.den_hy + j - 1));
  const float hy_c = upd_h(da, St::ldg1(hy + o, sHy), db, e_r, e_c, __ldg(S.den_hx + i));
  const float hy_l = upd_h(da, St::ldg1(hy + o - 1, sHy), db, e_c, e_l, __ldg(S.den_hx + i - 1));
  const float kp = S.kp ? St::ldg1(reinterpret_cast<const T*>(S.kp) + o, sK) : 0.f;
  const float jz_n = upd_j(S.ja, St::ldg1(jz + o, sJ), kp, e_c);
  float e = upd_e(S.ca, e_c, S.cb, __fsub_rn(hy_c, hy_l), __ldg(S.den_ex + i), __fsub_rn(hx_u, hx_c),
                  __ldg(S.den_ey + j), jz_n);
  for (int q = __ldg(S.row_start + j), q1 = __ldg(S.row_start + j + 1); q < q1; ++q) {
    const int4 pt = __ldg(S.pts + q);
    if (pt.y == kPointSource && pt.x == i) e = __fsub_rn(e, __ldg(S.src_val + (int64_t)n * S.n_src + pt.z));
  }
  St::st1(field_ptr_t<T>(S, kEz, wr) + o, e, S.isc[0]);
  St::st1(field_ptr_t<T>(S, kHx, wr) + o, hx_c, S.isc[1]);
  St::st1(field_ptr_t<T>(S, kHy, wr) + o, hy_c, S.isc[2]);
  St::st1(field_ptr_t<T>(S, kJz, wr) + o, jz_n, S.isc[3]);
}

// A ring unit of the two-step kernel (kUnitRing, t0, t1, 0; 16-bit
// storage): step n of R's edge cells t0 .. t1-1 (rows ri0 and ri1-1 over
// columns [ci0, ci1), then columns ci0 and ci1-1 over the rows between; rg =
// (ci0, ci1, ri0, ri1)) from slot 0 into slot 1, where the CPML-band
// kernel's step n+1 and the frame kernel read them.
template <class T>
__device__ void ring_unit(const DevShot& S, const int4 rg, const int4 ud, int n, int nthreads) {
  const int w = rg.y - rg.x, h = rg.w - rg.z - 2;
  for (int t = ud.y + (int)threadIdx.x; t < ud.z; t += nthreads) {
    int i, j;
    if (t < 2 * w) {
      i = rg.x + t % w;
      j = t < w ? rg.z : rg.w - 1;
    } else {
      const int q = t - 2 * w;
      j = rg.z + 1 + q % h;
      i = q < h ? rg.x : rg.y - 1;
    }
    frame_cell<T>(S, i, j, n, 0, 1);
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
    tband<C>(S, M, R, ud.y, ud.z, ud.w, (ud.x >> 4) & 7, n, err);
    if (*(volatile int*)err) return;
  }
}

template <class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks2)
step_tmat2_kernel(const __grid_constant__ DevShot S, const __grid_constant__ TensorMaps M,
                  const int4* __restrict__ units, int n_units, int n_global, int4 rg, int* ctr, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[C::kStages], empty[C::kStages];
  __shared__ int next;
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
  if (n < 1 || n + 1 > S.n_steps) return;
  // Units are taken in turn, so that CTAs that start late (the SM still
  // held by the CPML-band kernel running beside this one) take fewer.
  for (;;) {
    if (threadIdx.x == 0) next = *(volatile int*)err ? n_units : atomicAdd(ctr, 1);
    __syncthreads();
    const int u = next;
    __syncthreads();
    if (u >= n_units) return;
    const int4 ud = __ldg(units + u);
    if (ud.x & kUnitRing) {
      ring_unit<typename C::Elem>(S, rg, ud, n, C::kThreads);
    } else {
      tband2<C>(S, M, R, ud, n, err);
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256) frame_kernel(const __grid_constant__ DevShot S, int ci0, int ci1, int ri0,
                                                    int ri1, int n_global, int* ctr) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *ctr = 0;
  const int n = n_global - S.base_n;
  if (n < 1 || n > S.n_steps) return;
  const int w = ci1 - ci0 + 4;          // frame row width
  const int h = ri1 - ri0;              // side column height
  const int n_tb = 4 * w, n_all = n_tb + 4 * h;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_all; t += gridDim.x * blockDim.x) {
    int i, j;
    if (t < n_tb) {
      const int r = t / w;                     // rows ri0-2, ri0-1, ri1, ri1+1
      i = ci0 - 2 + t % w;
      j = r < 2 ? ri0 - 2 + r : ri1 + r - 2;
    } else {
      const int q = t - n_tb, r = q / h;       // columns ci0-2, ci0-1, ci1, ci1+1
      j = ri0 + q % h;
      i = r < 2 ? ci0 - 2 + r : ci1 + r - 2;
    }
    frame_cell<T>(S, i, j, n, (n - 1) & 1, n & 1);
  }
}

using TKernelFn = void (*)(DevShot, TensorMaps, const int4*, int, int, int*);
using TKernelFn2 = void (*)(DevShot, TensorMaps, const int4*, int, int, int4, int*, int*);

struct TShape {
  int warps, rows, stages;
  TKernelFn fn[3];
  size_t smem[3];
  int bx;
  TKernelFn2 fn2[3];   // two-step form
};

template <int W, int R, int ST>
constexpr TShape tentry() {
  using C32 = TCfg<W, R, ST, float>;
  using C16 = TCfg<W, R, ST, __half>;
  using CB16 = TCfg<W, R, ST, __nv_bfloat16>;
  return {W, R, ST, {step_tmat_kernel<C32>, step_tmat_kernel<C16>, step_tmat_kernel<CB16>},
          {C32::kSmem, C16::kSmem, CB16::kSmem}, C32::kBX,
          {step_tmat2_kernel<C32>, step_tmat2_kernel<C16>, step_tmat2_kernel<CB16>}};
}

// Compiled shapes (warps, rows per stage, stages); the first is the default.
const TShape kTShapes[] = {tentry<4, 4, 2>(), tentry<4, 2, 3>(), tentry<4, 4, 3>(), tentry<2, 8, 2>(),
                           tentry<4, 8, 2>(), tentry<8, 2, 2>(), tentry<4, 2, 2>()};
constexpr int kNumTShapes = sizeof(kTShapes) / sizeof(kTShapes[0]);

}  // namespace

int tmat_shape_count() { return kNumTShapes; }

int tmat_shape_find(int warps, int rows, int stages) {
  for (int k = 0; k < kNumTShapes; ++k)
    if (kTShapes[k].warps == warps && kTShapes[k].rows == rows && kTShapes[k].stages == stages) return k;
  return -1;
}

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

cudaError_t launch_step_tmat2(int shape, const DevShot& shot, const TensorMaps& maps, const int4* units,
                              int n_units, int n_global, int4 ring, int max_ctas, int* ctr, int* err,
                              cudaStream_t stream) {
  const TShape& e = kTShapes[shape];
  const int ctas = max_ctas < n_units ? max_ctas : n_units;
  if (ctas <= 0) return cudaSuccess;
  if (shot.sc[1] != shot.sc[2]) return cudaErrorInvalidValue;   // one H scale (stored-unit curl)
  const int st = shot.store;
  e.fn2[st]<<<ctas, e.warps * 32, e.smem[st], stream>>>(shot, maps, units, n_units, n_global, ring, ctr, err);
  return cudaGetLastError();
}

cudaError_t launch_frame(const DevShot& shot, int ci0, int ci1, int ri0, int ri1, int n_global, int* ctr,
                         cudaStream_t stream) {
  const int64_t cells = 4 * (int64_t)(ci1 - ci0 + 4) + 4 * (int64_t)(ri1 - ri0);
  const int blocks = (int)std::min<int64_t>((cells + 255) / 256, 1024);
  if (shot.store == 0)
    frame_kernel<float><<<blocks, 256, 0, stream>>>(shot, ci0, ci1, ri0, ri1, n_global, ctr);
  else if (shot.store == 1)
    frame_kernel<__half><<<blocks, 256, 0, stream>>>(shot, ci0, ci1, ri0, ri1, n_global, ctr);
  else
    frame_kernel<__nv_bfloat16><<<blocks, 256, 0, stream>>>(shot, ci0, ci1, ri0, ri1, n_global, ctr);
  return cudaGetLastError();
}

int tmat2_resident_ctas(int shape, int store, int device) {
  const TShape& e = kTShapes[shape];
  cudaFuncSetAttribute(e.fn2[store], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem[store]);
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e.fn2[store], e.warps * 32, e.smem[store]);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
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
