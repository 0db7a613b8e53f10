// Fused TMz step, shared-memory staged with bulk asynchronous copies (TMA).
//
// Same arithmetic and the same ping-pong buffers as step_stream_kernel, but
// the rows reach the warps through shared memory: a CTA of W warps owns a
// band of 128*W columns of one shot and walks a range of rows; one thread
// keeps a ring of ST row stages filled with cp.async.bulk copies (Ez(j+1),
// Hx(j), Hy(j), Jz(j), plasma drive (j), each the row segment [c0-4,
// c0+128W+4), halo included, in one copy; plus the CPML psi rows the band
// reads in row j), completion tracked by an mbarrier per stage.  Bytes in
// flight per SM are then set by the ring depth instead of by registers per
// warp, and the warp-edge neighbours (Ez(i0-1), Ez(i0+128), Hy(i0-1)) come
// from shared memory instead of dependent global loads.  The launch shape
// (W, ST) is a template parameter; TmaShape lists the compiled ones.
//
// Every wait is bounded: after kWaitNs (1 s) without progress the kernel records
// kErrWaitTimeout in the shot's error word, waits (bounded) for the copies it
// issued, and returns; the host reports FDTD2D_ERR_TIMEOUT.
#include <cstdio>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "internal.h"
#include "step_common.cuh"
#include "tma_common.cuh"

namespace fdtd2d {

namespace {

constexpr int kXSlot = 128;                    // floats reserved per staged x-strip row
constexpr int kTmaMaxPml = kXSlot - 8;         // x-strip rows fit their stage slot

// Launch shape: W warps (a band of 128*W columns) and an ST-stage ring, for
// field storage element type T.
template <int W, int ST, class T>
struct Cfg {
  using Elem = T;
  static constexpr int kWarps = W;
  static constexpr int kThreads = W * 32;
  static constexpr int kStages = ST;
  static constexpr int kBand = W * kCols;
  static constexpr int kHalo = 16 / (int)sizeof(T);        // halo elements each side: 16 bytes
  static constexpr int kSeg = kBand + 2 * kHalo;           // staged elements per array row
  // A stage holds one row j of the band (byte offsets): Ez(j+1), Hx, Hy, Jz,
  // drive segments (T); the psi_Hxy and psi_Ezy rows of the band (float; CPML
  // y-strip rows only); and the row's x-strip psi rows (float; psi_Hyx side
  // 0/1, psi_Ezx side 0/1; bands touching a strip only), each copied from its
  // 16-byte-aligned start.
  static constexpr uint32_t kSegBytes = kSeg * sizeof(T);
  static constexpr uint32_t kPsiOffB = 5 * kSegBytes;
  static constexpr uint32_t kPsiBytes = kBand * 4;
  static constexpr uint32_t kXOffB = kPsiOffB + 2 * kPsiBytes;
  static constexpr uint32_t kStageBytes = kXOffB + 4 * kXSlot * 4;
  static constexpr size_t kSmem = (size_t)ST * kStageBytes;
  // CTAs per SM the launch bounds ask for: W = 1 at 16 CTAs (no spills),
  // W = 2 at 10 (96 registers; 8 bytes of spills in FP32, none for 16-bit
  // storage; measured a little faster than 8 CTAs at 128 registers), W = 8
  // at 128 registers (2 CTAs)
  static constexpr int kMinBlocks = W == 1 ? 16 : (W == 2 ? 10 : (W <= 4 ? 4 : 2));
  static_assert(kSegBytes % 16 == 0 && kPsiOffB % 16 == 0 && kXOffB % 16 == 0 && kStageBytes % 16 == 0,
                "16-byte aligned stage slots");
};

struct Ring {
  unsigned char* stage;  // kStages * kStageBytes
  uint64_t* full;        // completion of a stage's copies
  uint64_t* empty;       // all warps done reading a stage
  uint32_t issued = 0;   // rows issued into the ring (producer thread only)
  uint32_t used = 0;     // rows consumed (every thread)
};

// CPML y-strip rows: psi_Hxy row (side, r) for Hx at row j and psi_Ezy row
// for Ez at row j, or -1 when row j is outside that strip.
__device__ __forceinline__ int hxy_row(const DevShot& S, int j) {
  const int P = S.npml;
  if (j <= P - 2) return j;
  if (j >= S.ny - P) return (P - 1) + (S.ny - 2 - j);
  return -1;
}
__device__ __forceinline__ int ezy_row(const DevShot& S, int j) {
  const int P = S.npml;
  if (j >= 1 && j <= P - 1) return j;
  if (j >= S.ny - P && j <= S.ny - 2) return P + (S.ny - 1 - j);
  return -1;
}

// x-strip sides a band reads: bit 0 = side 0 (columns < P), bit 1 = side 1
// (columns >= nx - P), including the Hy halo column c0 - 1.  With P below
// kTmaMaxPml only the first band reaches side 0.
template <int BAND>
__device__ __forceinline__ int band_x_sides(const DevShot& S, int c0) {
  return (c0 == 0 ? 1 : 0) | (c0 + BAND - 1 >= S.nx - S.npml ? 2 : 0);
}

// Float offset, within S.psi, of x-strip row (side, j) of the array at `o`.
__device__ __forceinline__ int64_t xstrip_off(const DevShot& S, int par, int64_t o, int side, int j) {
  return par * S.psi_buf + o + ((int64_t)side * S.ny + j) * S.npml;
}

// Producer: copy row `j` of the unit (band starting at c0) into the next stage.
template <class C>
__device__ bool issue_row(Ring& R, const DevShot& S, int par, int c0, int j, bool has_kp, int xs) {
  const uint32_t g = R.issued++;
  const int s = g % C::kStages;
  if (g >= (uint32_t)C::kStages && !mbar_wait(&R.empty[s], ((g / C::kStages) - 1) & 1)) return false;
  using T = typename C::Elem;
  const int64_t row = (int64_t)j * S.pitch + c0 - C::kHalo;
  unsigned char* dst = R.stage + s * C::kStageBytes;
  const int rh = hxy_row(S, j), re = ezy_row(S, j);
  uint32_t xbytes[4] = {0, 0, 0, 0};
  int64_t xa[4] = {0, 0, 0, 0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int side = q & 1;
    if (!((xs >> side) & 1)) continue;
    const int64_t off = xstrip_off(S, par, (q >> 1) ? S.o_ezx : S.o_hyx, side, j);
    xa[q] = off & ~(int64_t)3;
    xbytes[q] = (uint32_t)((((off + S.npml + 3) & ~(int64_t)3) - xa[q]) * 4);
  }
  mbar_expect_tx(&R.full[s], C::kSegBytes * (has_kp ? 5 : 4) + (rh >= 0 ? C::kPsiBytes : 0) + (re >= 0 ? C::kPsiBytes : 0) +
                                 xbytes[0] + xbytes[1] + xbytes[2] + xbytes[3]);
  const float* psr = S.psi + par * S.psi_buf;
  if (rh >= 0) bulk_copy(dst + C::kPsiOffB, psr + (int64_t)rh * S.pitch + c0, C::kPsiBytes, &R.full[s]);
  if (re >= 0)
    bulk_copy(dst + C::kPsiOffB + C::kPsiBytes, psr + S.o_ezy + (int64_t)re * S.pitch + c0, C::kPsiBytes, &R.full[s]);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (xbytes[q]) bulk_copy(dst + C::kXOffB + q * kXSlot * 4, S.psi + xa[q], xbytes[q], &R.full[s]);
  bulk_copy(dst + 0 * C::kSegBytes, field_ptr_t<T>(S, kEz, par) + row + S.pitch, C::kSegBytes, &R.full[s]);
  bulk_copy(dst + 1 * C::kSegBytes, field_ptr_t<T>(S, kHx, par) + row, C::kSegBytes, &R.full[s]);
  bulk_copy(dst + 2 * C::kSegBytes, field_ptr_t<T>(S, kHy, par) + row, C::kSegBytes, &R.full[s]);
  bulk_copy(dst + 3 * C::kSegBytes, field_ptr_t<T>(S, kJz, par) + row, C::kSegBytes, &R.full[s]);
  if (has_kp) bulk_copy(dst + 4 * C::kSegBytes, reinterpret_cast<const T*>(S.kp) + row, C::kSegBytes, &R.full[s]);
  return true;
}

// After a timed-out wait: wait (bounded) for every copy still in flight.
template <class C>
__device__ void drain(Ring& R) {
  for (uint32_t g = R.used; g < R.issued; ++g) mbar_wait(&R.full[g % C::kStages], (g / C::kStages) & 1);
}

template <class C>
__device__ void process_band(const DevShot& S, Ring& R, const float* __restrict__ cp, int c0, int j0, int j1, int n,
                             int* err) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nx = S.nx, ny = S.ny, P = S.npml;
  const int64_t pitch = S.pitch;
  const int par = (n - 1) & 1;
  const bool has_kp = S.kp != nullptr;
  const int xs = band_x_sides<C::kBand>(S, c0);
  using T = typename C::Elem;
  using St = Sto<T>;
  const T* __restrict__ ezo = field_ptr_t<T>(S, kEz, par);
  const T* __restrict__ hxo_p = field_ptr_t<T>(S, kHx, par);
  T* __restrict__ ezw = field_ptr_t<T>(S, kEz, par ^ 1);
  T* __restrict__ hxw = field_ptr_t<T>(S, kHx, par ^ 1);
  T* __restrict__ hyw = field_ptr_t<T>(S, kHy, par ^ 1);
  T* __restrict__ jzw = field_ptr_t<T>(S, kJz, par ^ 1);
  float* __restrict__ psw = S.psi + (par ^ 1) * S.psi_buf;
  // per-array scales (Ez, Hx, Hy, Jz, drive); 1 for F32 storage
  const float sE = S.sc[0], sHx = S.sc[1], sHy = S.sc[2], sJ = S.sc[3], sK = S.sc[4];

  const int i0 = c0 + warp * kCols;            // this warp's first column
  const int i = i0 + 4 * lane;
  const bool act = i < nx;
  const int ic = act ? i : 0;
  const int sl = C::kHalo + warp * kCols + 4 * lane;  // lane's 4 elements in a staged segment
  const int rows = j1 - j0;
  // The producer thread: lane 0 of a warp with no x-strip columns where the
  // band has one (the first band's strip is in warp 0, the last band's in
  // warp W-1), so the ring refill does not wait on the slower CPML lanes.
  const int prod_warp = (c0 == 0 && C::kWarps > 1) ? C::kWarps - 1 : 0;
  const bool producer = tid == prod_warp * 32;
  // The ring is drained between units (every issued row was consumed), and
  // every thread counts the consumed rows, so the ring position carries over
  // to whichever thread produces for this unit.
  R.issued = R.used;

  // Fill the ring.
  if (producer) {
    for (int r = 0; r < rows && r < C::kStages; ++r)
      if (!issue_row<C>(R, S, par, c0, j0 + r, has_kp, xs)) {
        atomicExch(err, kErrWaitTimeout);
        drain<C>(R);
        return;
      }
  }

  MediumRow<0> m;
  m.init(S);
  float dex[4], dhx[4];
  ld4(dex, S.den_ex + ic);
  ld4(dhx, S.den_hx + ic);
  const float dhx_left = i0 >= 1 ? __ldg(S.den_hx + i0 - 1) : 0.f;  // lane 0's halo column

  // Row j0 state from global memory: Ez(j0) (+ the band-edge halo values the
  // lane needs) and Hx_new(j0-1), recomputed from the old buffers.
  float ezc[4], hxp[4];
  zero4(ezc);
  zero4(hxp);
  if (act) St::ldg4(ezc, ezo + (int64_t)j0 * pitch + ic, sE);
  float ezl = (lane == 0 && i0 >= 1) ? St::ldg1(ezo + (int64_t)j0 * pitch + i0 - 1, sE) : 0.f;  // Ez(i0-1, j)
  float ezr = (lane == 31 && i0 + kCols < nx) ? St::ldg1(ezo + (int64_t)j0 * pitch + i0 + kCols, sE) : 0.f;
  if (j0 >= 1) {
    float ezp[4], hxo[4];
    zero4(ezp);
    zero4(hxo);
    if (act) {
      St::ldg4(ezp, ezo + (int64_t)(j0 - 1) * pitch + ic, sE);
      St::ldg4(hxo, hxo_p + (int64_t)(j0 - 1) * pitch + ic, sHx);
    }
    hx_row<0>(S, m, par, ic, j0 - 1, ezp, ezc, hxo, hxp, false);
  }

  // Per-row scalars (denominators, point range), loaded one row ahead.
  float dhy = __ldg(S.den_hy + j0), dey = __ldg(S.den_ey + j0);
  int p0 = __ldg(S.row_start + j0), p1 = __ldg(S.row_start + j0 + 1);

  for (int j = j0; j < j1; ++j) {
    const int jn = j + 1 < j1 ? j + 1 : j;
    const float dhy_n = __ldg(S.den_hy + jn), dey_n = __ldg(S.den_ey + jn);
    const int p1_n = __ldg(S.row_start + jn + 1);

    const uint32_t g = R.used;
    const int s = g % C::kStages;
    if (!mbar_wait(&R.full[s], (g / C::kStages) & 1)) {
      atomicExch(err, kErrWaitTimeout);
      if (producer) drain<C>(R);
      return;
    }
    const unsigned char* st = R.stage + s * C::kStageBytes;
    const T* sg0 = reinterpret_cast<const T*>(st);                       // Ez(j+1)
    const T* sg1 = reinterpret_cast<const T*>(st + 1 * C::kSegBytes);    // Hx(j)
    const T* sg2 = reinterpret_cast<const T*>(st + 2 * C::kSegBytes);    // Hy(j)
    const T* sg3 = reinterpret_cast<const T*>(st + 3 * C::kSegBytes);    // Jz(j)
    const T* sg4 = reinterpret_cast<const T*>(st + 4 * C::kSegBytes);    // drive(j)
    const float* sps = reinterpret_cast<const float*>(st + C::kPsiOffB);  // psi_Hxy, psi_Ezy rows
    const float* sxs = reinterpret_cast<const float*>(st + C::kXOffB);    // x-strip rows
    float ezn[4], hxo[4], hyo[4], jzo[4];
    St::lds4(ezn, sg0 + sl, sE);
    St::lds4(hxo, sg1 + sl, sHx);
    St::lds4(hyo, sg2 + sl, sHy);
    St::lds4(jzo, sg3 + sl, sJ);
    if (has_kp) {
      St::lds4(m.kp, sg4 + sl, sK);
    } else {
      zero4(m.kp);
    }
    // halo values of row j+1 for the next iteration, and Hy_old(i0-1, j)
    const float ezl_next = St::ld1(sg0 + C::kHalo + warp * kCols - 1, sE);
    const float ezr_next = St::ld1(sg0 + C::kHalo + warp * kCols + kCols, sE);
    const float hyo_left = St::ld1(sg2 + C::kHalo + warp * kCols - 1, sHy);
    // staged x-strip rows (psi_Hyx, psi_Ezx; side 0, 1): value r at x..[r]
    const float* xh0 = sxs + 0 * kXSlot + (int)(xstrip_off(S, 0, S.o_hyx, 0, j) & 3);
    const float* xh1 = sxs + 1 * kXSlot + (int)(xstrip_off(S, 0, S.o_hyx, 1, j) & 3);
    const float* xe0 = sxs + 2 * kXSlot + (int)(xstrip_off(S, 0, S.o_ezx, 0, j) & 3);
    const float* xe1 = sxs + 3 * kXSlot + (int)(xstrip_off(S, 0, S.o_ezx, 1, j) & 3);

    // ---- H update: Hx bulk + y-strip CPML (psi from the stage)
    const int rh = hxy_row(S, j), re = ezy_row(S, j);
    float hxn[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      hxn[k] = (i + k <= nx - 2) ? upd_h(S.da, hxo[k], S.db, ezc[k], ezn[k], dhy) : hxo[k];
    if (rh >= 0) {
      const int side = rh >= P - 1, r = side ? rh - (P - 1) : rh;
      const float b = cp[(side ? kBhY2 : kBhY1) * P + r];
      const float cc = cp[(side ? kChY2 : kChY1) * P + r];
      float psh[4], pn[4];
      lds4f(psh, sps + warp * kCols + 4 * lane);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        pn[k] = psh[k];
        if (i + k <= nx - 2) {
          pn[k] = upd_psi(b, psh[k], cc, ezc[k], ezn[k]);
          hxn[k] = __fmaf_rn(S.db, pn[k], hxn[k]);
        }
      }
      if (act) st4(psw + (int64_t)rh * pitch + ic, pn);
    }
    float ezr_k = __shfl_down_sync(0xffffffffu, ezc[0], 1);
    if (lane == 31) ezr_k = ezr;
    const float ezr4[4] = {ezc[1], ezc[2], ezc[3], ezr_k};
    float hyn[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      hyn[k] = (i + k <= nx - 2) ? upd_h(m.day(k), hyo[k], m.dby(k), ezr4[k], ezc[k], dhx[k]) : hyo[k];
    if (act && (i <= P - 2 || i + 3 >= nx - P)) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c <= P - 2) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 2 - c; }
        if (side >= 0) {
          const float b = cp[(side ? kBhX2 : kBhX1) * P + r];
          const float cc = cp[(side ? kChX2 : kChX1) * P + r];
          const float pn = upd_psi(b, (side ? xh1 : xh0)[r], cc, ezr4[k], ezc[k]);
          hyn[k] = __fmaf_rn(m.dby(k), pn, hyn[k]);
          psw[S.o_hyx + ((int64_t)side * ny + j) * P + r] = pn;
        }
      }
    }
    // Hy_new(i-1): lane 0 recomputes the band/warp-edge value from staged data.
    float hyl = __shfl_up_sync(0xffffffffu, hyn[3], 1);
    if (lane == 0) {
      hyl = 0.f;
      if (i0 >= 1) {
        const int c = i0 - 1;
        float h = upd_h(S.da, hyo_left, S.db, ezc[0], ezl, dhx_left);
        int side = -1, r = 0;
        if (c <= P - 2) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 2 - c; }
        if (side >= 0) {
          const float b = cp[(side ? kBhX2 : kBhX1) * P + r];
          const float cc = cp[(side ? kChX2 : kChX1) * P + r];
          const float pn = upd_psi(b, (side ? xh1 : xh0)[r], cc, ezc[0], ezl);
          h = __fmaf_rn(S.db, pn, h);
        }
        hyl = h;
      }
    }

    // ---- Jz, Ez
    const bool row_in = (j >= 1) && (j <= ny - 2);
    const float hyl4[4] = {hyl, hyn[0], hyn[1], hyn[2]};
    float ezw4[4], jzw4[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int c = i + k;
      const bool in = row_in && c >= 1 && c <= nx - 2;
      jzw4[k] = in ? upd_j(S.ja, jzo[k], m.kp[k], ezc[k]) : jzo[k];
      ezw4[k] = in ? upd_e(S.ca, ezc[k], S.cb, __fsub_rn(hyn[k], hyl4[k]), dex[k], __fsub_rn(hxp[k], hxn[k]),
                           dey, jzw4[k])
                   : ezc[k];
    }
    if (act && row_in && (i <= P - 1 || i + 3 >= nx - P)) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c >= 1 && c <= P - 1) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 1 - c; }
        if (side >= 0) {
          const float b = cp[(side ? kBeX2 : kBeX1) * P + r];
          const float cc = cp[(side ? kCeX2 : kCeX1) * P + r];
          const float pn = upd_psi(b, (side ? xe1 : xe0)[r], cc, hyn[k], hyl4[k]);
          ezw4[k] = __fmaf_rn(S.cb, pn, ezw4[k]);
          psw[S.o_ezx + ((int64_t)side * ny + j) * P + r] = pn;
        }
      }
    }
    if (act && re >= 0) {
      const int side = re >= P, r = side ? re - P : re;
      const float b = cp[(side ? kBeY2 : kBeY1) * P + r];
      const float cc = cp[(side ? kCeY2 : kCeY1) * P + r];
      float pse[4], pn[4];
      lds4f(pse, sps + C::kBand + warp * kCols + 4 * lane);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        pn[k] = pse[k];
        if (i + k >= 1 && i + k <= nx - 2) {
          pn[k] = upd_psi(b, pse[k], cc, hxp[k], hxn[k]);
          ezw4[k] = __fmaf_rn(S.cb, pn[k], ezw4[k]);
        }
      }
      st4(psw + S.o_ezy + (int64_t)re * pitch + ic, pn);
    }
    // Every read of this stage is done: release it to the producer.
    __syncwarp();
    if (lane == 0) mbar_arrive(&R.empty[s]);
    R.used++;

    // ---- sources, then detectors, of this row
    for (int p = p0; p < p1; ++p) {
      const int4 pt = __ldg(S.pts + p);
      const int k = pt.x - i;
      if (!act || k < 0 || k > 3) continue;
      float e = 0.f;
#pragma unroll
      for (int q = 0; q < 4; ++q) if (q == k) e = ezw4[q];
      if (pt.y == kPointSource) {
        e = __fsub_rn(e, __ldg(S.src_val + (int64_t)n * S.n_src + pt.z));
#pragma unroll
        for (int q = 0; q < 4; ++q) if (q == k) ezw4[q] = e;
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
        for (int q = 0; q < 4; ++q) if (q == k) { hxv = hxn[q]; hyv = hyn[q]; }
        if (S.record) {
          float* dst = S.ctrace + ((int64_t)(n - 1) * S.n_comp + pt.z) * 3;
          dst[0] = e; dst[1] = hxv; dst[2] = hyv;
        }
      }
    }

    if (act) {
      const int64_t o = (int64_t)j * pitch + ic;
      St::stcs4(hxw + o, hxn, S.isc[1]);
      St::stcs4(hyw + o, hyn, S.isc[2]);
      St::stcs4(ezw + o, ezw4, S.isc[0]);
      St::stcs4(jzw + o, jzw4, S.isc[3]);
    }

    // Producer: refill this stage with row j + C::kStages.
    if (producer && j + C::kStages < j1) {
      if (!issue_row<C>(R, S, par, c0, j + C::kStages, has_kp, xs)) {
        atomicExch(err, kErrWaitTimeout);
        drain<C>(R);
        return;
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hxp[k] = hxn[k];
      ezc[k] = ezn[k];
    }
    ezl = ezl_next;
    ezr = ezr_next;
    dhy = dhy_n;
    dey = dey_n;
    p0 = p1;
    p1 = p1_n;
  }
}

// The shot descriptor is a __grid_constant__ parameter: its fields are read
// through the constant cache, and the compiler need not reload them after the
// kernel's global stores (a descriptor in global memory could alias them).
template <class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks)
step_tma_kernel(const __grid_constant__ DevShot S, const int4* __restrict__ units, int n_units, int n_global,
                int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[C::kStages], empty[C::kStages];
  // The CPML coefficient table (kCpmlRows x P floats) sits after the ring:
  // its reads are per lane (x strips) or per row (y strips) on the critical
  // path, so they come from shared memory instead of the L1/L2.
  float* cp = reinterpret_cast<float*>(smem + C::kStages * C::kStageBytes);
  for (int t = threadIdx.x; t < kCpmlRows * S.npml; t += C::kThreads) cp[t] = S.cpml[t];
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  Ring R;
  R.stage = smem;
  R.full = full;
  R.empty = empty;
  const int n = n_global - S.base_n;
  if (n < 1 || n > S.n_steps) return;
  for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
    const int4 ud = __ldg(units + u);
    process_band<C>(S, R, cp, ud.y, ud.z, ud.w, n, err);
    if (*(volatile int*)err) return;
  }
}

// Batched form: one launch advances every shot of a batch by one step.  The
// shots' descriptors sit in a device array; units (shot, c0, j0, j1) are
// handed out dynamically (one atomic counter per step parity, so CTAs that
// drew short or fast units take more); each shot runs its own step
// n = n_global - base_n, and units of shots outside [1, n_steps] are skipped,
// so shots admitted at different times advance together.  n_global is read
// from device memory (the step-block base, advanced by the graph's last node)
// plus the launch's offset k within the block, so one captured graph of K
// launches serves every block.
template <class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks)
step_tma_batch_kernel(const DevShot* __restrict__ shots, const int4* __restrict__ units,
                      const int* __restrict__ n_units_p, const int* __restrict__ gstep_p, int k, int* counters,
                      int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[C::kStages], empty[C::kStages];
  __shared__ __align__(16) DevShot sS;
  __shared__ int s_unit;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int n_global = *gstep_p + k + 1;
  const int n_units = *n_units_p;
  int* ctr = counters + (n_global & 1);
  if (blockIdx.x == 0 && tid == 0) counters[(n_global + 1) & 1] = 0;   // the next step's counter
  __syncthreads();
  Ring R;
  R.stage = smem;
  R.full = full;
  R.empty = empty;
  float* cp = reinterpret_cast<float*>(smem + C::kStages * C::kStageBytes);   // CPML table of the current shot
  int cur = -1;
  for (;;) {
    if (tid == 0) s_unit = *(volatile int*)err ? n_units : atomicAdd(ctr, 1);
    __syncthreads();
    const int u = s_unit;
    if (u >= n_units) break;
    const int4 ud = __ldg(units + u);
    if (ud.x != cur) {
      const int* src = reinterpret_cast<const int*>(shots + ud.x);
      int* dst = reinterpret_cast<int*>(&sS);
      for (int t = tid; t < (int)(sizeof(DevShot) / 4); t += C::kThreads) dst[t] = __ldg(src + t);
      __syncthreads();
      for (int t = tid; t < kCpmlRows * sS.npml; t += C::kThreads) cp[t] = sS.cpml[t];
      cur = ud.x;
      __syncthreads();
    }
    const int n = n_global - sS.base_n;
    if (n >= 1 && n <= sS.n_steps) process_band<C>(sS, R, cp, ud.y, ud.z, ud.w, n, err);
    __syncthreads();   // every thread has read s_unit (and sS) before the next unit overwrites them
  }
}

using KernelFn = void (*)(DevShot, const int4*, int, int, int*);
using BatchFn = void (*)(const DevShot*, const int4*, const int*, const int*, int, int*, int*);

// One launch shape: the single-shot kernel per storage type (F32, F16,
// BF16) and the batched kernel (F32 storage).
struct ShapeEntry {
  int warps, stages;
  KernelFn fn[3];
  size_t smem[3];
  BatchFn bfn;
};

template <int W, int ST>
constexpr ShapeEntry entry() {
  using C32 = Cfg<W, ST, float>;
  using C16 = Cfg<W, ST, __half>;
  using CB16 = Cfg<W, ST, __nv_bfloat16>;
  return {W, ST, {step_tma_kernel<C32>, step_tma_kernel<C16>, step_tma_kernel<CB16>},
          {C32::kSmem, C16::kSmem, CB16::kSmem}, step_tma_batch_kernel<C32>};
}

// Compiled launch shapes; the first is the default.
const ShapeEntry kShapes[] = {entry<4, 3>(), entry<4, 2>(), entry<4, 4>(), entry<4, 6>(),
                              entry<8, 2>(), entry<8, 3>(), entry<8, 4>(), entry<2, 4>(), entry<2, 6>(),
                              entry<2, 2>(), entry<2, 3>(), entry<1, 2>(), entry<1, 3>(), entry<1, 4>()};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

}  // namespace

int tma_shape_count() { return kNumShapes; }

int tma_shape_find(int warps, int stages) {
  for (int k = 0; k < kNumShapes; ++k)
    if (kShapes[k].warps == warps && kShapes[k].stages == stages) return k;
  return -1;
}

void tma_shape_dims(int shape, int* warps, int* stages) {
  *warps = kShapes[shape].warps;
  *stages = kShapes[shape].stages;
}

int tma_shape_parse(const char* text) {
  int w = 0, st = 0;
  if (!text || std::sscanf(text, "%d,%d", &w, &st) != 2) return -1;
  return tma_shape_find(w, st);
}

void tma_shape_name(int shape, const char* kernel, char* out, size_t n) {
  std::snprintf(out, n, "%s<%d,%d>", kernel, kShapes[shape].warps, kShapes[shape].stages);
}

int tma_band_cols(int shape) { return kShapes[shape].warps * kCols; }

int tma_max_pml() { return kTmaMaxPml; }

// Dynamic shared memory of one CTA: the ring, then the CPML table.
static size_t smem_bytes(size_t ring, int npml) {
  return ring + (((size_t)kCpmlRows * npml * sizeof(float) + 15) & ~(size_t)15);
}

cudaError_t launch_step_tma(int shape, const DevShot& shot, const int4* units, int n_units, int n_global,
                            int max_ctas, int* err, cudaStream_t stream) {
  const ShapeEntry& e = kShapes[shape];
  const int ctas = max_ctas < n_units ? max_ctas : n_units;
  if (ctas <= 0) return cudaSuccess;
  const int st = shot.store;
  e.fn[st]<<<ctas, e.warps * 32, smem_bytes(e.smem[st], shot.npml), stream>>>(shot, units, n_units, n_global,
                                                                            err);
  return cudaGetLastError();
}

cudaError_t launch_step_tma_batch(int shape, const DevShot* shots, const int4* units, const int* n_units,
                                  const int* gstep, int k, int* counters, int max_pml, int ctas, int* err,
                                  cudaStream_t stream) {
  const ShapeEntry& e = kShapes[shape];
  e.bfn<<<ctas, e.warps * 32, smem_bytes(e.smem[0], max_pml), stream>>>(shots, units, n_units, gstep, k, counters,
                                                                         err);
  return cudaGetLastError();
}

int tma_batch_resident_ctas(int shape, int max_pml, int device) {
  const ShapeEntry& e = kShapes[shape];
  const size_t smem = smem_bytes(e.smem[0], max_pml);
  cudaFuncSetAttribute(e.bfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(e.smem[0], kTmaMaxPml));
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e.bfn, e.warps * 32, smem);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

int tma_resident_ctas(int shape, int npml, int store, int device) {
  const ShapeEntry& e = kShapes[shape];
  const size_t smem = smem_bytes(e.smem[store], npml);
  cudaFuncSetAttribute(e.fn[store], cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes(e.smem[store], kTmaMaxPml));
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e.fn[store], e.warps * 32, smem);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fdtd2d
