// Fused TMz step for sm_103a: Hx/Hy (+CPML psi) -> Jz -> Ez (+CPML psi) ->
// source -> detectors in ONE pass over HBM per step.
//
// The reference runs this as 8-12 launches per step (FDTD_2D_Full/kernel.cu
// :2073-2157), each re-reading the fields: about 84 B of HBM traffic per cell
// update.  Here each warp streams a 128-column block of one shot up a range
// of rows.  Per row it reads Ez(j+1), Hx(j), Hy(j), Jz(j) and the plasma
// coefficient once (float4 per lane, 512 B per warp per array, fully
// coalesced) and writes Ez, Hx, Hy, Jz once: the 36 B/cell minimum.
//
// Neighbour values come from registers: Ez(j) and Hx_new(j-1) roll from the
// previous row, Ez(i+1) and Hy_new(i-1) arrive by warp shuffle.  Only the warp
// edges (lane 0's Hy_new(i0-1), lane 31's Ez(i0+128)) and the first row of a
// unit (Hx_new(j0-1)) are recomputed from global memory; those reads hit L2.
// Because a unit may recompute a neighbour-owned H value, every field is
// ping-ponged (read buffer (n-1)&1, write n&1), so no unit ever sees a value
// from the step it is computing.
//
// All update arithmetic goes through explicit-rounding intrinsics
// (__fmaf_rn, __fmul_rn, ...), so the owner's value and a recomputed copy are
// bit-identical whatever the surrounding code, and results do not depend on
// how the grid is cut into units.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "internal.h"
#include "step_common.cuh"
#include "tma_common.cuh"

#include <cstdio>

namespace fdtd2d {

template <int MEDIUM, bool kCoh = false>
__device__ __forceinline__ void process_unit(const DevShot& S, const MatE* mat_e, const MatH* mat_h,
                                             int i0, int j0, int j1, int n, int lane) {
  const int nx = S.nx, ny = S.ny, P = S.npml;
  const int64_t pitch = S.pitch;
  const int par = (n - 1) & 1;
  const float* __restrict__ ezo = field_ptr(S, kEz, par);
  const float* __restrict__ hxo_p = field_ptr(S, kHx, par);
  const float* __restrict__ hyo_p = field_ptr(S, kHy, par);
  const float* __restrict__ jzo_p = field_ptr(S, kJz, par);
  float* __restrict__ ezw = field_ptr(S, kEz, par ^ 1);
  float* __restrict__ hxw = field_ptr(S, kHx, par ^ 1);
  float* __restrict__ hyw = field_ptr(S, kHy, par ^ 1);
  float* __restrict__ jzw = field_ptr(S, kJz, par ^ 1);
  float* __restrict__ psr = S.psi + par * S.psi_buf;          // psi read buffer
  float* __restrict__ psw = S.psi + (par ^ 1) * S.psi_buf;    // psi write buffer

  const int i = i0 + 4 * lane;
  const bool act = i < nx;
  const int ic = act ? i : 0;  // clamp for address formation of inactive lanes

  float dex[4], dhx[4];
  ld4(dex, S.den_ex + ic);
  ld4(dhx, S.den_hx + ic);

  MediumRow<MEDIUM> m;
  m.init(S);
  float ezc[4], hxp[4];
  zero4(ezc);
  zero4(hxp);
  if (act) ldf4<kCoh>(ezc, ezo + (int64_t)j0 * pitch + ic);
  if (j0 >= 1) {
    // Hx_new(j0-1): recomputed from old values (the unit below owns it).
    float ezp[4], hxo[4];
    zero4(ezp); zero4(hxo);
    if (act) {
      ldf4<kCoh>(ezp, ezo + (int64_t)(j0 - 1) * pitch + ic);
      ldf4<kCoh>(hxo, hxo_p + (int64_t)(j0 - 1) * pitch + ic);
    }
    m.load(S, mat_e, mat_h, (int64_t)(j0 - 1) * pitch + ic);
    hx_row<MEDIUM, kCoh>(S, m, par, ic, j0 - 1, ezp, ezc, hxo, hxp, false);
  }

  // Prefetched row j data.
  float ezn[4], hxo[4], hyo[4], jzo[4];
  zero4(ezn); zero4(hxo); zero4(hyo); zero4(jzo);
  if (act) {
    const int64_t o = (int64_t)j0 * pitch + ic;
    ldfs4<kCoh>(ezn, ezo + o + pitch);   // j0 + 1 <= ny - 1 always (units stop at ny-1)
    ldfs4<kCoh>(hxo, hxo_p + o);
    ldfs4<kCoh>(hyo, hyo_p + o);
    ldfs4<kCoh>(jzo, jzo_p + o);
  }

  for (int j = j0; j < j1; ++j) {
    const int64_t o = (int64_t)j * pitch + ic;
    m.load(S, mat_e, mat_h, o);

    // Prefetch row j+1 (Ez of j+2) while row j is computed.
    float ezn2[4], hxo2[4], hyo2[4], jzo2[4];
    zero4(ezn2); zero4(hxo2); zero4(hyo2); zero4(jzo2);
    if (act && j + 1 < j1) {
      ldfs4<kCoh>(ezn2, ezo + o + 2 * pitch);
      ldfs4<kCoh>(hxo2, hxo_p + o + pitch);
      ldfs4<kCoh>(hyo2, hyo_p + o + pitch);
      ldfs4<kCoh>(jzo2, jzo_p + o + pitch);
    }

    // The row's other loads, issued together before its arithmetic: the
    // warp-edge Ez (lane 31: column i0+128; lane 0: i0-1) and lane 0's old
    // Hy(i0-1), and (uniform medium; the material form has no registers to
    // spare) the old psi of the row's CPML strip cells.
    constexpr bool kHoist = MEDIUM == 0;
    const bool row_in = (j >= 1) && (j <= ny - 2);
    float ez_edge = 0.f, hy_edge = 0.f;
    if (lane == 31 && i0 + kCols < nx) ez_edge = ldf1<kCoh>(ezo + (int64_t)j * pitch + i0 + kCols);
    if (lane == 0 && i0 >= 1) {
      ez_edge = ldf1<kCoh>(ezo + (int64_t)j * pitch + i0 - 1);
      hy_edge = ldf1<kCoh>(hyo_p + (int64_t)j * pitch + i0 - 1);
    }
    const bool xs_h = act && (i <= P - 2 || i + 3 >= nx - P);
    const bool xs_e = act && row_in && (i <= P - 1 || i + 3 >= nx - P);
    const bool ys_e = act && row_in && (j <= P - 1 || j >= ny - P);
    float psi_h[4], psi_e[4], psi_y[4];
    zero4(psi_h);
    zero4(psi_e);
    zero4(psi_y);
    if (kHoist && xs_h) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c <= P - 2) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 2 - c; }
        if (side >= 0) psi_h[k] = ldf1<kCoh>(psr + S.o_hyx + ((int64_t)side * ny + j) * P + r);
      }
    }
    if (kHoist && xs_e) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c >= 1 && c <= P - 1) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 1 - c; }
        if (side >= 0) psi_e[k] = ldf1<kCoh>(psr + S.o_ezx + ((int64_t)side * ny + j) * P + r);
      }
    }
    if (kHoist && ys_e) {
      const int side = (j <= P - 1) ? 0 : 1;
      const int r = side ? (ny - 1 - j) : j;
      ldf4<kCoh>(psi_y, psr + S.o_ezy + ((int64_t)side * P + r) * pitch + ic);
    }

    // ---- H update (Dev_HxCalc/Dev_HxPML_Jdir_Calc, Dev_HyCalc/Dev_HyPML_Idir_Calc)
    float hxn[4];
    hx_row<MEDIUM, kCoh>(S, m, par, ic, j, ezc, ezn, hxo, hxn, act);

    float ezr_next = __shfl_down_sync(0xffffffffu, ezc[0], 1);
    if (lane == 31) ezr_next = ez_edge;
    const float ezr[4] = {ezc[1], ezc[2], ezc[3], ezr_next};
    float hyn[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hyn[k] = (i + k <= nx - 2 && covered<MEDIUM>(S, kCovHy, (long long)j * (nx - 1) + i + k))
                   ? upd_h(m.day(k), hyo[k], m.dby(k), ezr[k], ezc[k], dhx[k]) : hyo[k];
    }
    // Hy x-strip CPML (edge columns only).
    if (xs_h) {
      float pn[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c <= P - 2) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 2 - c; }
        if (side >= 0 && covered<MEDIUM>(S, kCovHyPml, (long long)j * (P - 1) + r)) {
          const float b = S.cpml[(side ? kBhX2 : kBhX1) * P + r];
          const float cc = S.cpml[(side ? kChX2 : kChX1) * P + r];
          const int64_t po = S.o_hyx + ((int64_t)side * ny + j) * P + r;
          pn[k] = upd_psi(b, kHoist ? psi_h[k] : ldf1<kCoh>(psr + po), cc, ezr[k], ezc[k]);
          hyn[k] = __fmaf_rn(m.dby(k), pn[k], hyn[k]);
          psw[po] = pn[k];
        }
      }
    }
    float hyl = __shfl_up_sync(0xffffffffu, hyn[3], 1);
    if (lane == 0) {
      hyl = 0.f;
      if (i0 >= 1) hyl = hy_cell<MEDIUM, kCoh>(S, mat_h, par, i0 - 1, j, ez_edge, ezc[0], hy_edge);
    }

    // ---- Jz (Dev_JzCalc) and Ez (Dev_EzCalc) on interior cells
    const float dey = S.den_ey[j];
    const float hyl4[4] = {hyl, hyn[0], hyn[1], hyn[2]};
    float ezw4[4], jzw4[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int c = i + k;
      const bool in = row_in && c >= 1 && c <= nx - 2;
      const long long le = (long long)(j - 1) * (nx - 2) + (c - 1);
      jzw4[k] = (in && covered<MEDIUM>(S, kCovJz, le)) ? upd_j(S.ja, jzo[k], m.kp[k], ezc[k]) : jzo[k];
      float e = ezc[k];
      if (in && covered<MEDIUM>(S, kCovEz, le)) {
        e = m.pec(k) ? 0.f
                     : upd_e(m.cA(k), ezc[k], m.cB(k), __fsub_rn(hyn[k], hyl4[k]), dex[k],
                             __fsub_rn(hxp[k], hxn[k]), dey, jzw4[k]);
      }
      ezw4[k] = e;
    }
    // Ez x-strip CPML (Dev_EzPML_Idir_Calc), then y-strip (Dev_EzPML_Jdir_Calc).
    if (xs_e) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        int side = -1, r = 0;
        if (c >= 1 && c <= P - 1) { side = 0; r = c; }
        else if (c >= nx - P && c <= nx - 2) { side = 1; r = nx - 1 - c; }
        if (side >= 0 && covered<MEDIUM>(S, kCovEzPmlI, (long long)(j - 1) * (P - 1) + (r - 1))) {
          const float b = S.cpml[(side ? kBeX2 : kBeX1) * P + r];
          const float cc = S.cpml[(side ? kCeX2 : kCeX1) * P + r];
          const int64_t po = S.o_ezx + ((int64_t)side * ny + j) * P + r;
          const float pn = upd_psi(b, kHoist ? psi_e[k] : ldf1<kCoh>(psr + po), cc, hyn[k], hyl4[k]);
          ezw4[k] = __fmaf_rn(m.cB(k), pn, ezw4[k]);
          psw[po] = pn;
        }
      }
    }
    if (ys_e) {
      const int side = (j <= P - 1) ? 0 : 1;
      const int r = side ? (ny - 1 - j) : j;
      const float b = S.cpml[(side ? kBeY2 : kBeY1) * P + r];
      const float cc = S.cpml[(side ? kCeY2 : kCeY1) * P + r];
      const int64_t po = S.o_ezy + ((int64_t)side * P + r) * pitch + ic;
      if (!kHoist) ldf4<kCoh>(psi_y, psr + po);
      float pn[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int c = i + k;
        pn[k] = psi_y[k];
        if (c >= 1 && c <= nx - 2 && covered<MEDIUM>(S, kCovEzPmlJ, (long long)(r - 1) * (nx - 2) + (c - 1))) {
          pn[k] = upd_psi(b, psi_y[k], cc, hxp[k], hxn[k]);
          ezw4[k] = __fmaf_rn(m.cB(k), pn[k], ezw4[k]);
        }
      }
      st4(psw + po, pn);
    }

    // ---- sources, then detectors, of this row (Dev_AESASourceCalc,
    //      Dev_AESADetectorSim, Dev_AESAComponentDetector)
    const int p0 = __ldg(S.row_start + j), p1 = __ldg(S.row_start + j + 1);
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
      st4(hxw + o, hxn);
      st4(hyw + o, hyn);
      st4(ezw + o, ezw4);
      st4(jzw + o, jzw4);
    }

    // roll
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hxp[k] = hxn[k];
      ezc[k] = ezn[k];
      ezn[k] = ezn2[k]; hxo[k] = hxo2[k]; hyo[k] = hyo2[k]; jzo[k] = jzo2[k];
    }
  }
}

// The shot descriptor is a __grid_constant__ parameter: its fields are read
// through the constant cache and need no reload after the kernel's stores.
template <int MEDIUM>
__global__ void __launch_bounds__(kThreads, 2)
step_stream_kernel(const __grid_constant__ DevShot S, const int4* __restrict__ units, int n_units,
                   int n_global) {
  __shared__ MatE s_mat_e[MEDIUM ? 256 : 1];
  __shared__ MatH s_mat_h[MEDIUM ? 256 : 1];
  if (MEDIUM) {
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
      s_mat_e[t] = S.mat_e[t];
      s_mat_h[t] = S.mat_h[t];
    }
    __syncthreads();
  }
  const int n = n_global - S.base_n;
  if (n < 1 || n > S.n_steps) return;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int u = warp; u < n_units; u += n_warps) {
    const int4 ud = __ldg(units + u);
    process_unit<MEDIUM>(S, s_mat_e, s_mat_h, ud.y, ud.z, ud.w, n, lane);
  }
}

cudaError_t launch_step(const DevShot& shot, const int4* units, int n_units, int n_global, int medium,
                        int n_warps_grid, cudaStream_t stream) {
  const int warps = n_warps_grid < n_units ? n_warps_grid : n_units;
  const int blocks = (warps * 32 + kThreads - 1) / kThreads;
  if (blocks <= 0) return cudaSuccess;
  if (medium == 0) {
    step_stream_kernel<0><<<blocks, kThreads, 0, stream>>>(shot, units, n_units, n_global);
  } else {
    step_stream_kernel<1><<<blocks, kThreads, 0, stream>>>(shot, units, n_units, n_global);
  }
  return cudaGetLastError();
}

// ---- persistent form: many steps per cooperative launch ------------------

// Grid-wide barrier of a cooperative launch.  Thread 0 of each CTA releases
// the CTA's writes, adds one to *count and waits until the count reaches
// `target` (every CTA has arrived), for at most wait_ns, or until another
// CTA has set *err.  False when the barrier did not complete.
__device__ bool grid_barrier(unsigned* count, unsigned target, int* err, uint64_t wait_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(count, 1u);
    int ok = 1;
    const uint64_t t0 = global_ns();
    for (;;) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
      if (v >= target) break;
      if (*(volatile int*)err != kErrNone) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > wait_ns) {
        atomicExch(err, kErrWaitTimeout);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// One wave-front tracker line of one step with one warp: rc_kernel's
// outputs (the column maximum from row j_cut with row 0 as the start, the
// edge level kept as a running maximum, the deepest row in [1, ny-3] at or
// above it), from L2.
__device__ void rc_warp(const float* ez, int64_t pitch, int ny, int is, int im, int j_cut, float level, float* edge,
                        int* spd, int lane) {
  float m = -INFINITY;
  for (int j = j_cut + lane; j < ny - 2; j += 32) m = fmaxf(m, __ldcg(ez + (int64_t)j * pitch + im));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  float e = 0.f;
  if (lane == 0) {
    float temp = __ldcg(ez + im);
    if (m > temp) temp = m;
    const float cand = temp * level;
    e = *edge;
    if (cand > e) e = cand;
    *edge = e;
  }
  e = __shfl_sync(0xffffffffu, e, 0);
  int best = 0;
  for (int j = 1 + lane; j <= ny - 3; j += 32)
    if (!(fabsf(__ldcg(ez + (int64_t)j * pitch + is)) < e)) best = j;
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if (lane == 0) *spd = best;
}

// Service warp k's work after step n (global) of a single shot: tracker
// line k, or (k == n_rc) the line probe's row.
__device__ void persist_service(const DevShot& S, const PersistAux& A, int n, int k, int lane) {
  const float* ez = field_ptr(S, kEz, (n - S.base_n) & 1);
  if (k < A.n_rc) {
    rc_warp(ez, S.pitch, S.ny, __ldg(A.scan_i + k), __ldg(A.max_i + k), A.j_cut, A.level, A.edge + k,
            A.spd + (int64_t)(n - 1) * A.n_rc + k, lane);
  } else if (n >= A.line_first && n <= A.line_last) {
    float* dst = A.line + (int64_t)(n - A.line_first) * A.line_n;
    const float* src = ez + (int64_t)A.line_j * S.pitch + A.line_i0;
    for (int t = lane; t < A.line_n; t += 32) dst[t] = __ldcg(src + t);
  }
}

// Steps n_first..n_last of one shot in one launch.  Warps [0, n_work) step
// the units (the same unit to the same warp every step, so a detector's DFT
// sum is always the same thread's); the last warps serve step n (tracker,
// line probe) while the others run step n+1, which writes the other buffer.
// Every mutable array is read from L2 (process_unit<M, true>), the grid
// barrier orders the steps, and the arithmetic is step_stream_kernel's, so
// the results are its bits.
template <int MEDIUM>
__global__ void __launch_bounds__(kThreads, 2)
step_persist_kernel(const __grid_constant__ DevShot S, const int4* __restrict__ units, int n_units, int n_first,
                    int n_last, int repeat, const __grid_constant__ PersistAux A, unsigned* bar, int* err) {
  __shared__ MatE s_mat_e[MEDIUM ? 256 : 1];
  __shared__ MatH s_mat_h[MEDIUM ? 256 : 1];
  if (MEDIUM) {
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
      s_mat_e[t] = S.mat_e[t];
      s_mat_h[t] = S.mat_h[t];
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
  const int n_work = n_warps - A.n_rc - (A.line_n > 0 ? 1 : 0);
  const int steps = repeat > 0 ? repeat : n_last - n_first + 1;
  const uint64_t wait_ns = A.wait_ns ? A.wait_ns : kWaitNs;
  unsigned target = 0;
  for (int s = 0; s <= steps; ++s) {
    if (warp < n_work) {
      const int nl = (repeat > 0 ? n_first : n_first + s) - S.base_n;
      if (s < steps && nl >= 1 && nl <= S.n_steps)
        for (int u = warp; u < n_units; u += n_work) {
          const int4 ud = __ldg(units + u);
          process_unit<MEDIUM, true>(S, s_mat_e, s_mat_h, ud.y, ud.z, ud.w, nl, lane);
        }
    } else if (s > 0 && repeat == 0) {
      persist_service(S, A, n_first + s - 1, warp - n_work, lane);
    }
    if (s == steps) break;
    target += gridDim.x;
    if (!grid_barrier(bar, target + A.bar_extra, err, wait_ns)) return;
  }
}

cudaError_t launch_step_persist(const DevShot& shot, const int4* units, int n_units, int n_first, int n_last,
                                int repeat, const PersistAux& aux, int medium, int ctas, unsigned* bar, int* err,
                                cudaStream_t stream) {
  if (ctas <= 0 || ctas * (kThreads / 32) <= aux.n_rc + (aux.line_n > 0 ? 1 : 0)) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  DevShot s = shot;
  PersistAux a = aux;
  void* args[] = {&s, (void*)&units, &n_units, &n_first, &n_last, &repeat, &a, &bar, &err};
  const void* fn = medium == 0 ? (const void*)step_persist_kernel<0> : (const void*)step_persist_kernel<1>;
  return cudaLaunchCooperativeKernel(fn, dim3(ctas), dim3(kThreads), args, 0, stream);
}

int persist_resident_ctas(int medium, int device) {
  int sms = 0, per_sm = 0, coop = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) return 0;
  if (medium == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_persist_kernel<0>, kThreads, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_persist_kernel<1>, kThreads, 0);
  }
  return sms * per_sm;
}

int resident_warps(int medium, int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (medium == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_stream_kernel<0>, kThreads, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_stream_kernel<1>, kThreads, 0);
  }
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm * (kThreads / 32);
}

// Source waveform, FDTD_2D_Full/kernel.cu:653 and Dev_calculateChirp
// (:694-698) with p = 1: amp[n]/N * cos(2*pi_c*(beta/2*t^2 + f0*t + phi/360)).
// Computed in FP64 with t = n*dt in FP64 (the reference forms t and the phase
// sum in FP32).  With pi_c = pi the phase is reduced modulo one cycle first.
__global__ void source_table_kernel(float* src_val, double2* twiddle, const float* env,
                                    const double* phase, int n_src, int n_steps, double dt,
                                    double scale, double f0, double beta_half, double src_pi,
                                    int exact_pi, double dft_fdt) {
  const int64_t total = (int64_t)(n_steps + 1) * n_src;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / n_src);
    const int e = (int)(t % n_src);
    const double tt = (double)n * dt;
    const double x = beta_half * tt * tt + f0 * tt + phase[e];
    const double cs = exact_pi ? cospi(2.0 * (x - floor(x))) : cos(2.0 * src_pi * x);
    src_val[t] = (float)(scale * (double)env[n] * cs);
  }
  if (twiddle) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n <= n_steps; n += gridDim.x * blockDim.x) {
      double ph = dft_fdt * (double)n;
      ph -= floor(ph);
      double sn, cs;
      sincospi(2.0 * ph, &sn, &cs);
      twiddle[n] = make_double2(cs, sn);
    }
  }
}

cudaError_t build_source_tables(float* src_val, double2* twiddle, const float* env,
                                const double* phase_cycles, int n_src, int n_steps, double dt,
                                double scale, double f0, double beta_half, double src_pi,
                                double dft_fdt, cudaStream_t stream) {
  const int exact = (src_pi == 3.14159265358979323846) ? 1 : 0;
  source_table_kernel<<<256, 256, 0, stream>>>(src_val, twiddle, env, phase_cycles, n_src, n_steps,
                                               dt, scale, f0, beta_half, src_pi, exact, dft_fdt);
  return cudaGetLastError();
}

// Dev_RCcalc (FDTD_2D_Full/kernel.cu:968-1044) as one CTA per line.  The
// reference walks each column serially with one thread (O(ny) dependent
// loads); here the column max and the downward scan are block reductions.
// The scan result is the largest j in [1, ny-3] where |Ez| is not below the
// edge level, which is where the reference's do-while from j = ny-2 stops.
__global__ void __launch_bounds__(1024) rc_kernel(const float* __restrict__ ez, int64_t pitch, int ny,
                                                  const int* __restrict__ scan_i, const int* __restrict__ max_i,
                                                  int j_cut, float level, float* __restrict__ edge,
                                                  int* __restrict__ spd_row) {
  constexpr int kPer = 8;   // scan-column rows a thread holds while the column max is formed
  __shared__ float s_max[32];
  __shared__ int s_best[32];
  __shared__ float s_edge;
  const int l = blockIdx.x;
  const int im = max_i[l], is = scan_i[l];
  const int tid = threadIdx.x, T = blockDim.x;
  const int lane = tid & 31, w = tid >> 5, nw = T >> 5;
  // The scan column's first kPer*T rows are loaded beside the max column, so
  // both columns' loads are in flight together.
  float sv[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int j = 1 + tid + k * T;
    sv[k] = j <= ny - 3 ? fabsf(ez[(int64_t)j * pitch + is]) : 0.f;
  }
  float m = -INFINITY;
#pragma unroll 4
  for (int j = j_cut + tid; j < ny - 2; j += T) m = fmaxf(m, ez[(int64_t)j * pitch + im]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) s_max[w] = m;
  __syncthreads();
  if (tid == 0) {
    float temp = ez[im];  // Dev_FindMax starts from row 0
    for (int k = 0; k < nw; ++k)
      if (s_max[k] > temp) temp = s_max[k];
    const float cand = temp * level;
    float e = edge[l];
    if (cand > e) e = cand;
    edge[l] = e;
    s_edge = e;
  }
  __syncthreads();
  const float e = s_edge;
  int best = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int j = 1 + tid + k * T;
    if (j <= ny - 3 && !(sv[k] < e)) best = max(best, j);
  }
  for (int j = 1 + tid + kPer * T; j <= ny - 3; j += T)
    if (!(fabsf(ez[(int64_t)j * pitch + is]) < e)) best = max(best, j);
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if (lane == 0) s_best[w] = best;
  __syncthreads();
  if (tid == 0) {
    int b = 0;
    for (int k = 0; k < nw; ++k) b = max(b, s_best[k]);
    spd_row[l] = b;
  }
}

cudaError_t launch_rc(const float* ez, int64_t pitch, int ny, int n_rc, const int* scan_i,
                      const int* max_i, int j_cut, float level, float* edge, int* spd_row,
                      cudaStream_t stream) {
  rc_kernel<<<n_rc, 1024, 0, stream>>>(ez, pitch, ny, scan_i, max_i, j_cut, level, edge, spd_row);
  return cudaGetLastError();
}

__global__ void line_kernel(const float* __restrict__ ez, int64_t pitch, int j, int i0, int n,
                            float* __restrict__ dst) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    dst[t] = ez[(int64_t)j * pitch + i0 + t];
}

cudaError_t launch_line(const float* ez, int64_t pitch, int j, int i0, int n, float* dst,
                        cudaStream_t stream) {
  line_kernel<<<(n + 255) / 256, 256, 0, stream>>>(ez, pitch, j, i0, n, dst);
  return cudaGetLastError();
}

__global__ void nonfinite_kernel(const float* __restrict__ a, int64_t n, int* flag) {
  int bad = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    bad |= !isfinite(a[t]);
  }
  bad = __syncthreads_or(bad);
  if (bad && threadIdx.x == 0) atomicAdd(flag, 1);
}

cudaError_t launch_nonfinite(const float* a, int64_t n, int* flag, cudaStream_t stream) {
  nonfinite_kernel<<<1024, 256, 0, stream>>>(a, n, flag);
  return cudaGetLastError();
}

// 16-bit storage: an element is Inf/NaN when its exponent bits are all ones
// (FP16: 0x7C00, BF16: 0x7F80).
__global__ void nonfinite16_kernel(const uint16_t* __restrict__ a, int64_t n, uint16_t mask, int* flag) {
  int bad = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    bad |= (a[t] & mask) == mask;
  }
  bad = __syncthreads_or(bad);
  if (bad && threadIdx.x == 0) atomicAdd(flag, 1);
}

cudaError_t launch_nonfinite16(const uint16_t* a, int64_t n, bool bf16, int* flag, cudaStream_t stream) {
  nonfinite16_kernel<<<1024, 256, 0, stream>>>(a, n, bf16 ? 0x7F80 : 0x7C00, flag);
  return cudaGetLastError();
}

// FP32 values to the storage type: dst[t] = src[t] * isc, rounded to nearest.
__global__ void to_half_kernel(const float* __restrict__ src, __half* __restrict__ dst, int64_t n, float isc) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = __float2half_rn(src[t] * isc);
}
__global__ void to_bf16_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int64_t n,
                               float isc) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = __float2bfloat16_rn(src[t] * isc);
}

cudaError_t launch_to_storage(const float* src, void* dst, int64_t n, int store, float isc, cudaStream_t stream) {
  if (store == 1)
    to_half_kernel<<<1024, 256, 0, stream>>>(src, static_cast<__half*>(dst), n, isc);
  else
    to_bf16_kernel<<<1024, 256, 0, stream>>>(src, static_cast<__nv_bfloat16*>(dst), n, isc);
  return cudaGetLastError();
}

}  // namespace fdtd2d
