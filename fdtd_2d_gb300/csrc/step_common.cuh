// Device helpers shared by the fused step kernels (step_kernels.cu,
// step_tma.cu): the update formulas with explicit rounding, per-cell medium
// coefficients, and the scalar/row paths that recompute halo H values.
#pragma once

#include "internal.h"

namespace fdtd2d {

// ---- update formulas (shared by the vector and the scalar paths) ----------

// Hx = DA*Hx + DB*((Ez_a - Ez_b)*den)        FDTD_2D_Full/kernel.cu:192-193, 313-314
__device__ __forceinline__ float upd_h(float da, float h, float db, float ea, float eb, float den) {
  return __fmaf_rn(db, __fmul_rn(__fsub_rn(ea, eb), den), __fmul_rn(da, h));
}

// psi = b*psi + c*(a - b')/d                  FDTD_2D_Full/kernel.cu:226-227, 478-479
// with cd = c/d folded on the host (the device CPML table holds c/d): an
// IEEE divide per CPML cell takes its slow path whenever the numerator is
// zero or subnormal (fields not yet arrived in the layer), which made the
// CPML bands several times slower than the bulk.  Folding moves each psi by
// at most a couple of FP32 ulps against the reference's c*(a-b')/d.
__device__ __forceinline__ float upd_psi(float b, float psi, float cd, float a, float a2) {
  return __fmaf_rn(b, psi, __fmul_rn(cd, __fsub_rn(a, a2)));
}

// Ez = CA*Ez + CB*(dHy*den_ex + dHx*den_ey - Jz)   FDTD_2D_Full/kernel.cu:444-446
__device__ __forceinline__ float upd_e(float ca, float e, float cb, float dhy, float dex,
                                       float dhx, float dey, float jz) {
  const float curl = __fsub_rn(__fmaf_rn(dhy, dex, __fmul_rn(dhx, dey)), jz);
  return __fmaf_rn(cb, curl, __fmul_rn(ca, e));
}

// upd_e on values in stored units: Ez/sE, H/sH, Jz/sJ, with cb_s = cb*sH/sE
// and rj = sJ/sH.  The scales are powers of two, so in the normal range each
// rounding here is the FP32 rounding above times an exact power of two; rj*Jz
// is exact, so the fma gives the subtraction's bits.  The result is upd_e's
// value divided by sE, bit for bit (with unit scales the two are identical).
__device__ __forceinline__ float upd_es(float ca, float e, float cb_s, float dhy, float dex, float dhx, float dey,
                                        float jz, float rj) {
  const float curl = __fmaf_rn(-rj, jz, __fmaf_rn(dhy, dex, __fmul_rn(dhx, dey)));
  return __fmaf_rn(cb_s, curl, __fmul_rn(ca, e));
}

// Jz = ja*Jz + kp*Ez where the cell carries plasma (kp != 0), else unchanged.
// At nu = 0, ja = 1 and kp = (e^2/m_e)*ne*dt: the reference's
// Jz + D_CJ*Ez*NE*dt (FDTD_2D_Full/kernel.cu:156-157).
__device__ __forceinline__ float upd_j(float ja, float jz, float kp, float ez) {
  return kp != 0.f ? __fmaf_rn(kp, ez, __fmul_rn(ja, jz)) : jz;
}

__device__ __forceinline__ void ld4(float (&d)[4], const float* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}
__device__ __forceinline__ void ld4_nc(float (&d)[4], const float* p) {
  // Streaming load of data read exactly once this step.
  const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
  d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}
// Loads of arrays a launch also writes (fields, psi).  kCoh false: through
// the read-only path (ldf4) or streaming (ldfs4), for kernels that run one
// step.  kCoh true: from L2, the point of coherence, because the array may
// have been written earlier in the same launch by another CTA (the
// persistent kernel's later steps); a read-only or L1-cached copy could be
// stale there.
template <bool kCoh>
__device__ __forceinline__ void ldf4(float (&d)[4], const float* p) {
  if constexpr (kCoh) {
    const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
  } else {
    ld4(d, p);
  }
}
template <bool kCoh>
__device__ __forceinline__ void ldfs4(float (&d)[4], const float* p) {
  if constexpr (kCoh) {
    ldf4<true>(d, p);
  } else {
    ld4_nc(d, p);
  }
}
template <bool kCoh>
__device__ __forceinline__ float ldf1(const float* p) {
  if constexpr (kCoh) {
    return __ldcg(p);
  } else {
    return *p;
  }
}
__device__ __forceinline__ void st4(float* p, const float (&d)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(d[0], d[1], d[2], d[3]);
}
__device__ __forceinline__ void zero4(float (&d)[4]) { d[0] = d[1] = d[2] = d[3] = 0.f; }

// Per-cell coefficients of one 4-cell row segment.  The uniform medium keeps
// only the plasma drive per cell; everything else is a shot-wide scalar.
template <int MEDIUM>
struct MediumRow;

template <>
struct MediumRow<0> {
  float da, db, ca, cb;
  float kp[4];
  __device__ __forceinline__ float dax(int) const { return da; }
  __device__ __forceinline__ float dbx(int) const { return db; }
  __device__ __forceinline__ float day(int) const { return da; }
  __device__ __forceinline__ float dby(int) const { return db; }
  __device__ __forceinline__ float cA(int) const { return ca; }
  __device__ __forceinline__ float cB(int) const { return cb; }
  __device__ __forceinline__ bool pec(int) const { return false; }
  __device__ __forceinline__ void init(const DevShot& S) { da = S.da; db = S.db; ca = S.ca; cb = S.cb; }
  __device__ __forceinline__ void load(const DevShot& S, const MatE*, const MatH*, int64_t off) {
    if (S.kp) {
      ld4_nc(kp, S.kp + off);
    } else {
      zero4(kp);
    }
  }
};

template <>
struct MediumRow<1> {
  float da_x[4], db_x[4], da_y[4], db_y[4], ca[4], cb[4], kp[4];
  bool pe[4];
  __device__ __forceinline__ float dax(int k) const { return da_x[k]; }
  __device__ __forceinline__ float dbx(int k) const { return db_x[k]; }
  __device__ __forceinline__ float day(int k) const { return da_y[k]; }
  __device__ __forceinline__ float dby(int k) const { return db_y[k]; }
  __device__ __forceinline__ float cA(int k) const { return ca[k]; }
  __device__ __forceinline__ float cB(int k) const { return cb[k]; }
  __device__ __forceinline__ bool pec(int k) const { return pe[k]; }
  __device__ __forceinline__ void init(const DevShot&) {}
  __device__ __forceinline__ void load(const DevShot& S, const MatE* mat_e, const MatH* mat_h, int64_t off) {
    const uchar4 a = *reinterpret_cast<const uchar4*>(S.id1 + off);
    const uchar4 b = *reinterpret_cast<const uchar4*>(S.id2 + off);
    const uchar4 c = *reinterpret_cast<const uchar4*>(S.id3 + off);
    const unsigned char ia[4] = {a.x, a.y, a.z, a.w};
    const unsigned char ib[4] = {b.x, b.y, b.z, b.w};
    const unsigned char ic[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const MatH hx = mat_h[ia[k]];
      const MatH hy = mat_h[ib[k]];
      const MatE e = mat_e[ic[k]];
      da_x[k] = hx.da; db_x[k] = hx.db;
      da_y[k] = hy.da; db_y[k] = hy.db;
      ca[k] = e.ca; cb[k] = e.cb; kp[k] = e.kp; pe[k] = e.pec != 0.f;
    }
  }
};

// Reference launch coverage (fdtd2d_setup.cover): only the material-ID
// kernel, which serves the Settings.ini path, carries the checks.
enum CoverKernel : int { kCovHx = 0, kCovHxPml, kCovHy, kCovHyPml, kCovJz, kCovEz, kCovEzPmlI, kCovEzPmlJ };

template <int MEDIUM>
__device__ __forceinline__ bool covered(const DevShot& S, int k, long long l) {
  return MEDIUM == 0 || l < S.cov[k];
}

// DB of one H cell (scalar path).
template <int MEDIUM>
__device__ __forceinline__ void h_coef(const DevShot& S, const MatH* mat_h, const uint8_t* ids,
                                       int64_t off, float& da, float& db) {
  if (MEDIUM == 0) {
    da = S.da; db = S.db;
  } else {
    const MatH h = mat_h[ids[off]];
    da = h.da; db = h.db;
  }
}

// New Hy at one cell (c, j) from old values (hyo: the old Hy there), CPML
// included.  Used for the lane-0 halo value Hy_new(i0-1, j).  Reads only the
// old buffers.
template <int MEDIUM, bool kCoh = false>
__device__ float hy_cell(const DevShot& S, const MatH* mat_h, int par, int c, int j,
                         float ez_c, float ez_c1, float hyo) {
  const int64_t off = (int64_t)j * S.pitch + c;
  float da, db;
  h_coef<MEDIUM>(S, mat_h, S.id2, off, da, db);
  float h = covered<MEDIUM>(S, kCovHy, (long long)j * (S.nx - 1) + c)
                ? upd_h(da, hyo, db, ez_c1, ez_c, S.den_hx[c]) : hyo;
  const int P = S.npml;
  int side = -1, r = 0;
  if (c <= P - 2) { side = 0; r = c; }
  else if (c >= S.nx - P && c <= S.nx - 2) { side = 1; r = S.nx - 2 - c; }
  if (side >= 0 && covered<MEDIUM>(S, kCovHyPml, (long long)j * (P - 1) + r)) {
    const float* tb = S.cpml + (side ? kBhX2 : kBhX1) * P;
    const float* tc = S.cpml + (side ? kChX2 : kChX1) * P;
    const float psi = ldf1<kCoh>(S.psi + par * S.psi_buf + S.o_hyx + ((int64_t)side * S.ny + j) * P + r);
    const float pn = upd_psi(tb[r], psi, tc[r], ez_c1, ez_c);
    h = __fmaf_rn(db, pn, h);
  }
  return h;
}

// One Hx row segment (i..i+3, j): bulk update + y-strip CPML.  `own` writes
// the new psi: only the owning unit does, and only from lanes that hold real
// columns (inactive lanes run with their address clamped to column 0).
template <int MEDIUM, bool kCoh = false>
__device__ __forceinline__ void hx_row(const DevShot& S, const MediumRow<MEDIUM>& m, int par, int i, int j, const float (&ezj)[4],
                                       const float (&ezj1)[4], const float (&hxo)[4],
                                       float (&out)[4], bool own) {
  const float den = S.den_hy[j];
  const int nx = S.nx;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    out[k] = (i + k <= nx - 2 && covered<MEDIUM>(S, kCovHx, (long long)j * (nx - 1) + i + k))
                 ? upd_h(m.dax(k), hxo[k], m.dbx(k), ezj[k], ezj1[k], den) : hxo[k];
  }
  const int P = S.npml;
  int side = -1, r = 0;
  if (j <= P - 2) { side = 0; r = j; }
  else if (j >= S.ny - P) { side = 1; r = S.ny - 2 - j; }
  if (side >= 0) {
    const float b = S.cpml[(side ? kBhY2 : kBhY1) * P + r];
    const float c = S.cpml[(side ? kChY2 : kChY1) * P + r];
    const int64_t poff = ((int64_t)side * (P - 1) + r) * S.pitch + i;
    float psi[4], pn[4];
    ldf4<kCoh>(psi, S.psi + par * S.psi_buf + poff);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      pn[k] = psi[k];
      if (i + k <= nx - 2 && covered<MEDIUM>(S, kCovHxPml, (long long)r * (nx - 1) + i + k)) {
        pn[k] = upd_psi(b, psi[k], c, ezj[k], ezj1[k]);
        out[k] = __fmaf_rn(m.dbx(k), pn[k], out[k]);
      }
    }
    if (own) st4(S.psi + (par ^ 1) * S.psi_buf + poff, pn);  // callers pass own = act
  }
}

}  // namespace fdtd2d
