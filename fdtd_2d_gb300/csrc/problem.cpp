// Setup precompute for parameterised shots (fdtd2d_problem_from_spec) and the
// CPML/denominator tables shared with the Settings.ini path.
//
// CPML grading follows initializeCPML (FDTD_2D_Full/FDTD_cuda.cu:1224-1578):
// polynomial sigma and kappa of order m, alpha of order ma, at integer (E) and
// half-integer (H) depths, recursion coefficients b = exp(-(sigma/kappa +
// alpha) dt/eps0) and c = sigma (b-1) / (sigma + kappa alpha) / kappa.  The
// reference stores sigma, kappa and alpha in FP32 arrays before forming b and
// c; this file keeps that rounding so the tables match the reference's.
#include "problem.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

namespace fdtd2d {

namespace {

struct Grade {
  std::vector<float> sig, kap, alp, b, c;
};

// One strip side of E (integer depth) tables: npml entries.
Grade grade_e(int P, double sig_max, double kappa_max, double alpha_max, double m, double ma,
              double dt, double eps) {
  Grade g;
  g.sig.resize(P); g.kap.resize(P); g.alp.resize(P); g.b.resize(P); g.c.resize(P);
  for (int i = 0; i < P; ++i) {
    g.sig[i] = (float)(sig_max * std::pow((P - 1 - i) / (P - 1.0), m));
    g.alp[i] = (float)(alpha_max * std::pow((double)(float)i / (P - 1.0), ma));
    g.kap[i] = (float)(1.0 + (kappa_max - 1.0) * std::pow((P - 1 - i) / (P - 1.0), m));
    const float rate = g.sig[i] / g.kap[i] + g.alp[i];          // FP32 as in the reference
    g.b[i] = (float)std::exp(-(double)rate * dt / eps);
    if ((g.sig[i] == 0.f && g.alp[i] == 0.f && i == P - 1) || g.sig[i] + g.kap[i] * g.alp[i] == 0.f) {
      g.c[i] = 0.f;  // the second test only guards degenerate (sigma = alpha = 0) gradings
    } else {
      const float den = g.sig[i] + g.kap[i] * g.alp[i];
      g.c[i] = (float)((double)g.sig[i] * ((double)g.b[i] - 1.0) / (double)den / (double)g.kap[i]);
    }
  }
  return g;
}

// One strip side of H (half-integer depth) tables: npml-1 entries.
Grade grade_h(int P, double sig_max, double kappa_max, double alpha_max, double m, double ma,
              double dt, double eps) {
  Grade g;
  const int L = P - 1;
  g.sig.resize(L); g.kap.resize(L); g.alp.resize(L); g.b.resize(L); g.c.resize(L);
  for (int i = 0; i < L; ++i) {
    g.sig[i] = (float)(sig_max * std::pow((P - 1 - i - 0.5) / (P - 1.0), m));
    g.alp[i] = (float)(alpha_max * std::pow((i + 1 - 0.5) / (P - 1.0), ma));
    g.kap[i] = (float)(1.0 + (kappa_max - 1.0) * std::pow((P - 1 - i - 0.5) / (P - 1.0), m));
    const float rate = g.sig[i] / g.kap[i] + g.alp[i];
    g.b[i] = (float)std::exp(-(double)rate * dt / eps);
    const float den = g.sig[i] + g.kap[i] * g.alp[i];
    g.c[i] = den == 0.f ? 0.f
                        : (float)((double)g.sig[i] * ((double)g.b[i] - 1.0) / (double)den / (double)g.kap[i]);
  }
  return g;
}

// Denominators (FDTD_2D_Full/FDTD_cuda.cu:1466-1578).
void denominators(std::vector<float>& den_e, std::vector<float>& den_h, int n, int P, double d,
                  const Grade& e1, const Grade& e2, const Grade& h1, const Grade& h2) {
  den_h.assign(n - 1, 0.f);
  den_e.assign(n - 1, 0.f);
  int ii = P - 2;
  for (int i = 0; i < n - 1; ++i) {
    if (i < P - 1) {
      den_h[i] = (float)(1.0 / ((double)h1.kap[i] * d));
    } else if (i >= n - P) {
      den_h[i] = (float)(1.0 / ((double)h2.kap[ii] * d));
      ii = ii - 1;
    } else {
      den_h[i] = (float)(1.0 / d);
    }
  }
  ii = P - 1;
  for (int i = 0; i < n - 1; ++i) {
    if (i < P) {
      den_e[i] = (float)(1.0 / ((double)e1.kap[i] * d));
    } else if (i >= n - P) {
      den_e[i] = (float)(1.0 / ((double)e2.kap[ii] * d));
      ii = ii - 1;
    } else {
      den_e[i] = (float)(1.0 / d);
    }
  }
}

// Deterministic, platform-independent standard-normal-like samples: SplitMix64
// uniforms summed Irwin-Hall style (4 terms, rescaled to unit variance).  Only
// IEEE adds and multiplies, no libm, so x86 and Arm hosts draw the same field.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double normalish() {
    double a = uniform(), b = uniform(), c = uniform(), d = uniform();
    double sum = ((a + b) + (c + d)) - 2.0;
    return sum * 1.7320508075688772;  // sqrt(12/4)
  }
};

// Unit-variance Gaussian random field with correlation exp(-r^2/l^2): white
// noise convolved separably with exp(-d^2/(2 s^2)), s = l/2, truncated at 4s,
// normalised by the kernel's energy (so the variance is 1 in expectation).
void gaussian_random_field(std::vector<float>& g, int nx, int ny, double corr, uint64_t seed) {
  const double s = corr / 2.0;
  const int R = std::max(1, (int)std::ceil(4.0 * s));
  std::vector<double> k(2 * R + 1);
  double e2 = 0;
  for (int d = -R; d <= R; ++d) {
    k[d + R] = std::exp(-(double)d * d / (2.0 * s * s));
    e2 += k[d + R] * k[d + R];
  }
  const double norm = 1.0 / e2;  // two passes: variance scales by e2 each
  const int wx = nx + 2 * R, wy = ny + 2 * R;
  std::vector<float> w((size_t)wx * wy);
  // The generator is a counter (each output mixes seed + k * golden), and a
  // value takes four outputs: value t starts from seed + 4t * golden, so the
  // values are formed in parallel and equal the sequential stream's.
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < (int64_t)w.size(); ++t) {
    Rng rng(seed + (uint64_t)t * 4u * 0x9E3779B97F4A7C15ull);
    w[(size_t)t] = (float)rng.normalish();
  }
  std::vector<float> tmp((size_t)wx * ny);
  // Each output sums k[d] * input over d = 0 .. 2R in that order; the loops
  // run d outside and the columns inside (contiguous, vectorisable), one
  // accumulator per column, which keeps every output's order of additions.
  // pass 1: along y
#pragma omp parallel
  {
    std::vector<double> acc((size_t)wx);
#pragma omp for schedule(static)
    for (int j = 0; j < ny; ++j) {
      std::fill(acc.begin(), acc.end(), 0.0);
      for (int d = 0; d <= 2 * R; ++d) {
        const double kd = k[(size_t)d];
        const float* src = &w[(size_t)(j + d) * wx];
        for (int i = 0; i < wx; ++i) acc[(size_t)i] += kd * src[i];
      }
      for (int i = 0; i < wx; ++i) tmp[(size_t)j * wx + i] = (float)acc[(size_t)i];
    }
  }
  g.assign((size_t)nx * ny, 0.f);
  // pass 2: along x
#pragma omp parallel
  {
    std::vector<double> acc((size_t)nx);
#pragma omp for schedule(static)
    for (int j = 0; j < ny; ++j) {
      std::fill(acc.begin(), acc.end(), 0.0);
      const float* row = &tmp[(size_t)j * wx];
      for (int d = 0; d <= 2 * R; ++d) {
        const double kd = k[(size_t)d];
        for (int i = 0; i < nx; ++i) acc[(size_t)i] += kd * row[i + d];
      }
      for (int i = 0; i < nx; ++i) g[(size_t)j * nx + i] = (float)(acc[(size_t)i] * norm);
    }
  }
}

}  // namespace

void Problem::bind() {
  fdtd2d_setup& t = s;
  const float** rows[16] = {&t.be_x_1, &t.ce_x_1, &t.be_x_2, &t.ce_x_2, &t.bh_x_1, &t.ch_x_1,
                            &t.bh_x_2, &t.ch_x_2, &t.be_y_1, &t.ce_y_1, &t.be_y_2, &t.ce_y_2,
                            &t.bh_y_1, &t.ch_y_1, &t.bh_y_2, &t.ch_y_2};
  for (int r = 0; r < 16; ++r) *rows[r] = tab[r].data();
  t.den_ex = den_ex.data(); t.den_hx = den_hx.data();
  t.den_ey = den_ey.data(); t.den_hy = den_hy.data();
  t.ne = ne.empty() ? nullptr : ne.data();
  t.id1 = id1.empty() ? nullptr : id1.data();
  t.id2 = id2.empty() ? nullptr : id2.data();
  t.id3 = id3.empty() ? nullptr : id3.data();
  t.mat_ca = mat_ca.empty() ? nullptr : mat_ca.data();
  t.mat_cb = mat_cb.empty() ? nullptr : mat_cb.data();
  t.mat_da = mat_da.empty() ? nullptr : mat_da.data();
  t.mat_db = mat_db.empty() ? nullptr : mat_db.data();
  t.mat_ne = mat_ne.empty() ? nullptr : mat_ne.data();
  t.n_materials = (int32_t)mat_ca.size();
  t.n_src = (int32_t)src.size();
  t.src = src.empty() ? nullptr : src.data();
  t.src_phase_deg = src_phase.empty() ? nullptr : src_phase.data();
  t.envelope = envelope.empty() ? nullptr : envelope.data();
  t.n_det = (int32_t)det.size();
  t.det = det.empty() ? nullptr : det.data();
  t.n_comp = (int32_t)comp.size();
  t.comp = comp.empty() ? nullptr : comp.data();
  t.n_rc = (int32_t)rc_scan.size();
  t.rc_scan_i = rc_scan.empty() ? nullptr : rc_scan.data();
  t.rc_max_i = rc_max.empty() ? nullptr : rc_max.data();
}

void build_cpml(Problem& p, int nx, int ny, int P, double dx, double dy, double dt,
                double sigma_factor, double kappa_max, double alpha_max, double m, double ma) {
  const double eps = eps0();
  const double eta = std::sqrt(mu0() / (eps * 1.0));
  const double sx = sigma_factor * (0.8 * (m + 1) / (dx * eta));
  const double sy = sigma_factor * (0.8 * (m + 1) / (dy * eta));
  // Both sides of a direction share one grading (the reference computes
  // identical _1 and _2 tables).
  const Grade ex = grade_e(P, sx, kappa_max, alpha_max, m, ma, dt, eps);
  const Grade hx = grade_h(P, sx, kappa_max, alpha_max, m, ma, dt, eps);
  const Grade ey = grade_e(P, sy, kappa_max, alpha_max, m, ma, dt, eps);
  const Grade hy = grade_h(P, sy, kappa_max, alpha_max, m, ma, dt, eps);
  p.tab[0] = ex.b; p.tab[1] = ex.c; p.tab[2] = ex.b; p.tab[3] = ex.c;
  p.tab[4] = hx.b; p.tab[5] = hx.c; p.tab[6] = hx.b; p.tab[7] = hx.c;
  p.tab[8] = ey.b; p.tab[9] = ey.c; p.tab[10] = ey.b; p.tab[11] = ey.c;
  p.tab[12] = hy.b; p.tab[13] = hy.c; p.tab[14] = hy.b; p.tab[15] = hy.c;
  denominators(p.den_ex, p.den_hx, nx, P, dx, ex, ex, hx, hx);
  denominators(p.den_ey, p.den_hy, ny, P, dy, ey, ey, hy, hy);
  p.s.nx = nx; p.s.ny = ny; p.s.npml = P;
  p.s.dx = dx; p.s.dy = dy; p.s.dt = dt;
}

}  // namespace fdtd2d

using namespace fdtd2d;

struct fdtd2d_problem {
  Problem p;
};

extern "C" {

void fdtd2d_spec_defaults(fdtd2d_spec* sp) {
  if (!sp) return;
  std::memset(sp, 0, sizeof(*sp));
  // Plain 512^2 shot: dx = 0.5 mm, Courant 0.99 (2-D), 10-cell CPML graded with
  // m = 3, sigma_max = 0.8(m+1)/(eta0 dx), kappa_max = 5, alpha_max = 0.05;
  // linear plasma slab x in [256, 502] up to 3e19 m^-3, nu = 1e9 1/s; point
  // source at (40, 256), 30 GHz Gaussian-modulated sine, width 0.2 ns;
  // detector at (42, 256); 4000 steps.
  sp->nx = 512; sp->ny = 512; sp->npml = 10; sp->n_steps = 4000;
  // Courant 0.98, not 0.99: with the explicit Drude leapfrog the scheme is
  // stable only while (c dt)^2 (1/dx^2 + 1/dy^2) + (w_p dt / 2)^2 <= 1, and at
  // 3e19 m^-3 and dx = 0.5 mm that sum is 1.013 at Courant 0.99 (0.992 at 0.98).
  sp->dx = 0.5e-3; sp->dy = 0.5e-3; sp->courant = 0.98; sp->dt = 0;
  sp->cpml_m = 3; sp->cpml_ma = 1; sp->sigma_factor = 1.0; sp->kappa_max = 5; sp->alpha_max = 0.05;
  sp->profile = 1; sp->ne_peak = 3e19; sp->x_lo = 256; sp->x_hi = 502;
  sp->x_center = 256; sp->width = 60; sp->grf_rms = 0; sp->grf_corr = 40; sp->seed = 1001;
  sp->nu = 1e9;
  sp->n_elem = 1; sp->src_i = 40; sp->src_j = 256; sp->src_di = 0; sp->src_dj = 0;
  sp->freq = 30e9; sp->steer_deg = 0; sp->amp = 1.0;
  sp->pulse = 0; sp->pulse_width = 0.2e-9; sp->pulse_t0 = 0;
  sp->n_det = 1; sp->det_i = 42; sp->det_j = 256; sp->det_di = 0; sp->det_dj = 0;
  sp->record_traces = 1; sp->dft_freq = 0; sp->storage = FDTD2D_STORE_F32;
}

static int problem_from_spec_try(const fdtd2d_spec* sp, fdtd2d_problem** out) {
  std::unique_ptr<fdtd2d_problem> pr(new fdtd2d_problem());
  Problem& p = pr->p;
  const int nx = sp->nx, ny = sp->ny;
  double dt = sp->dt;
  if (!(dt > 0)) dt = sp->courant / (kC0 * std::sqrt(1.0 / (sp->dx * sp->dx) + 1.0 / (sp->dy * sp->dy)));
  build_cpml(p, nx, ny, sp->npml, sp->dx, sp->dy, dt, sp->sigma_factor, sp->kappa_max,
             sp->alpha_max, sp->cpml_m, sp->cpml_ma);
  p.s.n_steps = sp->n_steps;
  p.s.medium = FDTD2D_MEDIUM_UNIFORM;
  p.s.ca = 1.0f;
  p.s.cb = (float)(dt / eps0());
  p.s.da = 1.0f;
  p.s.db = (float)(dt / mu0());
  p.s.nu = sp->nu;
  p.s.jz_coef = (double)(float)kElectronDrive;

  // plasma density at Ez cells
  if (sp->profile != 0) {
    p.ne.assign((size_t)nx * ny, 0.f);
    std::vector<float> g;
    if (sp->profile == 3 && sp->grf_rms != 0) gaussian_random_field(g, nx, ny, sp->grf_corr, sp->seed);
    // the profile depends on the column only
    std::vector<double> col((size_t)nx, 0.0);
    for (int i = 0; i < nx; ++i) {
      if (sp->profile == 1) {
        if (i >= sp->x_lo && i <= sp->x_hi && sp->x_hi > sp->x_lo)
          col[(size_t)i] = sp->ne_peak * (i - sp->x_lo) / (sp->x_hi - sp->x_lo);
      } else {
        col[(size_t)i] = 0.5 * sp->ne_peak * (1.0 + std::tanh((i - sp->x_center) / sp->width));
      }
    }
    const bool grf = sp->profile == 3 && !g.empty();
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j) {
      for (int i = 0; i < nx; ++i) {
        double n = col[(size_t)i];
        if (grf) n *= 1.0 + sp->grf_rms * g[(size_t)j * nx + i];
        p.ne[(size_t)j * nx + i] = (float)std::max(0.0, n);
      }
    }
  }

  // phased array: element e at (src_i + e di, src_j + e dj); steering phase
  // -360 * pitch * sin(theta) / lambda per element, on top of the reference's
  // 90 degree offset (cos(wt + 90) = -sin(wt); Ez -= s gives +sin injection).
  const double lambda = kC0 / sp->freq;
  const double pitch_m = std::sqrt(std::pow(sp->src_di * sp->dx, 2) + std::pow(sp->src_dj * sp->dy, 2));
  const double dphi = -360.0 * pitch_m * std::sin(sp->steer_deg * kPiExact / 180.0) / lambda;
  for (int e = 0; e < sp->n_elem; ++e) {
    p.src.push_back({sp->src_i + e * sp->src_di, sp->src_j + e * sp->src_dj});
    p.src_phase.push_back(90.0 + dphi * e);
  }
  p.envelope.assign(sp->n_steps + 1, 0.f);
  const double t0 = sp->pulse_t0 > 0 ? sp->pulse_t0 : 4.0 * sp->pulse_width;
  for (int n = 0; n <= sp->n_steps; ++n) {
    const double t = n * dt;
    double a;
    if (sp->pulse == 0) {
      const double u = (t - t0) / sp->pulse_width;
      a = std::exp(-u * u);
    } else {
      a = (t < sp->pulse_width) ? 0.5 * (1.0 - std::cos(kPiExact * t / sp->pulse_width)) : 1.0;
    }
    p.envelope[n] = (float)(sp->amp * a);
  }
  p.s.src_scale = 1.0;
  p.s.f0 = sp->freq;
  p.s.f1 = sp->freq;
  p.s.t1 = 1.0;
  p.s.src_pi = kPiExact;
  for (int e = 0; e < sp->n_det; ++e) p.det.push_back({sp->det_i + e * sp->det_di, sp->det_j + e * sp->det_dj});
  p.s.record_traces = sp->record_traces;
  p.s.dft_freq = sp->dft_freq > 0 ? sp->dft_freq : sp->freq;
  p.s.storage = sp->storage;
  p.s.field_max = sp->field_max;
  p.bind();
  *out = pr.release();
  return FDTD2D_OK;
}

int fdtd2d_problem_from_spec(const fdtd2d_spec* sp, fdtd2d_problem** out) {
  if (!sp || !out) return FDTD2D_ERR_INVALID;
  *out = nullptr;
  if (sp->nx < 8 || sp->ny < 8 || sp->npml < 2 || sp->n_steps < 1 || !(sp->dx > 0) || !(sp->dy > 0))
    return FDTD2D_ERR_INVALID;
  if (sp->n_elem < 0 || sp->n_det < 0) return FDTD2D_ERR_INVALID;
  // every real parameter finite, and the random field's correlation length
  // positive and within a few grid sizes (its kernel spans 4 half-lengths)
  const double reals[] = {sp->dx, sp->dy, sp->courant, sp->dt, sp->cpml_m, sp->cpml_ma, sp->sigma_factor,
                          sp->kappa_max, sp->alpha_max, sp->ne_peak, sp->x_lo, sp->x_hi, sp->x_center,
                          sp->width, sp->grf_rms, sp->grf_corr, sp->nu, sp->freq, sp->steer_deg, sp->amp,
                          sp->pulse_width, sp->pulse_t0, sp->dft_freq, sp->field_max};
  for (const double v : reals)
    if (!std::isfinite(v)) return FDTD2D_ERR_INVALID;
  if (sp->profile == 3 && sp->grf_rms != 0 &&
      !(sp->grf_corr > 0 && sp->grf_corr <= 4.0 * std::max(sp->nx, sp->ny)))
    return FDTD2D_ERR_INVALID;
  try {
    return problem_from_spec_try(sp, out);
  } catch (const std::bad_alloc&) {
    return FDTD2D_ERR_NOMEM;
  } catch (...) {
    return FDTD2D_ERR_INVALID;   // no C++ exception leaves the C ABI
  }
}

int fdtd2d_problem_from_ini(const char* path, fdtd2d_problem** out) {
  return fdtd2d::problem_from_ini_ex(path, true, out);
}

int fdtd2d_problem_from_ini_vacuum(const char* path, fdtd2d_problem** out) {
  return fdtd2d::problem_from_ini_ex(path, false, out);
}

const fdtd2d_setup* fdtd2d_problem_setup(const fdtd2d_problem* p) { return p ? &p->p.s : nullptr; }

void fdtd2d_problem_free(fdtd2d_problem* p) { delete p; }

}  // extern "C"

namespace fdtd2d {

namespace {
int problem_from_ini_try(const char* path, bool objects, fdtd2d_problem** out) {
  std::unique_ptr<fdtd2d_problem> pr(new fdtd2d_problem());
  std::string log;
  int rc = parse_ini(path, pr->p.ini, log);
  if (rc) return rc;
  ini_to_metric(pr->p.ini);
  rc = build_from_ini(pr->p.ini, pr->p, objects);
  if (rc) return rc;
  pr->p.bind();
  *out = pr.release();
  return FDTD2D_OK;
}
}  // namespace

int problem_from_ini_ex(const char* path, bool objects, fdtd2d_problem** out) {
  if (!path || !out) return FDTD2D_ERR_INVALID;
  *out = nullptr;
  try {
    return problem_from_ini_try(path, objects, out);
  } catch (const std::bad_alloc&) {
    return FDTD2D_ERR_NOMEM;
  } catch (...) {
    return FDTD2D_ERR_CONFIG;   // no C++ exception leaves the C ABI
  }
}

Problem* problem_internal(fdtd2d_problem* p) { return p ? &p->p : nullptr; }
}  // namespace fdtd2d
