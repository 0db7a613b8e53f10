// Host-code sanitizer harness (test infrastructure, built by
// tests/test_sanitize_cpu.py with -fsanitize=address,undefined): the problem
// builders (parameterised specs at edge sizes, Settings.ini files), the TOF
// and wave-front post-processing at window lengths around the filter
// width, and the oracle (FP64 and FP32).  Prints one line per case and
// "SANITIZE OK" at the end; a sanitizer report ends the run first.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/fdtd2d.h"

extern "C" {
struct oracle;
oracle* oracle_create(const fdtd2d_setup* s, int fp32);
void oracle_destroy(oracle* o);
int oracle_run(oracle* o, int n_first, int n_last);
int oracle_read_traces(oracle* o, int n0, int n1, float* det, float* cez, float* chx, float* chy);
int oracle_read_dft(oracle* o, double* re, double* im);
// The post-processing object also holds the driver's tracker read-out, which
// needs the CUDA library; not called here.
int fdtd2d_read_rc(fdtd2d_ctx*, int32_t, int32_t, int32_t*) { return FDTD2D_ERR_STATE; }
}

static int fails = 0;

static void run_oracle(const char* what, const fdtd2d_setup* s, int steps) {
  for (int fp32 = 0; fp32 < 2; ++fp32) {
    oracle* o = oracle_create(s, fp32);
    if (!o) {
      std::printf("%s: oracle_create failed\n", what);
      ++fails;
      return;
    }
    const size_t nd = s->n_det > 0 ? s->n_det : 1, nc = s->n_comp > 0 ? s->n_comp : 1;
    std::vector<float> det((size_t)steps * nd), cz((size_t)steps * nc), cx(cz.size()), cy(cz.size());
    std::vector<double> re(nd), im(nd);
    const int r0 = oracle_run(o, 1, steps);
    const int r1 = oracle_read_traces(o, 1, steps, det.data(), cz.data(), cx.data(), cy.data());
    const int r2 = oracle_read_dft(o, re.data(), im.data());
    std::printf("oracle %s fp32=%d: %d %d %d\n", what, fp32, r0, r1, r2);
    if (r0 || r1 || r2) ++fails;
    oracle_destroy(o);
  }
}

static void spec_case(const char* what, fdtd2d_spec s, int oracle_steps) {
  fdtd2d_problem* p = nullptr;
  const int rc = fdtd2d_problem_from_spec(&s, &p);
  std::printf("spec %s: %d\n", what, rc);
  if (rc) {
    ++fails;
    return;
  }
  if (oracle_steps > 0) run_oracle(what, fdtd2d_problem_setup(p), oracle_steps);
  fdtd2d_problem_free(p);
}

// A Settings.ini case.  FDTD2D_ERR_CONFIG is a clean refusal of a malformed
// file (the degenerate cases the test writes); any other error counts.
static void ini_case(const char* path) {
  fdtd2d_problem* p = nullptr;
  int rc = fdtd2d_problem_from_ini(path, &p);
  std::printf("ini %s: %d\n", path, rc);
  if (rc) {
    if (rc != FDTD2D_ERR_CONFIG) ++fails;
    return;
  }
  const fdtd2d_setup* s = fdtd2d_problem_setup(p);
  run_oracle(path, s, 12);
  const int w = fdtd2d_tof_width(p);
  for (int T : {0, 1, 5, 299, 300, 2500}) {
    std::vector<float> f((size_t)T * (w > 0 ? w : 1));
    for (int t = 0; t < T; ++t)
      for (int i = 0; i < w; ++i)
        f[(size_t)t * w + i] = std::sin(0.05f * t + 0.1f * i) * std::exp(-std::pow((t - 900) / 400.0, 2));
    rc = fdtd2d_write_tof(p, f.data(), T, "sanitize_out");
    std::printf("tof width %d times %d: %d\n", w, T, rc);
    if (rc && rc != FDTD2D_ERR_CONFIG) ++fails;
  }
  if (s->n_rc > 0) {
    for (int rows : {1, 2, 1999, 2001, 4000}) {
      std::vector<int32_t> spd((size_t)rows * s->n_rc);
      for (size_t k = 0; k < spd.size(); ++k) spd[k] = (int32_t)(k * 2654435761u % (unsigned)(s->ny - 3)) + 1;
      rc = fdtd2d_write_rc_lines(p, spd.data(), rows, "sanitize_out");
      std::printf("rc rows %d: %d\n", rows, rc);
      if (rc) ++fails;
    }
  }
  fdtd2d_problem_free(p);
}

int main(int argc, char** argv) {
  fdtd2d_spec s;
  fdtd2d_spec_defaults(&s);
  fdtd2d_spec t = s;
  t.nx = 96; t.ny = 80; t.npml = 10; t.src_i = 20; t.src_j = 40; t.det_i = 22; t.det_j = 40; t.x_lo = 48; t.x_hi = 94;
  spec_case("96x80 slab", t, 30);
  t.nx = 22; t.ny = 22; t.npml = 2; t.src_i = 5; t.src_j = 5; t.det_i = 6; t.det_j = 6; t.x_lo = 10; t.x_hi = 20;
  spec_case("22x22 P2", t, 30);
  t = s; t.nx = 23; t.ny = 9; t.npml = 3; t.profile = 3; t.grf_rms = 0.05; t.grf_corr = 40;
  t.src_i = 5; t.src_j = 4; t.det_i = 6; t.det_j = 4;
  spec_case("23x9 tanh x GRF corr 40", t, 0);
  t = s; t.profile = 3; t.grf_rms = 0.05; t.grf_corr = 0.5;
  spec_case("GRF corr 0.5", t, 0);
  t = s; t.profile = 2; t.width = 0;
  spec_case("tanh width 0", t, 0);
  t = s; t.n_elem = 0; t.n_det = 0;
  spec_case("no points", t, 0);
  t = s; t.storage = FDTD2D_STORE_F16; t.field_max = 0;
  spec_case("F16 scale estimate", t, 0);
  for (int a = 1; a < argc; ++a) ini_case(argv[a]);
  if (fails) {
    std::printf("SANITIZE FAILED %d\n", fails);
    return 1;
  }
  std::printf("SANITIZE OK\n");
  return 0;
}
