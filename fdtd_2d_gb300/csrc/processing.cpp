// Host post-processing of the drop-in driver:
//
//  * wave-front ("RC") lines: RClineFilterPostTime, CalculateRCfromPwrLines and
//    CalculateTaufromPwrLines (FDTD_2D_Full/kernel.cu:3188-3270) ->
//    RC_Line.txt, TAU_Line.txt.  The per-step front positions come from the
//    GPU tracker (fdtd2d_read_rc).
//  * time-of-flight estimation on a saved Ez line: processing_core and its
//    filters/estimators (FDTD_2D_Full/processing.cu:6-300) -> SD.txt, CF.txt,
//    ARC.txt, det_*.txt, *_field.txt.
//
// Arithmetic and output formats follow the reference (FP32 accumulators,
// printf/iostream formats); the file names are those the reference writes in
// its working directory, here placed in the output directory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <new>
#include <string>
#include <vector>

#include "../../include/fdtd2d.h"
#include "problem.h"

namespace fdtd2d {
Problem* problem_internal(fdtd2d_problem* p);

namespace {

using Vec = std::vector<float>;
using Mat = std::vector<Vec>;

std::string path_in(const std::string& dir, const std::string& name) {
  return dir.empty() ? name : dir + "/" + name;
}

// moving_average (processing.cu:181-204): window sum, centred write, edges
// copied from the nearest filtered sample.
void moving_average(const Vec& src, Vec& dst, int win) {
  float buf = 0;
  const int half = win / 2;
  const int times = (int)src.size();
  for (int t = 0; t < win - 1 && t < times; t++) buf += src[t];
  for (int t = win - 1; t < times; t++) {
    buf += src[t];
    dst[t - half] = buf / win;
    buf -= src[t - win + 1];
  }
  for (int t = half; t > 0; t--) {
    if (half - 1 >= 0 && times - t >= 0 && times - half - 1 >= 0) {
      dst[t] = dst[half - 1];
      dst[times - t] = dst[times - half - 1];
    }
  }
}

// medfilt (processing.cu:206-229)
void medfilt(const Vec& src, Vec& dst, int win) {
  Vec buf, tmp;
  const int half = win / 2;
  const int times = (int)src.size();
  for (int t = 0; t < win - 1 && t < times; t++) buf.push_back(src[t]);
  for (int t = win - 1; t < times; t++) {
    buf.push_back(src[t]);
    tmp = buf;
    std::sort(tmp.begin(), tmp.end());
    dst[t - half] = tmp[half];
    buf.erase(buf.begin());
  }
  for (int t = half; t > 0; t--) {
    if (half - 1 >= 0 && times - half - 1 >= 0) {
      dst[t] = dst[half - 1];
      dst[times - t] = dst[times - half - 1];
    }
  }
}

// filter (processing.cu:146-179)
void filter(const Vec& src, Vec& dst, int type, int win, int iters) {
  Vec tmp = src;
  for (int i = 0; i < iters; i++) {
    if (type == 1) {
      moving_average(tmp, dst, win);
      tmp = dst;
    } else if (type == 2) {
      medfilt(tmp, dst, win);
      tmp = dst;
    }
  }
}

float vmax(const Vec& v) {
  if (v.empty()) return 0;
  float r = v[0];
  for (size_t i = 1; i < v.size(); i++)
    if (v[i] > r) r = v[i];
  return r;
}

// The second difference, 0 at both ends.  A TOF window that opens after the
// run's last step leaves no samples: then there is nothing to write (the
// reference indexes the empty vector there).
void sec_diff(const Vec& src, Vec& dst) {
  if (dst.empty()) return;
  dst[0] = dst[dst.size() - 1] = 0;
  for (size_t i = 1; i + 1 < src.size(); i++) dst[i] = src[i - 1] - 2 * src[i] + src[i + 1];
}

// sd_method (processing.cu:231-245): first sign change of the filtered second
// difference while the signal is above threshold.
int sd_method(const Vec& src, const IniParams& A) {
  Vec tmp1 = src, tmp2 = tmp1;
  const float min_level = (float)A.p_tau_threshold * vmax(src);
  sec_diff(src, tmp1);
  filter(tmp1, tmp2, A.p_sdf_type, A.p_sdf_win, A.p_sdf_runs);
  for (int i = 0; i < (int)src.size() - 1; i++)
    if (src[i] > min_level && tmp2[i] * tmp2[i + 1] < 0) return i;
  return (int)src.size() - 1;
}

// cf_method / arc_method (processing.cu:247-277): constant-fraction crossing.
int cf_like(const Vec& src, const IniParams& A, int tau, float k) {
  const float min_level = (float)A.p_tau_threshold * vmax(src);
  for (int t = 0; t < (int)src.size() - (tau + 1); t++) {
    if (src[t] > min_level) {
      const float p1 = src[t] + k * src[t + tau];
      const float p2 = src[t + 1] + k * src[t + tau + 1];
      if (p1 * p2 < 0) return t;
    }
  }
  return (int)src.size() - 1;
}

void write_vec(const std::string& f, const Vec& v, int sieve, int from, double dt) {
  FILE* out = std::fopen(f.c_str(), "w");
  if (!out) return;
  for (int i = 0; i < (int)v.size(); i += std::max(1, sieve))
    std::fprintf(out, "%d %lf %lf\n", from + i, (double)v[i], (dt * v[i]) * 1e12);
  std::fclose(out);
}

void write_mat(const std::string& f, const Mat& m, int t_sieve, int d_sieve) {
  FILE* out = std::fopen(f.c_str(), "w");
  if (!out) return;
  const int cols = (int)m.size();
  if (cols) {
    const int rows = (int)m[0].size();
    for (int t = 0; t < rows; t += std::max(1, t_sieve)) {
      for (int i = 0; i < cols; i += std::max(1, d_sieve)) std::fprintf(out, "%f\t", m[i][t]);
      std::fprintf(out, "\n");
    }
  }
  std::fclose(out);
}

}  // namespace

// processing_core (processing.cu:6-144).  field[t][i]: t over the saved steps.
int processing_run(const Problem& p, const std::vector<std::vector<float>>& field,
                   const std::string& dir) {
  const IniParams& A = p.ini;
  const double dt = p.s.dt;
  const int sz = A.p_size_i;
  const int times = (int)field.size();
  if (sz <= 0) return FDTD2D_OK;
  Mat source(sz, Vec(times)), filtered;
  for (int i = 0; i < sz; i++)
    for (int t = 0; t < times; t++) source[i][t] = std::fabs(field[t][i]);
  filtered = source;
  Vec sd(sz), cf(sz), arc(sz);
  for (int i = 0; i < sz; i++) {
    filter(source[i], filtered[i], A.p_filter_type, A.p_filter_win, A.p_filter_runs);
    if (A.p_sec_der) sd[i] = (float)(A.p_begin_after + sd_method(filtered[i], A));
    if (A.p_cf) cf[i] = (float)(A.p_begin_after + cf_like(filtered[i], A, A.p_cf_tau, (float)A.p_cf_k));
    if (A.p_arc) arc[i] = (float)(A.p_begin_after + cf_like(filtered[i], A, A.p_arc_tau, (float)A.p_arc_k));
  }
  if (A.p_save_original) write_mat(path_in(dir, "original_field.txt"), source, A.p_time_sieve, A.p_dim_sieve);
  if (A.p_save_filtered) write_mat(path_in(dir, "filtered_field.txt"), filtered, A.p_time_sieve, A.p_dim_sieve);
  if (A.p_sec_der) write_vec(path_in(dir, "SD.txt"), sd, A.p_dim_sieve, A.p_pos_i, dt);
  if (A.p_cf) write_vec(path_in(dir, "CF.txt"), cf, A.p_dim_sieve, A.p_pos_i, dt);
  if (A.p_arc) write_vec(path_in(dir, "ARC.txt"), arc, A.p_dim_sieve, A.p_pos_i, dt);

  if (A.p_sim_detect && A.p_size_i - A.p_detector_size > 0 && A.p_detector_size > 0) {
    const int nd = A.p_size_i - A.p_detector_size;
    Mat real(nd, Vec(times, 0));
    filtered = real;
    Vec w(A.p_detector_size, (float)(1.0 / A.p_detector_size));
    if (A.p_load_weights) {
      std::ifstream ist(path_in(dir, "DetWeights.txt"));
      for (int i = 0; ist && i < A.p_detector_size; i++) {
        if (!ist.eof()) {
          ist >> w[i];
        } else {
          w = Vec(A.p_detector_size, 1);
          break;
        }
      }
    }
    const int half = A.p_detector_size / 2;
    for (int t = 0; t < times; t++) {
      for (int i = 0; i < sz - A.p_detector_size; i++) {
        float buf = 0;
        for (int j = -half; j < A.p_detector_size - half; j++) buf += source[i + half + j][t] * w[j + half];
        real[i][t] = buf / A.p_detector_size;
      }
    }
    sd = Vec(nd);
    cf = sd;
    arc = sd;
    for (int i = 0; i < nd; i++) {
      filter(real[i], filtered[i], A.p_filter_type, A.p_filter_win, A.p_filter_runs);
      if (A.p_sec_der) sd[i] = (float)(A.p_begin_after + sd_method(filtered[i], A));
      if (A.p_cf) cf[i] = (float)(A.p_begin_after + cf_like(filtered[i], A, A.p_cf_tau, (float)A.p_cf_k));
      if (A.p_arc) arc[i] = (float)(A.p_begin_after + cf_like(filtered[i], A, A.p_arc_tau, (float)A.p_arc_k));
    }
    if (A.p_save_detector && A.p_save_original)
      write_mat(path_in(dir, "detector_original_field.txt"), real, A.p_time_sieve, A.p_dim_sieve);
    if (A.p_save_detector && A.p_save_filtered)
      write_mat(path_in(dir, "detector_filtered_field.txt"), filtered, A.p_time_sieve, A.p_dim_sieve);
    if (A.p_sec_der) write_vec(path_in(dir, "det_SD.txt"), sd, A.p_dim_sieve, A.p_pos_i + half, dt);
    if (A.p_cf) write_vec(path_in(dir, "det_CF.txt"), cf, A.p_dim_sieve, A.p_pos_i + half, dt);
    if (A.p_arc) write_vec(path_in(dir, "det_ARC.txt"), arc, A.p_dim_sieve, A.p_pos_i + half, dt);
  }
  return FDTD2D_OK;
}

// Wave-front post-processing.  spd[t][l] holds the tracker row for step t
// (row 0 = 0, as the reference's zero-initialised buffer).
int rc_post_write(const Problem& p, const std::vector<int>& spd, int nmax, int nl,
                  const std::string& dir) {
  const IniParams& A = p.ini;
  // RClineFilterPostTime (kernel.cu:3250-3270): moving average of width w
  // over samples j in (i - w/2, i + w/2], 0 < j < nMax, accumulated in FP32
  // from the top of the window down.  Lines are independent: one thread
  // each, every sum in the reference's order.
  std::vector<float> fl((size_t)nmax * nl, 0.f);
  const int w = A.rc_window;
  const float weight = (float)(1.0 / std::abs(w));
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < nl; k++) {
    int wb = w / 2, we = -w / 2;
    for (int i = 0; i < nmax; i++) {
      float acc = 0;
      for (int j = wb; j > we; j--)
        if (j > 0 && j < nmax) acc += (float)spd[(size_t)j * nl + k] * weight;
      fl[(size_t)i * nl + k] = acc;
      wb++;
      we++;
    }
  }
  {
    // CalculateRCfromPwrLines (kernel.cu:3188-3214)
    std::ofstream out(path_in(dir, "RC_Line.txt"));
    if (!out) return FDTD2D_ERR_IO;
    for (int k = 0; k < nl; k++) {
      int temp = 0;
      float ft = 0;
      for (int i = 0; i < nmax; i++)
        if (spd[(size_t)i * nl + k] > temp) temp = spd[(size_t)i * nl + k];
      for (int i = 0; i < nmax; i++)
        if (fl[(size_t)i * nl + k] > ft) ft = fl[(size_t)i * nl + k];
      out << temp << " " << ft << " " << ft * A.ds << std::endl;
    }
  }
  {
    // CalculateTaufromPwrLines (kernel.cu:3216-3248): first step after 2000
    // at which the filtered front stops advancing.
    std::ofstream out(path_in(dir, "TAU_Line.txt"));
    if (!out) return FDTD2D_ERR_IO;
    for (int k = 0; k < nl; k++) {
      float ft = 0;
      int i = 2000;
      do {
        ft = (float)(i * 2);
        i++;
      } while (i < nmax && (fl[(size_t)i * nl + k] - fl[(size_t)(i - 1) * nl + k] >= 0));
      out << ft << " " << ft * p.s.dt * 1e12 << std::endl;
    }
  }
  return FDTD2D_OK;
}

int rc_run_and_write(fdtd2d_ctx* ctx, const Problem& p, const std::string& dir, int32_t nmax,
                     std::vector<int>* spd_rows) {
  const int nl = p.s.n_rc;
  if (nl <= 0) return FDTD2D_OK;
  std::vector<int> dev((size_t)nmax * nl);
  int rc = fdtd2d_read_rc(ctx, 1, nmax, dev.data());
  if (rc) return rc;
  // Reference buffer row n holds step n; row 0 is never written.
  std::vector<int> spd((size_t)nmax * nl, 0);
  for (int n = 1; n < nmax; ++n)
    for (int k = 0; k < nl; ++k) spd[(size_t)n * nl + k] = dev[(size_t)(n - 1) * nl + k];
  if (spd_rows) *spd_rows = spd;
  return rc_post_write(p, spd, nmax, nl, dir);
}

}  // namespace fdtd2d

using namespace fdtd2d;

// No C++ exception leaves the C ABI: allocation failures become
// FDTD2D_ERR_NOMEM, anything else FDTD2D_ERR_INVALID.
template <class F>
static int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return FDTD2D_ERR_NOMEM;
  } catch (...) {
    return FDTD2D_ERR_INVALID;
  }
}

extern "C" int fdtd2d_write_rc_lines(const fdtd2d_problem* h, const int32_t* spd, int32_t n_rows,
                                     const char* out_dir) {
  Problem* p = problem_internal(const_cast<fdtd2d_problem*>(h));
  if (!p || !spd || n_rows < 1 || !p->from_ini) return FDTD2D_ERR_INVALID;
  const int nl = p->s.n_rc;
  if (nl <= 0) return FDTD2D_ERR_STATE;
  return guarded([&] {
    std::vector<int> rows(spd, spd + (size_t)n_rows * nl);
    return rc_post_write(*p, rows, n_rows, nl, out_dir ? out_dir : "");
  });
}

extern "C" int32_t fdtd2d_tof_width(const fdtd2d_problem* h) {
  const Problem* p = problem_internal(const_cast<fdtd2d_problem*>(h));
  return (p && p->from_ini) ? std::max(0, p->ini.p_size_i) : 0;
}

extern "C" int fdtd2d_write_tof(const fdtd2d_problem* h, const float* field, int32_t times,
                                const char* out_dir) {
  Problem* p = problem_internal(const_cast<fdtd2d_problem*>(h));
  if (!p || (!field && times > 0) || times < 0 || !p->from_ini) return FDTD2D_ERR_INVALID;
  if (!processing_params_ok(p->ini)) return FDTD2D_ERR_CONFIG;
  const int sz = p->ini.p_size_i;
  return guarded([&] {
    std::vector<std::vector<float>> f(times, std::vector<float>(std::max(0, sz)));
    for (int t = 0; t < times; ++t)
      for (int i = 0; i < sz; ++i) f[t][i] = field[(size_t)t * sz + i];
    return processing_run(*p, f, out_dir ? out_dir : "");
  });
}
