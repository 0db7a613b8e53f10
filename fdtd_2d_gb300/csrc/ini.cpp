// Settings.ini reader and the reference's setup chain for the drop-in path.
//
// Parsing follows the semantics of the inih parser the reference vendors
// (FDTD_2D_Full/INIlib/ini.c, INIReader.cpp): lines of at most 199 characters,
// ';' or '#' comment lines, inline ';' comments only after whitespace,
// "name = value" or "name : value", continuation lines for a value that
// start with whitespace, section/name keys compared case-insensitively, and
// integers parsed with base auto-detection (strtol base 0).  A file that
// cannot be opened is an error; a malformed line is not (readINIparam checks
// only ParseError() < 0, FDTD_2D_Full/FDTD_cuda.cu:30).
//
// The setup chain restates, in order, readINIparam (FDTD_cuda.cu:27-176),
// recuclParametersToMetric (:305-382), initialize/setUp (:443-1218),
// buildObject and its medium builders (:2602-2660, 3114-3378),
// buildSourceProfile (:3539-3655), calculate2Darrai/calculateDetect2Darrai
// (:3380-3490) and initializeCPML (:1224-1578), keeping the reference's
// integer truncations and FP32 storage.
#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "problem.h"

namespace fdtd2d {

namespace {

std::string lower(std::string s) {
  for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

char* rtrim(char* s) {
  char* p = s + std::strlen(s);
  while (p > s && std::isspace((unsigned char)p[-1])) *--p = '\0';
  return s;
}

char* ltrim(char* s) {
  while (*s && std::isspace((unsigned char)*s)) ++s;
  return s;
}

// First occurrence of `c`, or of a ';' that follows whitespace, or the end.
char* find_stop(char* s, char c) {
  bool ws = false;
  while (*s && *s != c && !(ws && *s == ';')) {
    ws = std::isspace((unsigned char)*s) != 0;
    ++s;
  }
  return s;
}

class Ini {
 public:
  int error = 0;
  std::map<std::string, std::string> kv;

  bool load(const char* path) {
    FILE* f = std::fopen(path, "r");
    if (!f) {
      error = -1;
      return false;
    }
    char line[200];
    char section[50] = "";
    char prev[50] = "";
    int lineno = 0;
    while (std::fgets(line, sizeof(line), f)) {
      ++lineno;
      char* start = line;
      if (lineno == 1 && (unsigned char)start[0] == 0xEF && (unsigned char)start[1] == 0xBB &&
          (unsigned char)start[2] == 0xBF)
        start += 3;
      start = ltrim(rtrim(start));
      if (*start == ';' || *start == '#') continue;
      if (*prev && *start && start > line) {
        add(section, prev, start);  // continuation of the previous value
        continue;
      }
      if (*start == '[') {
        char* end = find_stop(start + 1, ']');
        if (*end == ']') {
          *end = '\0';
          std::snprintf(section, sizeof(section), "%s", start + 1);
          prev[0] = '\0';
        } else if (!error) {
          error = lineno;
        }
        continue;
      }
      if (!*start) continue;
      char* end = find_stop(start, '=');
      if (*end != '=') end = find_stop(start, ':');
      if (*end == '=' || *end == ':') {
        *end = '\0';
        char* name = rtrim(start);
        char* value = ltrim(end + 1);
        char* stop = find_stop(value, '\0');
        if (*stop == ';') *stop = '\0';
        rtrim(value);
        std::snprintf(prev, sizeof(prev), "%s", name);
        add(section, name, value);
      } else if (!error) {
        error = lineno;
      }
    }
    std::fclose(f);
    return true;
  }

  void add(const char* section, const char* name, const char* value) {
    std::string& v = kv[lower(std::string(section) + "=" + name)];
    if (!v.empty()) v += "\n";
    v += value;
  }

  const std::string* find(const char* s, const char* n) const {
    auto it = kv.find(lower(std::string(s) + "=" + n));
    return it == kv.end() ? nullptr : &it->second;
  }

  long integer(const char* s, const char* n, long d) const {
    const std::string* v = find(s, n);
    if (!v) return d;
    char* end = nullptr;
    const long x = std::strtol(v->c_str(), &end, 0);
    return end > v->c_str() ? x : d;
  }

  double real(const char* s, const char* n, double d) const {
    const std::string* v = find(s, n);
    if (!v) return d;
    char* end = nullptr;
    const double x = std::strtod(v->c_str(), &end);
    return end > v->c_str() ? x : d;
  }

  bool boolean(const char* s, const char* n, bool d) const {
    const std::string* v = find(s, n);
    if (!v) return d;
    const std::string t = lower(*v);
    if (t == "true" || t == "yes" || t == "on" || t == "1") return true;
    if (t == "false" || t == "no" || t == "off" || t == "0") return false;
    return d;
  }
};

inline double f32(double x) { return (double)(float)x; }

// A double to int as the reference's x86 build converts it (cvttsd2si): the
// value truncated toward zero when it fits an int, else INT_MIN (NaN, the
// infinities and out-of-range values alike).  C++ leaves those cases
// undefined and Arm saturates them; degenerate Settings.ini values (a zero
// radius, a fractional power of a negative base) reach them.
inline int x86_int(double v) { return (v > -2147483649.0 && v < 2147483648.0) ? (int)v : INT_MIN; }

}  // namespace

int parse_ini(const char* path, IniParams& p, std::string& log) {
  Ini r;
  if (!r.load(path)) {
    log = "can't load Settings.ini";
    return FDTD2D_ERR_CONFIG;
  }
  // Defaults are the reference's Settings.cuh macros (FDTD_2D_Full/Settings.cuh).
  p.gpu_device = (int)r.integer("hardware", "GPU_device", 0);
  p.s2d = (int)r.integer("regimes", "SourceToDetect", 0);
  p.ds = r.real("grid", "ds", 1);
  p.dt_coef = r.real("grid", "dt_coef", 0.5);
  p.imax = (int)r.integer("grid", "Imax", 550);
  p.jmax = (int)r.integer("grid", "Jmax", 600);
  p.exp_time_key = r.integer("grid", "Use_Exp_time", 0) != 0 ? 1 : 0;  // stored in a bool
  p.n_max = (int)r.integer("grid", "Max_time", 10000);
  p.exp_time = r.real("grid", "Exp_time", 10);
  p.src_i = (int)r.integer("grid", "Isource", 300);
  p.src_j = (int)r.integer("grid", "Jsource", 20);
  p.src_k = 1;
  p.det_i = (int)r.integer("grid", "Idetect", 250);
  p.det_j = (int)r.integer("grid", "Jdetect", 30);
  p.det_k = 1;
  p.s_pi = (int)r.integer("AESA", "SIsize", 40);
  p.s_delta_auto = (int)r.integer("AESA", "SAutoDelta", 0);
  p.s_di = (int)r.integer("AESA", "SIdelta", 5);
  p.s_angle = f32(r.real("AESA", "SPAngle", 0));
  p.d_pi = (int)r.integer("AESA", "DIsize", 40);
  p.d_delta_auto = (int)r.integer("AESA", "SAutoDelta", 0);  // the reference reads SAutoDelta here too
  p.d_di = (int)r.integer("AESA", "DIdelta", 5);
  p.chirp = (int)r.integer("PulseParam", "Chirp", 0);
  p.freq_a = f32(r.real("PulseParam", "FreqA", 28));
  p.freq_b = f32(r.real("PulseParam", "FreqB", 30));
  p.fronts = (int)r.integer("PulseParam", "Fronts", 2000);
  p.plato = (int)r.integer("PulseParam", "Plato", 2000);
  p.fronts_ns = r.real("PulseParam", "Fronts_ns", 3);
  p.plato_ns = r.real("PulseParam", "Plato_ns", 3);
  p.amp = r.real("PulseParam", "Pulse_amp", 1000);
  p.save_from = (int)r.integer("2Dsave", "From", 0);
  p.save_to = (int)r.integer("2Dsave", "To", 40000);
  p.save_time_sieve = (int)r.integer("2Dsave", "TimeSieve", 240);
  p.save_grid_sieve = (int)r.integer("2Dsave", "GridSieve", 1);
  p.build_medium = (int)r.integer("medium", "Build", 0);
  p.med_i = (int)r.integer("medium", "Icen", 275);
  p.med_j = (int)r.integer("medium", "Jcen", 305);
  p.med_k = 1;
  p.sph_a = f32(r.real("medium", "A", 1));
  p.sph_b = f32(r.real("medium", "B", 1));
  p.sph_c = f32(r.real("medium", "C", 1));
  p.sph_p = (int)r.integer("medium", "P", 1);
  p.sph_q = (int)r.integer("medium", "Q", 1);
  p.sph_n = (int)r.integer("medium", "N", 1);
  p.eq_r = (int)r.integer("medium", "Radius", 50);
  p.eq_alpha = f32(r.real("medium", "Alpha", 2.0));
  p.eq_beta = f32(r.real("medium", "Beta", 1.0));
  p.eq_ne0 = f32(r.real("medium", "ne0", 1e19));
  p.eq_nea = f32(r.real("medium", "neA", 0));
  p.torus_br = (int)r.integer("medium", "TorusBR", 175);
  p.fluc_build = (int)r.integer("mediumFluc", "FlucBuild", 0);
  p.fluc_i = (int)r.integer("mediumFluc", "FlucIcen", 275);
  p.fluc_j = (int)r.integer("mediumFluc", "FlucJcen", 305);
  p.fluc_k = 1;
  p.fluc_a = f32(r.real("mediumFluc", "FlucA", 1));
  p.fluc_b = f32(r.real("mediumFluc", "FlucB", 1));
  p.fluc_c = f32(r.real("mediumFluc", "FlucC", 1));
  p.fluc_p = (int)r.integer("mediumFluc", "FlucP", 1);
  p.fluc_q = (int)r.integer("mediumFluc", "FlucQ", 1);
  p.fluc_n = (int)r.integer("mediumFluc", "FlucN", 1);
  p.fluc_angle_i = f32(r.real("mediumFluc", "FlucAngleI", 0));
  p.fluc_angle_j = f32(r.real("mediumFluc", "FlucAngleJ", 0));
  p.fluc_angle_k = f32(r.real("mediumFluc", "FlucAngleK", 0));
  p.fluc_sign = (int)r.integer("mediumFluc", "FlucSign", 1);
  p.fluc_r = (int)r.integer("mediumFluc", "FlucRadius", 10);
  p.fluc_alpha = f32(r.real("mediumFluc", "FlucAlpha", 2.0));
  p.fluc_beta = f32(r.real("mediumFluc", "FlucBeta", 1.0));
  p.fluc_ne0 = f32(r.real("mediumFluc", "FlucNe0", 1e19));
  p.draw2d = (int)r.integer("KameraConf", "Draw2D", 0);
  p.preset = (int)r.integer("KameraConf", "2Dpreset", 7);
  p.patrubok = (int)r.integer("KameraConf", "PatrubokL", 5);
  p.draw_wall = (int)r.integer("KameraConf", "DrawWall", 0);
  p.wall_pos = (int)r.integer("KameraConf", "WallPos", 950);
  p.rc_i = (int)r.integer("RC_calc", "Iline", 300);
  p.rc_size = (int)r.integer("RC_calc", "LIsize", 40);
  p.rc_delta = (int)r.integer("RC_calc", "LIdelta", 5);
  p.rc_level = f32(r.real("RC_calc", "Rlevel", 0.1));
  p.rc_window = (int)r.integer("RC_calc", "FilterWindow", 200);
  p.p_perform = r.boolean("Processing", "Perform", false);
  p.p_sec_der = r.boolean("Processing", "SecDer", false);
  p.p_cf = r.boolean("Processing", "CF", false);
  p.p_arc = r.boolean("Processing", "ARC", false);
  p.p_save_filtered = r.boolean("Processing", "SaveFiltered", false);
  p.p_save_original = r.boolean("Processing", "SaveOriginal", false);
  p.p_sim_detect = r.boolean("Processing", "DetSim", false);
  p.p_save_detector = r.boolean("Processing", "DetSave", false);
  p.p_load_weights = r.boolean("Processing", "DetWLoad", false);
  p.p_detector_size = (int)r.integer("Processing", "DetSize", 30);
  p.p_filter_type = (int)r.integer("Processing", "FilterType", 1);
  p.p_dim_sieve = (int)r.integer("Processing", "DimSieve", 1);
  p.p_time_sieve = (int)r.integer("Processing", "TimeSieve", 1);
  p.p_begin_after = (int)r.integer("Processing", "BeginAfter", 0);
  p.p_finish_at = (int)r.integer("Processing", "FinishAt", 0);
  p.p_pos_i = (int)r.integer("Processing", "PosI", 0);
  p.p_pos_j = (int)r.integer("Processing", "PosJ", 0);
  p.p_pos_k = (int)r.integer("Processing", "PosK", 0);
  p.p_size_i = (int)r.integer("Processing", "SizeI", 0);
  p.p_filter_win = (int)r.integer("Processing", "FilterWin", 300);
  p.p_filter_runs = (int)r.integer("Processing", "FilterRuns", 1);
  p.p_sdf_win = (int)r.integer("Processing", "SDFWin", p.p_filter_win);
  p.p_sdf_type = (int)r.integer("Processing", "SDFType", p.p_filter_type);
  p.p_sdf_runs = (int)r.integer("Processing", "SDFRuns", p.p_filter_runs);
  p.p_cf_tau = (int)r.integer("Processing", "CFTau", 300);
  p.p_arc_tau = (int)r.integer("Processing", "ARCTau", 300);
  p.p_tau_threshold = f32(r.real("Processing", "TauThreshold", 0));
  p.p_arc_k = f32(r.real("Processing", "ARCK", -0.5));
  p.p_cf_k = f32(r.real("Processing", "CFK", -0.5));
  if (r.error > 0) log = "Settings.ini: malformed line " + std::to_string(r.error) + " (ignored)";
  return FDTD2D_OK;
}

// recuclParametersToMetric (FDTD_2D_Full/FDTD_cuda.cu:305-382): millimetres to
// cells (int truncation of x*(1/ds)), the 3-D Courant dt, and step counts from
// nanoseconds when Use_Exp_time is set.
void ini_to_metric(IniParams& p) {
  const double inv = 1.0 / p.ds;
  p.dx = p.ds * 1E-3;
  p.dy = p.ds * 1E-3;
  p.dz = p.ds * 1E-3;
  p.imax = x86_int(p.imax * inv);
  p.jmax = x86_int(p.jmax * inv);
  p.src_i = x86_int(p.src_i * inv);
  p.src_j = x86_int(p.src_j * inv);
  p.det_i = x86_int(p.det_i * inv);
  p.det_j = x86_int(p.det_j * inv);
  p.med_i = x86_int(p.med_i * inv);
  p.med_j = x86_int(p.med_j * inv);
  p.med_k = 1;
  p.eq_r = x86_int(p.eq_r * inv);
  p.s_pi = x86_int(p.s_pi * inv);
  p.s_di = x86_int(p.s_di * inv);
  p.d_pi = x86_int(p.d_pi * inv);
  p.d_di = x86_int(p.d_di * inv);
  p.fluc_i = x86_int(p.fluc_i * inv);
  p.fluc_j = x86_int(p.fluc_j * inv);
  p.fluc_k = 1;
  p.fluc_r = x86_int(p.fluc_r * inv);
  p.dt = (0.99 / (kC0 * std::sqrt(1.0 / (p.dx * p.dx) + 1.0 / (p.dy * p.dy) + 1.0 / (p.dz * p.dz)))) *
         p.dt_coef;
  p.rc_i = x86_int(p.rc_i / p.ds);
  p.rc_size = x86_int(p.rc_size / p.ds);
  p.rc_delta = x86_int(p.rc_delta / p.ds);
  p.p_pos_i = x86_int(p.p_pos_i / p.ds);
  p.p_pos_j = x86_int(p.p_pos_j / p.ds);
  p.p_pos_k = x86_int(p.p_pos_k / p.ds);
  p.p_size_i = x86_int(p.p_size_i / p.ds);
  if (p.exp_time_key == 1) {
    // a time in steps; -1 (rejected when the problem is built) when it is
    // not finite, negative or beyond 2^28 steps
    auto steps = [&](double ns) {
      const double v = (ns * 1e-9) / p.dt;
      return (std::isfinite(v) && v >= 0 && v < 268435456.0) ? (int)v : -1;
    };
    p.n_max = steps(p.exp_time);
    p.fronts = steps(p.fronts_ns);
    p.plato = steps(p.plato_ns);
    p.p_begin_after = x86_int(p.p_begin_after * (1e-9 / p.dt));
    p.p_finish_at = x86_int(p.p_finish_at * (1e-9 / p.dt));
  }
}

namespace {

constexpr int kNumMaterials = 150;
constexpr int kPmlSize = 11;          // PML_SIZE, FDTD_2D_Full/Settings.cuh:23
constexpr int kMCoef = 100;           // M_COEF, Settings.cuh:166
constexpr double kPiMacro = 3.14;     // M_PI macro, Settings.cuh:7

struct Maps {
  int nx, ny;
  std::vector<int32_t>& id1;
  std::vector<int32_t>& id2;
  std::vector<int32_t>& id3;
  int32_t& at(std::vector<int32_t>& m, int I, int J) { return m[(size_t)J * nx + I]; }
  bool ok(int I, int J) const { return I >= 0 && J >= 0 && I < nx && J < ny; }
  // yeeCubeFace (FDTD_cuda.cu:2793-2819)
  void face(int I, int J, int t, char f) {
    if (f == 'x') { set(id1, I, J, t); set(id1, I, J + 1, t); }
    if (f == 'y') { set(id2, I, J, t); set(id2, I + 1, J, t); }
    if (f == 'z') { set(id3, I, J, t); set(id3, I + 1, J, t); set(id3, I + 1, J + 1, t); set(id3, I, J + 1, t); }
  }
  void set(std::vector<int32_t>& m, int I, int J, int t) {
    if (ok(I, J)) at(m, I, J) = t;
  }
  // addYeeCube (FDTD_cuda.cu:2873-2972): raise a plasma level, floor at 8.
  void add(std::vector<int32_t>& m, int I, int J, int t) {
    if (!ok(I, J)) return;
    int32_t& v = at(m, I, J);
    if (v == 0) v = 8;
    v = (v + t > 8) ? v + t : 8;
  }
  void add_face(int I, int J, int t, char f) {
    if (f == 'x') { add(id1, I, J, t); add(id1, I, J + 1, t); }
    if (f == 'y') { add(id2, I, J, t); add(id2, I + 1, J, t); }
    if (f == 'z') { add(id3, I, J, t); add(id3, I + 1, J, t); add(id3, I + 1, J + 1, t); add(id3, I, J + 1, t); }
  }
  // yeeCube (FDTD_cuda.cu:2771-2791): only the Ez map is written.
  void cube(int I, int J, int t) { face(I, J, t, 'z'); }
};

// The level of every sampled point (i, j) = (si*a, sj*b), i < nx - 1,
// j < ny - 1, evaluated in parallel (the pow/sqrt work); the callers then
// write the maps serially in the reference's loop order, so overlapping
// writes resolve as there.
template <class Level>
std::vector<int> sample_levels(int nx, int ny, int si, int sj, const Level& level) {
  const int ni = (nx - 1 + si - 1) / si, nj = (ny - 1 + sj - 1) / sj;
  std::vector<int> v((size_t)std::max(ni, 0) * std::max(nj, 0));
#pragma omp parallel for schedule(static)
  for (int a = 0; a < ni; ++a)
    for (int b = 0; b < nj; ++b) v[(size_t)a * nj + b] = level(a * si, b * sj);
  return v;
}

// One pass of sampled faces in the reference's order: apply(i, j, level).
template <class Level, class Apply>
void face_pass(const Maps& M, int si, int sj, const Level& level, const Apply& apply) {
  const std::vector<int> v = sample_levels(M.nx, M.ny, si, sj, level);
  const int nj = (M.ny - 1 + sj - 1) / sj;
  for (int i = 0, a = 0; i < M.nx - 1; i += si, ++a)
    for (int j = 0, b = 0; j < M.ny - 1; j += sj, ++b) apply(i, j, v[(size_t)a * nj + b]);
}

// buildSphericalMedium, equation type 2 (FDTD_cuda.cu:3114-3209).  The
// reference evaluates with its global k = 0 against MediumCen.K = 1.
void sphere_medium(const IniParams& p, Maps& M) {
  const float ra = (float)p.eq_r, alpha = (float)p.eq_alpha, beta = (float)p.eq_beta;
  const int k = 0;
  auto level = [&](int i, int j) {
    const float chis = (float)std::sqrt(
        ((p.sph_p * std::pow((float)i - p.med_i, 2)) / std::pow((float)p.sph_a, 2)) +
        ((p.sph_q * std::pow((float)j - p.med_j, 2)) / std::pow((float)p.sph_b, 2)) +
        ((p.sph_n * std::pow((float)k - p.med_k, 2)) / std::pow((float)p.sph_c, 2)));
    return x86_int((kMCoef * std::pow((1 - std::pow(((chis) / ra), alpha)), beta)) + 8);
  };
  face_pass(M, 1, 2, level, [&](int i, int j, int m) { if (m >= 8) M.face(i, j, m, 'x'); });
  face_pass(M, 2, 1, level, [&](int i, int j, int m) { if (m >= 8) M.face(i, j, m, 'y'); });
  face_pass(M, 2, 2, level, [&](int i, int j, int m) { if (m >= 8) M.face(i, j, m, 'z'); });
}

// buildSphericalMediumFluc, equation type 2 (FDTD_cuda.cu:3211-3311).
void fluc_medium(const IniParams& p, const std::vector<float>& pne, Maps& M) {
  if (p.fluc_build != 2) return;
  int ne0 = 0;
  for (int i = 8; i < kNumMaterials && pne[i] < (float)p.fluc_ne0; ++i) ne0 = i - 8;
  const float ax = (float)(p.fluc_angle_i * 3.14159 / 180);
  const float ay = (float)(p.fluc_angle_j * 3.14159 / 180);
  const float az = (float)(p.fluc_angle_k * 3.14159 / 180);
  const int k = 0;
  const float ra = (float)p.fluc_r, alpha = (float)p.fluc_alpha, beta = (float)p.fluc_beta;
  const int Ic = p.fluc_i, Jc = p.fluc_j, Kc = p.fluc_k;
  auto level = [&](int i, int j) {
    const int i_ = x86_int((k - Kc) * std::sin(ay) + (i - Ic) * std::cos(ay) * std::cos(az) -
                         (j - Jc) * std::cos(ay) * std::sin(az));
    const int j_ = x86_int((i - Ic) * (std::cos(ax) * std::sin(az) + std::cos(az) * std::sin(ax) * std::sin(ay)) +
                         (j - Jc) * (std::cos(ax) * std::cos(az) - std::sin(ax) * std::sin(ay) * std::sin(az)) -
                         (k - Kc) * std::cos(ay) * std::sin(ax));
    const int k_ = x86_int((i - Ic) * (std::sin(ax) * std::sin(az) - std::cos(ax) * std::cos(az) * std::sin(ay)) +
                         (j - Jc) * (std::cos(az) * std::sin(ax) + std::cos(ax) * std::sin(ay) * std::sin(az)) +
                         (k - Kc) * std::cos(ax) * std::cos(ay));
    const float chis = (float)std::sqrt(((p.fluc_p * std::pow((float)i_, 2)) / std::pow((float)p.fluc_a, 2)) +
                                        ((p.fluc_q * std::pow((float)j_, 2)) / std::pow((float)p.fluc_b, 2)) +
                                        ((p.fluc_n * std::pow((float)k_, 2)) / std::pow((float)p.fluc_c, 2)));
    return x86_int(std::floor(ne0 * std::pow((1 - std::pow(((chis) / ra), alpha)), beta)));
  };
  const int sg = p.fluc_sign;
  face_pass(M, 1, 2, level, [&](int i, int j, int m) { if (m >= 0) M.add_face(i, j, sg * m, 'x'); });
  face_pass(M, 2, 1, level, [&](int i, int j, int m) { if (m >= 0) M.add_face(i, j, sg * m, 'y'); });
  face_pass(M, 2, 2, level, [&](int i, int j, int m) { if (m >= 0) M.add_face(i, j, sg * m, 'z'); });
}

// buildTorusMedium, equation type 2 (FDTD_cuda.cu:3314-3378); M_PI is the
// macro 3.14 there.  Its local k = 1 is passed to yeeCube as the K index,
// which with Kmax = 1 lands every write one row higher (J*Imax + K*Imax + I).
void torus_medium(const IniParams& p, Maps& M) {
  const float R0 = (float)p.torus_br, Z0 = (float)p.med_k;
  const int ne0 = kMCoef;
  const float nea = 8, alpha = (float)p.eq_alpha, beta = (float)p.eq_beta, a = (float)p.eq_r;
  const float kk = 1;
  auto level = [&](int i, int j) {
    float px = (float)(i - p.med_i), py = (float)(j - p.med_j), pz = kk - Z0;
    float phi;
    if (px > 0) {
      phi = std::atan(py / px);
    } else {
      const int sign = (py >= 0) - (py < 0);
      phi = (px < 0) ? (float)(std::atan(py / px) + sign * kPiMacro) : (float)(sign * (kPiMacro / 2));
    }
    px = px * std::cos(phi) + py * std::sin(phi) - R0;
    pz /= kk;
    const float r_ = std::sqrt(px * px + pz * pz);
    return x86_int((ne0 - nea) * std::pow(1 - std::pow(r_ / a, alpha), beta) + nea);
  };
  face_pass(M, 1, 1, level, [&](int i, int j, int m) { if (m >= 8) M.cube(i, j + 1, m); });
}

// buildPlateMedium (FDTD_cuda.cu:3079-3111): steel (material 5) from WallPos up.
void plate_medium(const IniParams& p, Maps& M) {
  for (int i = 1; i < M.nx - 1; ++i)
    for (int j = p.wall_pos; j < M.ny - 1; ++j) M.cube(i, j, 5);
}

// calculate2Darrai / calculateDetect2Darrai (FDTD_cuda.cu:3380-3490): element
// positions Istart + d*e with Istart = cen - size/2 (integer division).
std::vector<int> array_positions(int cen, int size, int d, int* count) {
  const int q = size / d + 1;
  const int start = cen - size / 2;
  std::vector<int> a(q);
  for (int e = 0; e < q; ++e) a[e] = start + d * e;
  *count = q;
  return a;
}

}  // namespace

bool processing_params_ok(const IniParams& ip) {
  return ip.p_filter_win >= 1 && ip.p_sdf_win >= 1 && ip.p_cf_tau >= 0 && ip.p_arc_tau >= 0;
}

int build_from_ini(const IniParams& ip, Problem& p, bool objects) {
  p.from_ini = true;
  const int nx = ip.imax, ny = ip.jmax, P = kPmlSize;
  if (nx < 2 * P + 2 || ny < 2 * P + 2 || ip.n_max < 1) return FDTD2D_ERR_CONFIG;
  if (ip.draw2d != 0) {
    p.warnings += "Draw2D chamber figures are not supported by this build\n";
    return FDTD2D_ERR_CONFIG;
  }
  if (ip.s_di <= 0 || ip.d_di <= 0) return FDTD2D_ERR_CONFIG;
  // Values the reference would index or allocate with out of range: array
  // sizes below zero, and the TOF filter windows and delays (its moving
  // average and constant-fraction search step by them).
  if (ip.s_pi < 0 || ip.d_pi < 0 || (ip.rc_delta > 0 && ip.rc_size < 0)) return FDTD2D_ERR_CONFIG;
  // pulse fronts and plateau in steps (the envelope table is written from them)
  if (ip.fronts < 0 || ip.plato < 0 || ip.fronts > (1 << 28) || ip.plato > (1 << 28)) return FDTD2D_ERR_CONFIG;
  if (ip.p_perform && !processing_params_ok(ip)) return FDTD2D_ERR_CONFIG;
  const double dt = ip.dt;
  const double eps = eps0(), mu = mu0();

  // Materials (initialize + setUp, FDTD_cuda.cu:516-560, 1122-1200).
  std::vector<double> epsilon(kNumMaterials, eps), muv(kNumMaterials, mu), sigma(kNumMaterials, 0.0),
      ro(kNumMaterials, 0.0);
  epsilon[2] = 4.0 * eps; sigma[2] = 0.005;
  epsilon[3] = 8.0 * eps; sigma[3] = 3.96E7;
  epsilon[4] = 9.5 * eps; sigma[4] = 5.76E7;
  epsilon[5] = 9.0 * eps; sigma[5] = 2e6;
  epsilon[6] = 2.1 * eps; sigma[6] = 7.8e-4;
  epsilon[7] = 81 * eps; sigma[7] = 1e-2;
  p.mat_ca.assign(kNumMaterials, 0.f);
  p.mat_cb.assign(kNumMaterials, 0.f);
  p.mat_da.assign(kNumMaterials, 0.f);
  p.mat_db.assign(kNumMaterials, 0.f);
  p.mat_ne.assign(kNumMaterials, 0.f);
  const float ne0 = (float)ip.eq_ne0, nea = (float)ip.eq_nea;
  for (int i = 8; i < kNumMaterials; ++i) p.mat_ne[i] = (float)((((i - 8) * 0.01)) * (ne0 - nea) + nea);
  for (int i = 0; i < kNumMaterials; ++i) {
    const double se = sigma[i] * dt / (2.0 * epsilon[i]);
    const double sm = ro[i] * dt / (2.0 * muv[i]);
    p.mat_ca[i] = (float)((1.0 - se) / (1.0 + se));
    p.mat_cb[i] = (float)((dt / (epsilon[i])) / (1.0 + se));
    p.mat_da[i] = (float)((1.0 - sm) / (1.0 + sm));
    p.mat_db[i] = (float)((dt / (muv[i])) / (1.0 + sm));
  }

  // Medium maps (buildObject, FDTD_cuda.cu:2602-2660).
  p.id1.assign((size_t)nx * ny, 0);
  p.id2.assign((size_t)nx * ny, 0);
  p.id3.assign((size_t)nx * ny, 0);
  Maps M{nx, ny, p.id1, p.id2, p.id3};
  if (objects) {
    if (ip.build_medium == 1) sphere_medium(ip, M);
    if (ip.build_medium == 2) torus_medium(ip, M);
    if (ip.fluc_build != 0) fluc_medium(ip, p.mat_ne, M);
  }
  // The steel wall: Build_Stell_wall takes DrawWall only outside the
  // SourceToDetect mode (initlimits, FDTD_2D_Full/FDTD_cuda.cu:384-437), so
  // neither run of that mode has it.
  if (ip.draw_wall == 1 && ip.s2d != 1) plate_medium(ip, M);
  for (size_t t = 0; t < p.id1.size(); ++t) {
    if (p.id1[t] >= kNumMaterials || p.id2[t] >= kNumMaterials || p.id3[t] >= kNumMaterials ||
        p.id1[t] < 0 || p.id2[t] < 0 || p.id3[t] < 0) {
      p.warnings += "medium level outside the 150-material table\n";
      return FDTD2D_ERR_CONFIG;
    }
  }

  // Arrays.  Source elements sit at column arrayI[e]+e and row Jsource+arrayK[0]
  // (arrayK[0] = K_SOURCE - 1/2 = 1): Dev_AESASourceCalc's linear index adds
  // the element index to the column and arrayK to the row (kernel.cu:639-653).
  int q_src = 0, q_det = 0, q_rc = 0;
  p.array_i = array_positions(ip.src_i, ip.s_pi, ip.s_di, &q_src);
  p.det_array_i = array_positions(ip.det_i, ip.d_pi, ip.d_di, &q_det);
  p.rc_array_i = ip.rc_delta > 0 ? array_positions(ip.rc_i, ip.rc_size, ip.rc_delta, &q_rc) : std::vector<int>();
  const int k_src = ip.src_k - 1 / 2;   // Kstart = floor(K - sizeK/2), sizeK = 1
  const int k_det = ip.det_k - 1 / 2;
  if (q_det > q_src) {
    // Dev_AESAComponentDetector indexes the source array with detector indices.
    p.warnings += "detector array longer than the source array\n";
    return FDTD2D_ERR_CONFIG;
  }
  for (int e = 0; e < q_src; ++e) {
    p.src.push_back({p.array_i[e] + e, ip.src_j + k_src});
    p.src_phase.push_back((double)(float)(90 + (float)ip.s_angle * e));
  }
  for (int e = 0; e < q_det; ++e) p.det.push_back({p.det_array_i[e] + e, ip.det_j + k_det});
  for (int e = 0; e < q_det; ++e) p.comp.push_back({p.array_i[e] + e, ip.det_j + k_src});

  // Source envelope (buildSourceProfile, FDTD_cuda.cu:3539-3655).  Entries past
  // the pulse are never written by the reference (heap garbage there, zero in
  // practice for large allocations); they are 0 here, as is SourceP[nMax],
  // which the step loop reads one past the end.
  const int nmax = ip.n_max;
  const int plato_w = ip.plato, front_w = ip.fronts / 2;
  std::vector<float> namp(std::max(1, ip.fronts), 0.f);
  for (int i = 0; i < 2 * front_w; ++i) {
    const double up = std::pow(double(i - front_w), 2.);
    const double lc = double(front_w) / double(2.5);
    namp[i] = (float)(ip.amp * (std::exp(-1.0 * up / std::pow(lc, 2.))));
  }
  p.source_p.assign(nmax, 0.f);
  {
    int j = 0, i = 0;
    for (i = 0; i < front_w && j < nmax; i++, j++) p.source_p[i] = namp[i];
    for (i = front_w; i < front_w + plato_w && j < nmax; i++, j++) p.source_p[i] = (float)ip.amp;
    for (i = 0; i < front_w && j < nmax; i++, j++) p.source_p[front_w + plato_w + i] = namp[front_w + i];
  }
  p.envelope.assign(nmax + 1, 0.f);
  for (int n = 0; n < nmax; ++n) p.envelope[n] = p.source_p[n];
  const float fcoef = (float)(ip.freq_a * 1E9);
  const float fcoef2 = (float)((ip.chirp == 1 ? ip.freq_b : ip.freq_a) * 1E9);
  const float pulse_w = (float)((plato_w + 2 * front_w) * dt);

  // Wave-front tracker (Dev_RCcalc launched with j_cut = SourceCen.J + 150,
  // kernel.cu:2170): the max runs on column RCdetArrayI[l], the scan on
  // RCdetArrayI[l] + l (the element index leaks into the column as for the
  // source), edge level starts at 10.0 (kernel.cu:1517).
  for (int l = 0; l < q_rc; ++l) {
    p.rc_scan.push_back(p.rc_array_i[l] + l);
    p.rc_max.push_back(p.rc_array_i[l]);
  }
  // TOF line probe (Dev_SaveLine, kernel.cu:666-688): its linear thread index
  // must stay below SizeI, which confines the copy to row j = 1; cells
  // i in [max(1, PosI), min(SizeI, PosI + SizeI - 1)] are copied, and only
  // when PosJ == 1 and PosK == 0.  Other entries stay at their initial zero.
  p.line_offset = 0;
  if (ip.p_perform && ip.p_pos_j == 1 && ip.p_pos_k == 0 && ip.p_size_i > 0) {
    const int c0 = std::max(1, ip.p_pos_i);
    const int c1 = std::min(std::min(ip.p_size_i, ip.p_pos_i + ip.p_size_i - 1), nx - 2);
    const int first = ip.p_begin_after + 1;
    const int last = std::min(ip.p_finish_at, nmax);
    if (c1 >= c0 && last >= first && first >= 1) {
      p.s.line_n = c1 - c0 + 1;
      p.s.line_i0 = c0;
      p.s.line_j = 1;
      p.s.line_first = first;
      p.s.line_last = last;
      p.line_offset = c0 - ip.p_pos_i;
    }
  }

  // Launch coverage (kernel.cu:2027-2033 with 1024-thread blocks of 512x2):
  // the bulk grid has floor(floor(Imax*Jmax/1024)/2) x 3 blocks, the I-strip
  // grid floor(PML_SIZE*Jmax/1024) blocks, the J-strip grid
  // floor(Imax*PML_SIZE/1024) blocks.
  // The SourceToDetect vacuum shot launches with 1024 x 1 blocks and one
  // block more than the floor (kernel.cu:1671-1675), which covers every cell.
  {
    const int64_t bulk = objects ? (int64_t)(((int64_t)nx * ny / 1024) / 2) * 3 * 1024
                                 : ((int64_t)nx * ny / 1024 + 1) * 1024;
    const int64_t pml_i = ((int64_t)P * ny / 1024 + (objects ? 0 : 1)) * 1024;
    const int64_t pml_j = ((int64_t)nx * P / 1024 + (objects ? 0 : 1)) * 1024;
    const int64_t cov[8] = {bulk, pml_j, bulk, pml_i, bulk, bulk, pml_i, pml_j};
    for (int k = 0; k < 8; ++k) p.s.cover[k] = cov[k] > 0 ? cov[k] : -1;  // -1: no thread at all
  }

  build_cpml(p, nx, ny, P, ip.dx, ip.dy, dt, 0.75, 15.0, 0.24, 3, 1);
  p.s.n_rc = (int32_t)p.rc_scan.size();
  p.s.rc_scan_i = p.rc_scan.empty() ? nullptr : p.rc_scan.data();
  p.s.rc_max_i = p.rc_max.empty() ? nullptr : p.rc_max.data();
  p.s.rc_j_cut = ip.src_j + 150;
  p.s.rc_level = (float)ip.rc_level;
  p.s.rc_edge0 = 10.0f;
  p.s.n_steps = nmax;
  p.s.medium = FDTD2D_MEDIUM_MATERIAL_ID;
  p.s.nu = 0;
  p.s.jz_coef = (double)(float)kElectronDrive;
  p.s.src_scale = 1.0 / (double)(q_src * 1);
  p.s.f0 = fcoef;
  p.s.f1 = fcoef2;
  p.s.t1 = pulse_w;
  p.s.src_pi = kPiMacro;
  p.s.record_traces = 1;
  p.s.dft_freq = 0;
  p.s.storage = FDTD2D_STORE_F32;
  return FDTD2D_OK;
}

}  // namespace fdtd2d
