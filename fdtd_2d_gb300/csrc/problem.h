// Host-side setup precompute (the reference's L2 layer, FDTD_2D_Full/FDTD_cuda.cu).
// A Problem owns every array its fdtd2d_setup view points to.  It also keeps
// the Settings.ini parameters the drop-in driver needs for its output files.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fdtd2d.h"

namespace fdtd2d {

// Physical constants as the reference defines them (FDTD_2D_Full/FDTD_cuda.cuh:20-21,
// FDTD_cuda.cu:501-502).
constexpr double kC0 = 2.99792458E8;
constexpr double kPiRef = 3.14159265358979;      // `pi` in FDTD_cuda.cuh:20
constexpr double kPiExact = 3.14159265358979323846;
constexpr double kElectronDrive = 2.81794E-8;    // D_CJ, e^2/m_e (kernel.cu:119), stored as float
inline double mu0() { return 4.0 * kPiRef * 1.0E-7; }
inline double eps0() { return 1.0 / (kC0 * kC0 * mu0()); }

// Settings.ini parameters after recuclParametersToMetric (cells, steps).
struct IniParams {
  int gpu_device = 0;
  int s2d = 0;
  double ds = 1, dt_coef = 0.5;
  int imax = 550, jmax = 600;
  int exp_time_key = 0;
  int n_max = 10000;
  double exp_time = 10;
  int src_i = 300, src_j = 20, src_k = 1;
  int det_i = 250, det_j = 30, det_k = 1;
  int s_pi = 40, s_delta_auto = 0, s_di = 5;
  double s_angle = 0;
  int d_pi = 40, d_delta_auto = 0, d_di = 5;
  int chirp = 0;
  double freq_a = 28, freq_b = 30;
  int fronts = 2000, plato = 2000;
  double fronts_ns = 3, plato_ns = 3;
  double amp = 1000;
  int save_from = 0, save_to = 40000, save_time_sieve = 240, save_grid_sieve = 1;
  int build_medium = 0;
  int med_i = 275, med_j = 305, med_k = 1;
  double sph_a = 1, sph_b = 1, sph_c = 1;
  int sph_p = 1, sph_q = 1, sph_n = 1;
  int eq_r = 50;
  double eq_alpha = 2.0, eq_beta = 1.0, eq_ne0 = 1e19, eq_nea = 0;
  int torus_br = 175;
  int fluc_build = 0;
  int fluc_i = 275, fluc_j = 305, fluc_k = 1;
  double fluc_a = 1, fluc_b = 1, fluc_c = 1;
  int fluc_p = 1, fluc_q = 1, fluc_n = 1;
  double fluc_angle_i = 0, fluc_angle_j = 0, fluc_angle_k = 0;
  int fluc_sign = 1;
  int fluc_r = 10;
  double fluc_alpha = 2.0, fluc_beta = 1.0, fluc_ne0 = 1e19;
  int draw2d = 0, preset = 7, patrubok = 5, draw_wall = 0, wall_pos = 950;
  int rc_i = 300, rc_size = 40, rc_delta = 5, rc_window = 200;
  double rc_level = 0.1;
  // [Processing] (FDTD_2D_Full/processing.cuh:8-50)
  bool p_perform = false, p_sec_der = false, p_cf = false, p_arc = false;
  bool p_save_filtered = false, p_save_original = false, p_sim_detect = false;
  bool p_save_detector = false, p_load_weights = false;
  int p_detector_size = 30, p_filter_type = 1, p_dim_sieve = 1, p_time_sieve = 1;
  int p_begin_after = 0, p_finish_at = 0, p_pos_i = 0, p_pos_j = 0, p_pos_k = 0, p_size_i = 0;
  int p_filter_win = 300, p_filter_runs = 1, p_sdf_win = 300, p_sdf_type = 1, p_sdf_runs = 1;
  int p_cf_tau = 300, p_arc_tau = 300;
  double p_tau_threshold = 0, p_arc_k = -0.5, p_cf_k = -0.5;
  // derived
  double dx = 1e-3, dy = 1e-3, dz = 1e-3, dt = 0;
};

struct Problem {
  fdtd2d_setup s{};
  // storage behind the view
  std::vector<float> tab[16];                 // CPML tables in fdtd2d_setup order
  std::vector<float> den_ex, den_hx, den_ey, den_hy;
  std::vector<float> ne;                      // uniform medium density map
  std::vector<int32_t> id1, id2, id3;         // material maps
  std::vector<float> mat_ca, mat_cb, mat_da, mat_db, mat_ne;
  std::vector<fdtd2d_point> src, det, comp;
  std::vector<double> src_phase;
  std::vector<float> envelope;
  // reference bookkeeping for the drop-in driver
  bool from_ini = false;
  IniParams ini;
  std::vector<int> array_i, det_array_i, rc_array_i;
  std::vector<float> source_p;                // SourceP[nMax] as the reference writes it
  std::vector<int32_t> rc_scan, rc_max;       // wave-front tracker columns
  int line_offset = 0;                        // probe column 0 within the TOF line
  std::string warnings;

  void bind();                                // point `s` at the vectors
};

// Build the 16 CPML tables and the 4 denominator tables with the reference's
// grading formulas (FDTD_2D_Full/FDTD_cuda.cu:1206-1214, 1224-1578), using the
// given sigma factor, kappa_max, alpha_max and orders.
void build_cpml(Problem& p, int nx, int ny, int npml, double dx, double dy, double dt,
                double sigma_factor, double kappa_max, double alpha_max, double m, double ma);

int parse_ini(const char* path, IniParams& ip, std::string& log);
void ini_to_metric(IniParams& ip);
// objects = false is the SourceToDetect vacuum run: no medium, no fluctuation
// (buildObject with ObjectsEnable == false, FDTD_2D_Full/FDTD_cuda.cu:2602-2625).
// The TOF processing's windows and delays are usable: filter windows of at
// least one sample, delays not negative.
bool processing_params_ok(const IniParams& ip);
int build_from_ini(const IniParams& ip, Problem& p, bool objects = true);

// fdtd2d_problem_from_ini with the objects switch of build_from_ini.
int problem_from_ini_ex(const char* path, bool objects, fdtd2d_problem** out);

}  // namespace fdtd2d
