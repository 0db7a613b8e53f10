// Drop-in program driver: Settings.ini in, the reference's output files out.
//
// Restates main -> initlimits (FDTD_2D_Full/FDTD_cuda.cu:20, 384-441) and the
// host side of DevFieldCalculation (FDTD_2D_Full/kernel.cu:1928-2818) on top
// of the C ABI: the time loop runs on the GPU through fdtd2d_run, and the
// files are written with the reference's formats:
//
//   Detect.txt        kernel.cu:2409-2421  "%lf\t%12lf\t%12lf\n " per step row;
//                     the third conversion has no argument in the reference
//                     (undefined output); this driver prints 0.
//   detAll.txt        kernel.cu:2432-2454  time in us, 6 component sums x1000
//   detEz/Hx/Hy.txt   kernel.cu:2456-2493  per-element samples x1000
//   Ez.txt            kernel.cu:2173-2303  slices every TimeSieve steps
//   FieldSaveDat.txt  kernel.cu:3041-3051
//   SourceP.txt       FDTD_cuda.cu:3647-3650
//   RcDet_data.txt    FDTD_cuda.cu:3492-3537
//   deb.txt           kernel.cu:2681-2751 (ID3 map dump)
//   iniLOG.txt, log.txt
//
// SourceToDetect = 1 (initlimits, FDTD_cuda.cu:389-417) adds a first shot
// without medium and wall (DevSourceToDetectInfluenceCalc, kernel.cu:1620-1926)
// whose traces go to Detect_S2D.txt ("%lf\t%12lf\n ", time in us),
// detAll_S2D.txt, detEz/Hx/Hy_S2D.txt, and DifDetEx.txt of the main shot holds
// the component-trace differences (kernel.cu:2497-2538).  Here the vacuum shot
// runs beside the main one on its own stream instead of before it.
//
// Sample rows follow the reference: row i of every trace file is the sample
// taken at step i (row 0 is all zeros, the step-nMax sample is never printed).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <new>
#include <thread>
#include <vector>

#include "../../include/fdtd2d.h"
#include "problem.h"

namespace fdtd2d {
Problem* problem_internal(fdtd2d_problem* p);
int rc_run_and_write(fdtd2d_ctx* ctx, const Problem& p, const std::string& dir, int32_t n_last,
                     std::vector<int>* spd_rows);
int processing_run(const Problem& p, const std::vector<std::vector<float>>& field,
                   const std::string& dir);
}  // namespace fdtd2d

using namespace fdtd2d;

namespace {

struct File {
  FILE* f = nullptr;
  File(const std::string& path, const char* mode) { f = std::fopen(path.c_str(), mode); }
  ~File() {
    if (f) std::fclose(f);
  }
  explicit operator bool() const { return f != nullptr; }
};

// One Ez slice as the reference prints it (kernel.cu:2173-2303): a line per
// column i of "%12f " values over j, and a newline in each of the other
// slice files per line.  The lines are formatted in parallel into strings,
// then written in order, so the files hold the bytes a serial loop writes.
void write_slice(FILE* fez, FILE* fex, FILE* fhx, FILE* fhy, FILE* fhz, const std::vector<float>& ez, int nx,
                 int ny, int sieve) {
  std::vector<int> cols;
  for (int i = 1; i < nx - 1; i += sieve) cols.push_back(i);
  std::vector<std::string> lines(cols.size());
#pragma omp parallel for schedule(dynamic, 4)
  for (int k = 0; k < (int)cols.size(); ++k) {
    std::string& line = lines[k];
    char buf[64];
    for (int j = 1; j < ny - 1; j += sieve) {
      const int len = std::snprintf(buf, sizeof buf, "%12f ", ez[(size_t)j * nx + cols[k]]);
      line.append(buf, (size_t)len);
    }
  }
  for (const std::string& line : lines) {
    std::fwrite(line.data(), 1, line.size(), fez);
    std::fputc('\n', fex);
    std::fputc('\n', fez);
    std::fputc('\n', fhx);
    std::fputc('\n', fhy);
    std::fputc('\n', fhz);
  }
}

std::string join(const std::string& dir, const char* name) {
  if (dir.empty()) return name;
  return dir + "/" + name;
}

void now_strings(char* tbuf, char* dbuf) {
  std::time_t t = std::time(nullptr);
  std::tm tm{};
  localtime_r(&t, &tm);
  std::strftime(tbuf, 64, "%H:%M:%S", &tm);
  std::strftime(dbuf, 64, "%m/%d/%y", &tm);
}

// logINIread (FDTD_2D_Full/FDTD_cuda.cu:178-303): echo of the raw parameters.
void write_ini_log(const std::string& dir, const IniParams& r) {
  File f(join(dir, "iniLOG.txt"), "a");
  if (!f) return;
  char tb[64], db[64];
  now_strings(tb, db);
  std::fprintf(f.f, "Config loaded from 'Settings.ini' on time %s date %s:\nHardware:\n GPU_device=%d\nRegimes: \n SourceToDetect=%d\nGrid param: \n Use_Exp_time=%d\n Imax=%d\n Jmax=%d\n Max_time=%d\n Exp_time=%g\n ds=%g\n dt_coef=%g\n Isource=%d\n Jsource=%d\n Idetect=%d\n Jdetect=%d\n",
               tb, db, r.gpu_device, r.s2d, r.exp_time_key, r.imax, r.jmax, r.n_max, r.exp_time, r.ds,
               r.dt_coef, r.src_i, r.src_j, r.det_i, r.det_j);
  std::fprintf(f.f, "AESA\n SIsize=%d\n SAutoDelta=%d\n SIdelta=%d\n SPAngle=%g\n DIsize=%d\n DAutoDelta=%d\n DIdelta=%d\nPulseParam:\n Chirp=%d\n FreqA=%g\n FreqB=%g\n Fronts=%d\n Plato=%d\n Fronts_ns=%g\n Plato_ns=%g\n Pulse_amp=%g\n2Dsave:\n From=%d\n To=%d\n TimeSieve=%d\n GridSieve=%d\nmedium:\n Build=%d\n Icen=%d\n Jcen=%d\n\n A=%g\n B=%g\n C=%g\n P=%d\n Q=%d\n N=%d\n\n Radius=%d\n Alpha=%g\n Beta=%g\n ne0=%g\n neA=%g\nmediumFluc:\n FlucBuild=%d\n FlucIcen=%d\n FlucJcen=%d\n\n FlucA=%g\n FlucB=%g\n FlucC=%g\n FlucP=%d\n FlucQ=%d\n FlucN=%d\n\n FlucAngleI=%g\n FlucAngleJ=%g\n FlucAngleK=%g\n FlucSign=%d\n\n FlucRadius=%d\n FlucAlpha=%g\n FlucBeta=%g\n FlucNe0=%g\n TorusBR=%d\nKameraConf:\n Draw2D=%d\n 2Dpreset=%d\n PatrubokL=%d\n DrawWall=%d\n WallPos=%d\n\nRC_calc:\n Iline=%d\n LIsize=%d\n LIdelta=%d\n FilterWindow=%d\n Rlevel=%g\n",
               r.s_pi, r.s_delta_auto, r.s_di, r.s_angle, r.d_pi, r.d_delta_auto, r.d_di, r.chirp,
               r.freq_a, r.freq_b, r.fronts, r.plato, r.fronts_ns, r.plato_ns, r.amp, r.save_from,
               r.save_to, r.save_time_sieve, r.save_grid_sieve, r.build_medium, r.med_i, r.med_j,
               r.sph_a, r.sph_b, r.sph_c, r.sph_p, r.sph_q, r.sph_n, r.eq_r, r.eq_alpha, r.eq_beta,
               r.eq_ne0, r.eq_nea, r.fluc_build, r.fluc_i, r.fluc_j, r.fluc_a, r.fluc_b, r.fluc_c,
               r.fluc_p, r.fluc_q, r.fluc_n, r.fluc_angle_i, r.fluc_angle_j, r.fluc_angle_k,
               r.fluc_sign, r.fluc_r, r.fluc_alpha, r.fluc_beta, r.fluc_ne0, r.torus_br, r.draw2d,
               r.preset, r.patrubok, r.draw_wall, r.wall_pos, r.rc_i, r.rc_size, r.rc_delta,
               r.rc_window, r.rc_level);
  std::fprintf(f.f, "\nProcessing:\n Perform=%d\n SecDer=%d\n SDFType=%d\n SDFWin=%d\n SDFRuns=%d\n CF=%d\n CFTau=%d\n CFK=%g\n ARC=%d\n ARCTau=%d\n ARCK=%g\n TauThreshold=%g\n FilterType=%d\n FilterWin=%d\n FilterRuns=%d\n SaveFiltered=%d\n SaveOriginal=%d\n PosI=%d\n PosJ=%d\n PosK=%d\n SizeI=%d\n BeginAfter=%d\n FinishAt=%d\n TimeSieve=%d\n DimSieve=%d\n SimDetect=%d\n DetSave=%d\n DetSize=%d\n DetWLoad=%d\n-----------------------------------------------------------------------------\n",
               r.p_perform, r.p_sec_der, r.p_sdf_type, r.p_sdf_win, r.p_sdf_runs, r.p_cf, r.p_cf_tau,
               r.p_cf_k, r.p_arc, r.p_arc_tau, r.p_arc_k, r.p_tau_threshold, r.p_filter_type,
               r.p_filter_win, r.p_filter_runs, r.p_save_filtered, r.p_save_original, r.p_pos_i,
               r.p_pos_j, r.p_pos_k, r.p_size_i, r.p_begin_after, r.p_finish_at, r.p_time_sieve,
               r.p_dim_sieve, r.p_sim_detect, r.p_save_detector, r.p_detector_size,
               r.p_load_weights);
}

// Traces of one shot in the reference's host layout: row i = step i, row 0
// zeros, rows 0..nmax-1.
struct Traces {
  int nd = 0, nc = 0, nmax = 0;
  std::vector<float> det, cez, chx, chy;
  int read(fdtd2d_ctx* ctx, const fdtd2d_setup& s) {
    nd = s.n_det; nc = s.n_comp; nmax = s.n_steps;
    std::vector<float> d((size_t)nmax * nd), e((size_t)nmax * nc), x((size_t)nmax * nc), y((size_t)nmax * nc);
    const int rc = fdtd2d_read_traces(ctx, 1, nmax, d.data(), e.data(), x.data(), y.data());
    if (rc) return rc;
    det.assign((size_t)nmax * nd, 0.f);
    cez.assign((size_t)nmax * nc, 0.f);
    chx.assign((size_t)nmax * nc, 0.f);
    chy.assign((size_t)nmax * nc, 0.f);
    // sample of step n (traces row n-1) goes to row n; step nmax is not kept
    std::copy(d.begin(), d.end() - nd, det.begin() + nd);
    std::copy(e.begin(), e.end() - nc, cez.begin() + nc);
    std::copy(x.begin(), x.end() - nc, chx.begin() + nc);
    std::copy(y.begin(), y.end() - nc, chy.begin() + nc);
    return FDTD2D_OK;
  }
};

// detEz/detHx/detHy rows (kernel.cu:2456-2493): per step, one line per element
// and a blank line.
void write_components(const Traces& t, FILE* ez, FILE* hx, FILE* hy, FILE* pp) {
  for (int i = 0; i < t.nmax; ++i) {
    for (int k = 0; k < t.nc; ++k) {
      std::fprintf(ez, "%12lf\t", (double)t.cez[(size_t)i * t.nc + k] * 1000);
      std::fprintf(hx, "%12lf\t", (double)t.chx[(size_t)i * t.nc + k] * 1000);
      std::fprintf(hy, "%12lf\t", (double)t.chy[(size_t)i * t.nc + k] * 1000);
      std::fputc('\n', ez);
      std::fputc('\n', hx);
      std::fputc('\n', hy);
      if (pp) std::fputc('\n', pp);
    }
    std::fputc('\n', ez);
    std::fputc('\n', hx);
    std::fputc('\n', hy);
    if (pp) std::fputc('\n', pp);
  }
}

// The SourceToDetect vacuum shot's files (kernel.cu:1640-1652, 1818-1918).
int write_s2d_files(const Traces& t, double dt, const std::string& dir) {
  File pDet(join(dir, "Detect_S2D.txt"), "w"), pAll(join(dir, "detAll_S2D.txt"), "w");
  File pEz(join(dir, "detEz_S2D.txt"), "w"), pHx(join(dir, "detHx_S2D.txt"), "w"),
      pHy(join(dir, "detHy_S2D.txt"), "w");
  File e1(join(dir, "CompDetect_S2D.txt"), "w"), e2(join(dir, "detEx_S2D.txt"), "w"),
      e3(join(dir, "detEy_S2D.txt"), "w"), e4(join(dir, "detHz_S2D.txt"), "w"), e5(join(dir, "detP_S2D.txt"), "w");
  if (!pDet || !pAll || !pEz || !pHx || !pHy) return FDTD2D_ERR_IO;
  for (int i = 0; i < t.nmax; ++i) {
    double sum = 0;
    for (int k = 0; k < t.nd; ++k) sum += t.det[(size_t)i * t.nd + k];
    std::fprintf(pDet.f, "%lf\t%12lf\n ", (dt * i) * 1000000, sum * 1000);
  }
  for (int i = 0; i < t.nmax; ++i) {
    double s3 = 0, s4 = 0, s5 = 0;
    for (int k = 0; k < t.nc; ++k) {
      s3 += t.cez[(size_t)i * t.nc + k];
      s4 += t.chx[(size_t)i * t.nc + k];
      s5 += t.chy[(size_t)i * t.nc + k];
    }
    std::fprintf(pAll.f, "%lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\n", (dt * i) * 1000000, 0.0, 0.0,
                 s3 * 1000, s4 * 1000, s5 * 1000, 0.0);
  }
  write_components(t, pEz.f, pHx.f, pHy.f, nullptr);
  return FDTD2D_OK;
}

// DifDetEx.txt (kernel.cu:2497-2538): per step the sums over elements of the
// component differences main - vacuum (each difference an FP32 subtraction,
// summed in FP64), and |E x H| of the summed differences with Ex = Ey = Hz = 0.
void write_difference(const Traces& m, const Traces& v, double dt, FILE* f) {
  for (int i = 0; i < m.nmax; ++i) {
    double s3 = 0, s4 = 0, s5 = 0;
    for (int k = 0; k < m.nc; ++k) {
      const size_t o = (size_t)i * m.nc + k;
      s3 += (double)(float)(m.cez[o] - v.cez[o]);
      s4 += (double)(float)(m.chx[o] - v.chx[o]);
      s5 += (double)(float)(m.chy[o] - v.chy[o]);
    }
    const double s1 = 0, s2 = 0, s6 = 0;
    const float eh_i = (float)(s2 * s6 - s3 * s5);
    const float eh_j = (float)(-(s1 * s6 - s3 * s4));
    const float eh_k = (float)(s1 * s5 - s2 * s4);
    const double mag = std::sqrt((double)eh_i * eh_i + (double)eh_j * eh_j + (double)eh_k * eh_k);
    std::fprintf(f, "%lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\n ", (dt * i) * 1000000, s1 * 1000,
                 s2 * 1000, s3 * 1000, s4 * 1000, s5 * 1000, s6 * 1000, mag * 1000);
  }
}

}  // namespace

static int run_settings_body(const char* ini_path, const char* out_dir, int device);

extern "C" int fdtd2d_run_settings(const char* ini_path, const char* out_dir, int device) {
  if (!ini_path) return FDTD2D_ERR_INVALID;
  try {
    return run_settings_body(ini_path, out_dir, device);
  } catch (const std::bad_alloc&) {
    return FDTD2D_ERR_NOMEM;
  } catch (...) {
    return FDTD2D_ERR_CONFIG;   // no C++ exception leaves the C ABI
  }
}

static int run_settings_body(const char* ini_path, const char* out_dir, int device) {
  const std::string dir = out_dir ? out_dir : "";
  const auto t_start = std::chrono::steady_clock::now();
  IniParams raw;
  std::string log;
  int rc = parse_ini(ini_path, raw, log);
  if (rc) return rc;
  write_ini_log(dir, raw);

  fdtd2d_problem* handle = nullptr;
  rc = fdtd2d_problem_from_ini(ini_path, &handle);
  if (rc) return rc;
  Problem& p = *problem_internal(handle);
  const IniParams& ip = p.ini;
  const fdtd2d_setup& s = p.s;
  const int nx = s.nx, ny = s.ny, nmax = s.n_steps;

  // SourceP.txt, RcDet_data.txt (written during setup by the reference)
  {
    File f(join(dir, "SourceP.txt"), "w");
    if (!f) { fdtd2d_problem_free(handle); return FDTD2D_ERR_IO; }
    for (int k = 0; k < nmax; ++k) std::fprintf(f.f, "%f\n", p.source_p[k]);
    File r(join(dir, "RcDet_data.txt"), "w");
    if (r) {
      for (int v : p.rc_array_i) std::fprintf(r.f, "%d ", v);
      std::fprintf(r.f, "\n0 ");
    }
  }

  fdtd2d_ctx* ctx = nullptr;
  if (device < 0) device = ip.gpu_device;  // [hardware] GPU_device, as cudaSetDevice(GPU_device)
  rc = fdtd2d_create(&s, device, &ctx);
  if (rc) {
    fdtd2d_problem_free(handle);
    return rc;
  }
  // SourceToDetect: the vacuum shot, stepped alongside the main one.
  fdtd2d_problem* vac_handle = nullptr;
  fdtd2d_ctx* vac = nullptr;
  if (ip.s2d == 1) {
    rc = problem_from_ini_ex(ini_path, false, &vac_handle);
    if (rc == FDTD2D_OK) rc = fdtd2d_create(fdtd2d_problem_setup(vac_handle), device, &vac);
    if (rc) {
      if (vac_handle) fdtd2d_problem_free(vac_handle);
      fdtd2d_destroy(ctx);
      fdtd2d_problem_free(handle);
      return rc;
    }
  }
  int32_t vac_done = 0;
  // Step both shots to n in chunks, so the vacuum shot's launches stay queued
  // beside the main shot's on their own stream.
  auto advance = [&](int32_t from, int32_t to) -> int {
    for (int32_t a = from; a <= to; a += 256) {
      const int32_t b = std::min(to, a + 255);
      if (vac) {
        const int r = fdtd2d_run(vac, vac_done + 1, b);
        if (r) return r;
        vac_done = b;
      }
      const int r = fdtd2d_run(ctx, a, b);
      if (r) return r;
    }
    return FDTD2D_OK;
  };

  File pEz(join(dir, "Ez.txt"), "w");
  File pEx(join(dir, "Ex.txt"), "wb"), pEy(join(dir, "Ey.txt"), "wb");
  File pHx(join(dir, "Hx.txt"), "w"), pHy(join(dir, "Hy.txt"), "w"), pHz(join(dir, "Hz.txt"), "w");
  if (!pEz) {
    if (vac) {
      fdtd2d_destroy(vac);
      fdtd2d_problem_free(vac_handle);
    }
    fdtd2d_destroy(ctx);
    fdtd2d_problem_free(handle);
    return FDTD2D_ERR_IO;
  }
  // Step loop with the reference's slice-save cadence (kernel.cu:2173-2303):
  // inside [From, To] a counter runs 1..TimeSieve and a slice is written when
  // it reaches TimeSieve.
  // Two slice buffers: a slice is written on a writer thread while the GPU
  // steps on towards the next one (at most one write in flight, so the
  // slices reach the files in order).
  std::vector<float> ez_buf[2] = {std::vector<float>((size_t)nx * ny), std::vector<float>((size_t)nx * ny)};
  std::thread writer;
  int save_counter = 0, save_app = 1;
  int32_t done = 0;
  const int sieve = ip.save_grid_sieve > 0 ? ip.save_grid_sieve : 1;
  for (int n = 1; n <= nmax && rc == FDTD2D_OK; ++n) {
    bool save = false;
    if (n >= ip.save_from && n <= ip.save_to) {
      if (save_app == ip.save_time_sieve) {
        save = true;
        save_app = 1;
      } else {
        save_app++;
      }
    }
    if (!save && n < nmax) continue;
    rc = advance(done + 1, n);
    done = n;
    if (rc || !save) continue;
    std::vector<float>& ez = ez_buf[save_counter & 1];
    if (writer.joinable()) writer.join();   // the other buffer's write is done before this one is read into
    rc = fdtd2d_read_field(ctx, FDTD2D_FIELD_EZ, ez.data());
    if (rc) break;
    save_counter++;
    writer = std::thread(write_slice, pEz.f, pEx.f, pHx.f, pHy.f, pHz.f, std::cref(ez), nx, ny, sieve);
  }
  if (writer.joinable()) writer.join();
  if (rc == FDTD2D_OK) rc = fdtd2d_synchronize(ctx);

  if (rc == FDTD2D_OK) {
    // FieldSaveDat.txt (VriteSaveParameters)
    File f(join(dir, "FieldSaveDat.txt"), "w");
    int count_m = 0;
    for (int i = 1; i < nx - 1; i += sieve) count_m++;
    if (f) std::fprintf(f.f, "%d %d", count_m, save_counter);
  }

  // Detector files (rows: step i).
  Traces tr, vtr;
  if (rc == FDTD2D_OK) rc = tr.read(ctx, s);
  if (rc == FDTD2D_OK && vac) {
    rc = vtr.read(vac, *fdtd2d_problem_setup(vac_handle));
    if (rc == FDTD2D_OK) rc = write_s2d_files(vtr, s.dt, dir);
  }
  if (rc == FDTD2D_OK) {
    const int nd = tr.nd, nc = tr.nc;
    File pDet(join(dir, "Detect.txt"), "w");
    File pAll(join(dir, "detAll.txt"), "w");
    File pdEz(join(dir, "detEz.txt"), "w"), pdHx(join(dir, "detHx.txt"), "w"),
        pdHy(join(dir, "detHy.txt"), "w"), pdP(join(dir, "detP.txt"), "w");
    File e1(join(dir, "detEx.txt"), "w"), e2(join(dir, "detEy.txt"), "w"), e3(join(dir, "detHz.txt"), "w");
    File pDif(join(dir, "DifDetEx.txt"), "w"), e5(join(dir, "CompDetect.txt"), "w");
    File e6(join(dir, "LineDetect.txt"), "w"), e7(join(dir, "LineDetect2.txt"), "w");
    File e8(join(dir, "test.txt"), "w"), e9(join(dir, "SDetect.txt"), "w");
    if (!pDet || !pAll || !pdEz || !pdHx || !pdHy || !pDif) rc = FDTD2D_ERR_IO;
    for (int i = 0; i < nmax && rc == FDTD2D_OK; ++i) {
      double sum = 0;
      for (int k = 0; k < nd; ++k) sum += tr.det[(size_t)i * nd + k];
      std::fprintf(pDet.f, "%lf\t%12lf\t%12lf\n ", (s.dt * i) * 1e12, sum * 1000, 0.0);
      double s3 = 0, s4 = 0, s5 = 0;
      for (int k = 0; k < nc; ++k) {
        s3 += tr.cez[(size_t)i * nc + k];
        s4 += tr.chx[(size_t)i * nc + k];
        s5 += tr.chy[(size_t)i * nc + k];
      }
      std::fprintf(pAll.f, "%lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\t%12lf\n ", (s.dt * i) * 1000000,
                   0.0, 0.0, s3 * 1000, s4 * 1000, s5 * 1000, 0.0);
    }
    if (rc == FDTD2D_OK) write_components(tr, pdEz.f, pdHx.f, pdHy.f, pdP ? pdP.f : nullptr);
    if (rc == FDTD2D_OK && vac) write_difference(tr, vtr, s.dt, pDif.f);
  }
  if (vac) {
    fdtd2d_destroy(vac);
    fdtd2d_problem_free(vac_handle);
    vac = nullptr;
  }

  // Wave-front tracker outputs (RC_Line.txt, TAU_Line.txt).
  if (rc == FDTD2D_OK) rc = rc_run_and_write(ctx, p, dir, nmax, nullptr);
  // TOF processing on the saved line (processing_core, FDTD_2D_Full/kernel.cu:2313).
  if (rc == FDTD2D_OK && ip.p_perform) {
    const int first = ip.p_begin_after + 1;
    const int last = std::min(ip.p_finish_at, nmax);
    const int times = std::max(0, last - first + 1);
    std::vector<std::vector<float>> field(times, std::vector<float>(std::max(0, ip.p_size_i), 0.f));
    if (s.line_n > 0) {
      std::vector<float> buf((size_t)times * s.line_n);
      rc = fdtd2d_read_line(ctx, s.line_first, s.line_last, buf.data());
      for (int t = 0; t < times && rc == FDTD2D_OK; ++t)
        for (int c = 0; c < s.line_n; ++c) field[t][p.line_offset + c] = buf[(size_t)t * s.line_n + c];
    }
    if (rc == FDTD2D_OK) rc = processing_run(p, field, dir);
  }

  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  if (rc == FDTD2D_OK) {
    File f(join(dir, "log.txt"), "a");
    if (f) {
      char tb[64], db[64];
      now_strings(tb, db);
      std::fprintf(f.f, "-------------------------------------------------------------------------\n");
      std::fprintf(f.f, "OS date:\t\t\t\t%s\n", db);
      std::fprintf(f.f, "OS time:\t\t\t\t%s\n", tb);
      std::fprintf(f.f, "-------------------------------------------------------------------------\n");
      std::fprintf(f.f,
                   "NET PARAMETERS \n Ex(%d, %d, %d) \n Ey(%d, %d, %d) \n Ez(%d, %d, %d) \n Hx(%d, %d, %d) \n Hy(%d, %d, %d) \n Hz(%d, %d, %d)\n\n(dx ,dy, dz) - dt: (%f mm, %f mm, %f mm) - %f ns\n",
                   nx - 1, ny, 0, nx, ny - 1, 0, nx, ny, 1, nx, ny - 1, 1, nx - 1, ny, 1, nx - 1, ny - 1, 0,
                   ip.dx * 1000, ip.dy * 1000, ip.dz * 1000, s.dt * 1e9);
      std::fprintf(f.f, "\nSIMULATION PARAMETERS\n Total Simulation time: %d time steps or %e seconds\n", nmax,
                   nmax * s.dt);
      std::fprintf(f.f,
                   "\nSAVE DATA PARAMETER\nSlises saved: %d\nData saved from time %d to time %d \nTime sieve parameter: %d \nNet sieve parameter: %d\nData multiplier: %f\n",
                   save_counter, ip.save_from, ip.save_to, ip.save_time_sieve, ip.save_grid_sieve, 1.0);
      std::fprintf(f.f,
                   "\nSORCE AND DETECTOR\n Source point: (%d, %d, %d)\n Detector point(%d, %d, %d)\n Detector size: %dx%d points",
                   ip.src_i, ip.src_j, ip.src_k, ip.det_i, ip.det_j, ip.det_k, 10, 10);
      std::fprintf(f.f, "\n\nCalculation on GPU\n Calculation time: %f seconds\n\n", secs);
    }
    // deb.txt: the Ez material map, rows i, columns j (kernel.cu:2737-2751)
    File d(join(dir, "deb.txt"), "w");
    File m(join(dir, "materials.txt"), "w");
    if (d) {
      for (int i = 1; i < nx - 1; i++) {
        for (int j = 1; j < ny - 1; j++) std::fprintf(d.f, "%d ", p.id3[(size_t)j * nx + i]);
        std::fprintf(d.f, "\n");
      }
      std::fprintf(d.f, "\n\n");
      std::fprintf(d.f, "\n\n");
    }
  }
  fdtd2d_destroy(ctx);
  fdtd2d_problem_free(handle);
  return rc;
}
