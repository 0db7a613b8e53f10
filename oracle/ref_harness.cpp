// Harness around the reference program compiled for the CPU (oracle/ref_build.py).
// TEST INFRASTRUCTURE ONLY.
//
// Usage: ref_fdtd2d <run_dir>
// Runs the reference's main (renamed ref_program_main) in <run_dir>, where it
// reads Settings.ini and writes its output files, then dumps the setup tables
// and the final device state it leaves behind to <run_dir>/ref_dump.bin:
// records of (name[32], type char 'f'/'i'/'d', int64 count, raw data).
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "ref_shim/cuda_runtime.h"

thread_local uint3 blockIdx, threadIdx;
thread_local dim3 blockDim, gridDim;

void* ref_shim_alloc(size_t bytes) { return std::calloc(1, bytes + 65536); }

void ref_program_main();

// Reference globals (FDTD_2D_Full/FDTD_cuda.cuh, kernel.cu).
extern int Imax, Jmax, nMax, numMaterials;
extern double dt, dx, dy;
extern float *be_x_1, *ce_x_1, *be_x_2, *ce_x_2, *bh_x_1, *ch_x_1, *bh_x_2, *ch_x_2;
extern float *be_y_1, *ce_y_1, *be_y_2, *ce_y_2, *bh_y_1, *ch_y_1, *bh_y_2, *ch_y_2;
extern float *den_ex, *den_hx, *den_ey, *den_hy;
extern float *CA, *CB, *DA, *DB, *pne;
extern int *ID1, *ID2, *ID3;
extern int *arrayI, *arrayK, *det_arrayI, *det_arrayK, qantI, qantK, det_qantI, det_qantK;
extern int *RCdetArrayI, RC_qantI;
extern float *SourceP, fCoef, fCoef2, fPulseW;
extern float *detect, *det_Ez, *det_Hx, *det_Hy;
extern int *PspdLine;
extern float *DEz, *DHx, *DHy, *DJz;
extern float *D_psi_Ezx_1, *D_psi_Ezx_2, *D_psi_Ezy_1, *D_psi_Ezy_2;
extern float *D_psi_Hyx_1, *D_psi_Hyx_2, *D_psi_Hxy_1, *D_psi_Hxy_2;

namespace {
FILE* g_out;
void rec(const char* name, char type, int64_t count, const void* data) {
  char nm[32] = {};
  std::snprintf(nm, sizeof(nm), "%s", name);
  std::fwrite(nm, 1, 32, g_out);
  std::fwrite(&type, 1, 1, g_out);
  std::fwrite(&count, 8, 1, g_out);
  const size_t sz = type == 'd' ? 8 : 4;
  if (count > 0 && data) std::fwrite(data, sz, (size_t)count, g_out);
}
}  // namespace

int main(int argc, char** argv) {
  if (argc < 2 || chdir(argv[1]) != 0) {
    std::fprintf(stderr, "usage: ref_fdtd2d <run_dir>\n");
    return 2;
  }
  ref_program_main();
  g_out = std::fopen("ref_dump.bin", "wb");
  if (!g_out) return 3;
  const int P = 11;  // PML_SIZE
  int scal[4] = {Imax, Jmax, nMax, numMaterials};
  rec("scalars", 'i', 4, scal);
  double dsc[3] = {dt, dx, dy};
  rec("dt_dx_dy", 'd', 3, dsc);
  float fsc[3] = {fCoef, fCoef2, fPulseW};
  rec("fcoef_fcoef2_pulsew", 'f', 3, fsc);
  const char* tn[16] = {"be_x_1", "ce_x_1", "be_x_2", "ce_x_2", "bh_x_1", "ch_x_1", "bh_x_2", "ch_x_2",
                        "be_y_1", "ce_y_1", "be_y_2", "ce_y_2", "bh_y_1", "ch_y_1", "bh_y_2", "ch_y_2"};
  float* tv[16] = {be_x_1, ce_x_1, be_x_2, ce_x_2, bh_x_1, ch_x_1, bh_x_2, ch_x_2,
                   be_y_1, ce_y_1, be_y_2, ce_y_2, bh_y_1, ch_y_1, bh_y_2, ch_y_2};
  for (int k = 0; k < 16; ++k) rec(tn[k], 'f', (k % 8) >= 4 ? P - 1 : P, tv[k]);
  rec("den_ex", 'f', Imax - 1, den_ex);
  rec("den_hx", 'f', Imax - 1, den_hx);
  rec("den_ey", 'f', Jmax - 1, den_ey);
  rec("den_hy", 'f', Jmax - 1, den_hy);
  rec("CA", 'f', numMaterials, CA);
  rec("CB", 'f', numMaterials, CB);
  rec("DA", 'f', numMaterials, DA);
  rec("DB", 'f', numMaterials, DB);
  rec("pne", 'f', numMaterials, pne);
  const int64_t cells = (int64_t)Imax * Jmax;
  rec("ID1", 'i', cells, ID1);
  rec("ID2", 'i', cells, ID2);
  rec("ID3", 'i', cells, ID3);
  rec("arrayI", 'i', qantI, arrayI);
  rec("arrayK", 'i', qantK, arrayK);
  rec("det_arrayI", 'i', det_qantI, det_arrayI);
  rec("det_arrayK", 'i', det_qantK, det_arrayK);
  rec("RCdetArrayI", 'i', RC_qantI, RCdetArrayI);
  rec("SourceP", 'f', nMax, SourceP);
  const int64_t nd = (int64_t)det_qantI * det_qantK;
  rec("detect", 'f', (int64_t)nMax * nd, detect);
  rec("det_Ez", 'f', (int64_t)nMax * nd, det_Ez);
  rec("det_Hx", 'f', (int64_t)nMax * nd, det_Hx);
  rec("det_Hy", 'f', (int64_t)nMax * nd, det_Hy);
  rec("PspdLine", 'i', (int64_t)nMax * RC_qantI, PspdLine);
  rec("Ez", 'f', cells, DEz);
  rec("Hx", 'f', (int64_t)Imax * (Jmax - 1), DHx);
  rec("Hy", 'f', (int64_t)(Imax - 1) * Jmax, DHy);
  rec("Jz", 'f', cells, DJz);
  rec("psi_Ezx_1", 'f', (int64_t)P * Jmax, D_psi_Ezx_1);
  rec("psi_Ezx_2", 'f', (int64_t)P * Jmax, D_psi_Ezx_2);
  rec("psi_Hyx_1", 'f', (int64_t)(P - 1) * Jmax, D_psi_Hyx_1);
  rec("psi_Hyx_2", 'f', (int64_t)(P - 1) * Jmax, D_psi_Hyx_2);
  rec("psi_Ezy_1", 'f', (int64_t)Imax * P, D_psi_Ezy_1);
  rec("psi_Ezy_2", 'f', (int64_t)Imax * P, D_psi_Ezy_2);
  rec("psi_Hxy_1", 'f', (int64_t)Imax * (P - 1), D_psi_Hxy_1);
  rec("psi_Hxy_2", 'f', (int64_t)Imax * (P - 1), D_psi_Hxy_2);
  std::fclose(g_out);
  return 0;
}
