// Device-side description of one shot and the launch helpers shared by the
// step kernels and the C-ABI layer.  Host code fills DevShot once per shot and
// keeps an array of them in device memory; the kernels read it through a
// const pointer so one launch can advance many shots (the batched form).
#pragma once

#include <cstdint>
#include <new>
#include <cuda.h>
#include <cuda_runtime.h>

namespace fdtd2d {

// Point kinds in the per-row point table.  Within a row the table is sorted
// by (kind, column) so every source of a row is applied before any detector
// reads the cell, matching the reference order source -> detectors
// (FDTD_2D_Full/kernel.cu:2134, 2151-2157).
enum PointKind : int { kPointSource = 0, kPointDetEz = 1, kPointDetComp = 2 };

// Packed CPML table rows (each row has npml floats; H rows use npml-1).
enum CpmlRow : int {
  kBeX1 = 0, kCeX1, kBeX2, kCeX2, kBhX1, kChX1, kBhX2, kChX2,
  kBeY1, kCeY1, kBeY2, kCeY2, kBhY1, kChY1, kBhY2, kChY2, kCpmlRows
};

// Material-ID medium: per-material coefficients for the Ez cell (ID3) and the
// H cells (ID1 for Hx, ID2 for Hy).  kp is the Jz drive coefficient
// beta*ne; pec marks material 1 (FDTD_2D_Full/kernel.cu:435).
struct MatE { float ca, cb, kp, pec; };
struct MatH { float da, db; };

struct DevShot {
  int nx, ny, pitch, npml;
  int n_steps;
  int base_n;                 // global step offset (batched/serving shots)
  float ca, cb, da, db;       // uniform medium coefficients
  float ja;                   // Jz decay (1 - nu dt/2)/(1 + nu dt/2)
  float dx, dy;               // the float dx, dy the reference passes to the psi kernels

  const float* kp;            // [ny][pitch] Jz drive beta*ne (uniform medium), may be null
  const uint8_t* id1;         // [ny][pitch] material ids (material medium)
  const uint8_t* id2;
  const uint8_t* id3;
  const MatE* mat_e;          // [256]
  const MatH* mat_h;          // [256]

  // Field buffers: fb[b] holds [4 fields (Ez, Hx, Hy, Jz)][cells]; each
  // field array holds ny rows of `pitch` elements; column 0 of row 0 sits
  // kMargin elements into it, so every row has a zero margin on both sides
  // that bulk row copies may read as halo.  field_ptr() points at column 0.
  // Step n reads fb[(n-1)&1] and writes fb[n&1]; a launch may be given a
  // descriptor whose fb points elsewhere.  fb[2] and fb[3] are the extra
  // buffers of the two-step (temporally blocked) path, null without it: a
  // two-step launch reads fb[0] (state n-1) and writes fb[2] (state n+1),
  // and fb[1] (state n) on the ring cells its neighbours read.
  float* fb[4];
  int64_t cells;
  // CPML psi slab [2 ping-pong buffers][psi_buf]; within a buffer (side s = 0
  // low edge, 1 high edge):
  //   o_hxy: [s][r][pitch]  r in [0,P-2]   (Hx, y strips)
  //   o_ezy: [s][r][pitch]  r in [0,P-1]   (Ez, y strips; r = 0 unused)
  //   o_hyx: [s][j][P]      r in [0,P-2]   (Hy, x strips)
  //   o_ezx: [s][j][P]      r in [0,P-1]   (Ez, x strips; r = 0 unused)
  float* psi;
  int64_t psi_buf, o_ezy, o_hyx, o_ezx;   // o_hxy = 0
  const float* cpml;          // [kCpmlRows][P]
  const float* den_ex;        // [pitch] (entries >= nx-1 are zero)
  const float* den_hx;        // [pitch]
  const float* den_ey;        // [ny]
  const float* den_hy;        // [ny]
  // The denominators inside the CPML-free part of the grid, when each table
  // is constant there (den_ex and den_hx over columns [npml, nx-npml-1],
  // den_ey and den_hy over rows [npml, ny-npml-1]): den_c = (den_ex,
  // den_hx, den_ey, den_hy) there, and den_uniform = 1.  The two-step
  // kernel, whose cells and halo all lie inside that part, takes them as
  // launch constants instead of loading the tables (the same floats, so the
  // same bits); the host runs it only when den_uniform is set.
  int den_uniform;
  float den_c[4];

  // sources and detectors, by row
  const int* row_start;       // [ny+1] offsets into pts
  const int4* pts;            // (col, kind, element index, 0)
  // Source waveform s_e(n) and DFT twiddles are tabulated per step by
  // build_source_tables (FP64 math, once per shot) so the step kernel does no
  // transcendental work.
  const float* src_val;       // [n_steps+1][n_src]
  const double2* twiddle;     // [n_steps+1] (cos, sin)(2 pi f n dt)
  int n_src;
  int n_det, n_comp;
  int record;
  float* trace;               // [n_steps][n_det]
  float* ctrace;              // [n_steps][n_comp][3]  (Ez, Hx, Hy)
  double2* dft;               // [n_det]
  // Reference launch coverage per update kernel (material medium only):
  // a cell update with reference thread index l >= cov[k] is skipped.
  long long cov[8];
  // Field storage (FDTD2D_STORE_*): Ez, Hx, Hy, Jz and the drive map hold
  // F32, F16 or BF16 elements (fb and kp point at elements of that type);
  // stored = value * isc[a], value = stored * sc[a], sc a power of two per
  // array a in (Ez, Hx, Hy, Jz, drive).  Arithmetic is FP32 throughout.
  int store;
  float sc[5], isc[5];
};

enum FieldId : int { kEz = 0, kHx = 1, kHy = 2, kJz = 3 };

// Left margin of every field row (floats); also the right margin pitch adds.
constexpr int kMargin = 32;

__host__ __device__ inline float* field_ptr(const DevShot& S, int f, int b) {
  return S.fb[b] + (int64_t)f * S.cells + kMargin;
}

// The same for storage element type T (F32 storage: T = float).
template <class T>
__host__ __device__ inline T* field_ptr_t(const DevShot& S, int f, int b) {
  return reinterpret_cast<T*>(S.fb[b]) + (int64_t)f * S.cells + kMargin;
}

// Bytes per stored field element.
inline int store_bytes(int store) { return store == 0 ? 4 : 2; }

// Row pitch (floats) for nx columns: 128-byte rows with kMargin on each side.
inline int row_pitch(int nx) { return (nx + 31) / 32 * 32 + 2 * kMargin; }

// Floats per field buffer: ny rows plus slack so that a bulk copy of a row
// segment that runs past the last row's margin stays inside the allocation.
inline int64_t buffer_floats(int nx, int ny) { return (int64_t)(ny + 2) * row_pitch(nx) + 1024; }

// A unit of work is one warp-wide column block (128 cells) of one shot over a
// contiguous range of rows: (shot, i0, j0, j1).
constexpr int kCols = 128;
constexpr int kThreads = 256;

// Launch the fused register-streaming step for step n_global (minus the
// shot's base_n) of one shot over its `units`.  medium: 0 uniform, 1 ids.
cudaError_t launch_step(const DevShot& shot, const int4* units, int n_units,
                        int n_global, int medium, int n_warps_grid,
                        cudaStream_t stream);

// Launch capacity: number of warps the step kernel keeps resident at once.
int resident_warps(int medium, int device);

// What the persistent kernel's service warps do after each step, while the
// other warps run the next one: the wave-front tracker's lines (launch_rc's
// work, one warp per line) and the line probe (launch_line's), for the steps
// they cover.  Zero counts: none.
struct PersistAux {
  int n_rc;
  const int* scan_i;
  const int* max_i;
  int j_cut;
  float level;
  float* edge;                // [n_rc]
  int* spd;                   // [step][n_rc], row n-1 for step n
  int line_n, line_j, line_i0, line_first, line_last;
  float* line;                // [n - line_first][line_n]
  // Bound on each grid-barrier wait in ns (0: the default, 1 s), and a count
  // added to every barrier's target.  Both exist for the test that makes a
  // barrier wait run out (FDTD2D_WAIT_NS, FDTD2D_TEST_BARRIER_EXTRA read at
  // create): with bar_extra = 1 no barrier completes, each CTA gives up after
  // wait_ns, records the timeout and returns.  Normal runs leave both 0.
  unsigned long long wait_ns;
  int bar_extra;
};

// The register-streaming step for steps n_first..n_last (global numbering)
// in one cooperative launch of `ctas` CTAs (at most persist_resident_ctas):
// the warps step the units, a grid barrier (bounded in time; *err set when
// it gives out) between steps.  repeat > 0: step n_first `repeat` times
// instead (a timing trial: the same reads and writes each time).  bar: one
// device word the launch zeroes first.
cudaError_t launch_step_persist(const DevShot& shot, const int4* units, int n_units, int n_first, int n_last,
                                int repeat, const PersistAux& aux, int medium, int ctas, unsigned* bar, int* err,
                                cudaStream_t stream);
int persist_resident_ctas(int medium, int device);

// Device error codes written by kernels with bounded waits.
enum DeviceError : int { kErrNone = 0, kErrWaitTimeout = 1 };

// Runs the body of a C-ABI entry point so that no C++ exception crosses the
// ABI: a host allocation failure becomes FDTD2D_ERR_NOMEM (-2), anything
// else FDTD2D_ERR_INVALID (-1).
template <class F>
int abi_guard(F&& f) noexcept {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return -2;
  } catch (...) {
    return -1;
  }
}

// Shared-memory staged step (step_tma.cu), uniform medium: one CTA per unit
// of a band of columns.  Compiled launch shapes (warps per CTA, ring stages)
// are indexed 0..tma_shape_count()-1; shape 0 is the default.
int tma_shape_count();
int tma_shape_find(int warps, int stages);   // -1 if not compiled
void tma_shape_dims(int shape, int* warps, int* stages);
// "W,ST" -> shape index, -1 if not compiled
int tma_shape_parse(const char* text);
// "<kernel><W,ST>"
void tma_shape_name(int shape, const char* kernel, char* out, size_t n);
int tma_band_cols(int shape);
int tma_max_pml();   // largest CPML depth the staged kernel takes
int tma_resident_ctas(int shape, int npml, int store, int device);

// Tensor maps of one shot for the multi-row staged kernel (step_tmat.cu):
// Hx, Hy, Jz of field buffer b as one rank-3 tensor (column, row, field),
// Ez of buffer b and the drive map as rank-2 tensors (column, row); column 0
// of row 0 is the origin, columns outside [0, nx) and rows outside [0, ny)
// read as zero.
struct TensorMaps {
  CUtensorMap hj[4], e[4], k;   // per field-buffer slot, as DevShot::fb
};

// Multi-row staged kernel for the interior of a shot: units (0, c0, j0, j1)
// whose band and halo column lie outside the x strips and whose rows lie in
// [npml, ny - npml).  Shapes: (warps, rows per stage, stages).
int tmat_shape_count();
int tmat_shape_find(int warps, int rows, int stages);   // -1 if not compiled
void tmat_shape_dims(int shape, int* warps, int* rows, int* stages);
int tmat_band_cols(int shape);
int tmat_box_cols(int shape);   // columns per tensor box (band + 16 halo = boxes x box_cols)
int tmat_rows(int shape);
int tmat_resident_ctas(int shape, int store, int device);
cudaError_t launch_step_tmat(int shape, const DevShot& shot, const TensorMaps& maps, const int4* units,
                             int n_units, int n_global, int max_ctas, int* err, cudaStream_t stream);

// Two-step (temporally blocked) form of the same kernel: steps n and n+1 of
// units (flags, c0, j0, j1) in one pass over state n-1, with n = n_global -
// base_n.  The units tile a region R = [ring.x, ring.y) x [ring.z, ring.w)
// whose cells and 1-cell surround have no CPML; each unit recomputes step n
// one cell around itself and writes state n+1 to slot 2 (bits 4-6 of flags:
// the unit's leading warps left of R).  State n of R's edge cells goes to
// slot 1, for the CPML-band kernel's step n+1: with FP32 storage from the
// units next to them (flags kRing*), with 16-bit storage from ring units
// (kUnitRing, t0, t1, 0: edge cells t0 .. t1-1, rows ring.z and ring.w-1,
// then columns ring.x and ring.y-1).  CTAs take units in turn from *ctr,
// which must be 0 at launch (launch_frame resets it).
enum UnitFlags : int { kRingTop = 1, kRingBottom = 2, kRingLeft = 4, kRingRight = 8, kUnitRing = 256 };
int tmat2_resident_ctas(int shape, int store, int device);
cudaError_t launch_step_tmat2(int shape, const DevShot& shot, const TensorMaps& maps, const int4* units,
                              int n_units, int n_global, int4 ring, int max_ctas, int* ctr, int* err,
                              cudaStream_t stream);
// Step n (n_global - base_n) of the 2-cell frame around R = [ci0, ci1) x
// [ri0, ri1) (columns [ci0-2, ci1+2) x rows [ri0-2, ri1+2), minus R) from
// slot (n-1)&1 into slot n&1, sources applied, detectors left to the CPML
// band kernel; the frame and its 1-cell surround must lie outside the CPML.
// Sets *ctr = 0.
cudaError_t launch_frame(const DevShot& shot, int ci0, int ci1, int ri0, int ri1, int n_global, int* ctr,
                         cudaStream_t stream);
// Launches the instantiation for shot.store.
cudaError_t launch_step_tma(int shape, const DevShot& shot, const int4* units, int n_units, int n_global,
                            int max_ctas, int* err, cudaStream_t stream);
// Batched form: one launch advances every shot in `shots` by one step, units
// (shot, c0, j0, j1) handed out dynamically; n_global = *gstep + k + 1.
// counters: 2 ints, zero before the first launch.
cudaError_t launch_step_tma_batch(int shape, const DevShot* shots, const int4* units, const int* n_units,
                                  const int* gstep, int k, int* counters, int max_pml, int ctas, int* err,
                                  cudaStream_t stream);
int tma_batch_resident_ctas(int shape, int max_pml, int device);

// Tabulate s_e(n) = scale*env[n]*cos(2*pi_c*(beta/2 t^2 + f0 t + phase_e)),
// t = n*dt, for n = 0..n_steps, and the DFT twiddles, in FP64.
cudaError_t build_source_tables(float* src_val, double2* twiddle, const float* env,
                                const double* phase_cycles, int n_src, int n_steps, double dt,
                                double scale, double f0, double beta_half, double src_pi,
                                double dft_fdt, cudaStream_t stream);

// Wave-front tracker for one step: one CTA per line (see fdtd2d_setup.n_rc).
cudaError_t launch_rc(const float* ez, int64_t pitch, int ny, int n_rc, const int* scan_i,
                      const int* max_i, int j_cut, float level, float* edge, int* spd_row,
                      cudaStream_t stream);

// Copy n cells of row j starting at column i0 into dst.
cudaError_t launch_line(const float* ez, int64_t pitch, int j, int i0, int n, float* dst,
                        cudaStream_t stream);

// Count non-finite values in n floats (atomic count into *flag).
cudaError_t launch_nonfinite(const float* a, int64_t n, int* flag, cudaStream_t stream);
cudaError_t launch_nonfinite16(const uint16_t* a, int64_t n, bool bf16, int* flag, cudaStream_t stream);
// n FP32 values to F16 (store 1) or BF16 (store 2) elements, times isc.
cudaError_t launch_to_storage(const float* src, void* dst, int64_t n, int store, float isc, cudaStream_t stream);

}  // namespace fdtd2d
