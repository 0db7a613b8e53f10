// Allocation-free variant of the non-finite scan (fdtd2d_check_finite).
//
// Who needs it: code that must not call cudaMalloc -- for example a host
// application that hands this library device buffers from its own memory
// pool and forbids other allocations, code running where an allocation would
// synchronise the device or break a latency budget, or a caller that checks a
// buffer it does not own through a context.  fdtd2d_check_finite needs a
// context (created with cudaMalloc) and a counter allocated with it; this
// entry point takes a plain device pointer and keeps its scratch in a
// fixed-size array that lives in this library's module for the whole process.
//
// Scratch: kPartials per-block partial counts plus one total, in a
// file-scope __device__ array.  Every GPU that loads the library holds it
// (16 KiB) until the process exits.  Each call overwrites every slot it reads,
// so nothing has to be zeroed between calls, but all calls share the one
// array: calls whose GPU work overlaps (different streams, or host threads
// using the same device) race on it and must be serialised by the caller.
#include "../../include/fdtd2d.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

namespace {

constexpr int kPartials = 2048;                 // one slot per block
constexpr int64_t kChunk = int64_t(1) << 20;    // values scanned per block
constexpr int64_t kMaxValues = kPartials * kChunk;  // 2^31 values per call
constexpr int kThreads = 256;

// [0, kPartials): per-block counts; [kPartials]: the total.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kPartials + 1];

__global__ void count_nonfinite_partial(const float* __restrict__ a, int64_t n,
                                        unsigned long long* __restrict__ partial) {
  const int64_t begin = (int64_t)blockIdx.x * kChunk;
  const int64_t end = begin + kChunk < n ? begin + kChunk : n;
  unsigned long long c = 0;
  for (int64_t t = begin + threadIdx.x; t < end; t += blockDim.x) c += !isfinite(a[t]);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ unsigned long long s[kThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long sum = 0;
    for (int w = 0; w < kThreads / 32; ++w) sum += s[w];
    partial[blockIdx.x] = sum;  // every launched block writes its slot
  }
}

__global__ void count_nonfinite_total(unsigned long long* __restrict__ scratch, int blocks) {
  unsigned long long c = 0;
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) c += scratch[b];
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ unsigned long long s[kThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long sum = 0;
    for (int w = 0; w < kThreads / 32; ++w) sum += s[w];
    scratch[kPartials] = sum;
  }
}

// Device address of the scratch array, looked up once per device context.
// The runtime resolves the symbol for the current device's primary context;
// a device reset (cudaDeviceReset) destroys that context and the module's
// memory with it, and the next use creates a new context where the array
// has another address.  So the cached address is kept together with the
// identity of the context it was resolved in (cuCtxGetId, through the
// runtime's driver entry points) and resolved again when that changes.
// Where the identity cannot be read, the address is resolved on every call.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct CtxFns {
  CtxGetCurrentFn current = nullptr;
  CtxGetIdFn id = nullptr;
};

const CtxFns& ctx_fns() {
  static const CtxFns fns = [] {
    CtxFns f;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f.current = reinterpret_cast<CtxGetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f.id = reinterpret_cast<CtxGetIdFn>(p);
    return f;
  }();
  return fns;
}

// Identity of the calling thread's current context, 0 when unknown.
unsigned long long current_ctx_id() {
  const CtxFns& f = ctx_fns();
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (f.current && f.id && f.current(&ctx) == CUDA_SUCCESS && ctx && f.id(ctx, &id) == CUDA_SUCCESS) return id;
  return 0;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned long long* g_ptr[kMaxDevices] = {};
unsigned long long g_ctx[kMaxDevices] = {};

int scratch_for_current_device(unsigned long long** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FDTD2D_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  const unsigned long long id = current_ctx_id();
  if (!g_ptr[dev] || id == 0 || id != g_ctx[dev]) {
    void* p = nullptr;
    // The symbol's host-side name is only a stand-in; the kernels need the
    // device address, which the runtime resolves for the current device
    // (creating its primary context if there is none yet).
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FDTD2D_ERR_CUDA;
    g_ptr[dev] = static_cast<unsigned long long*>(p);
    g_ctx[dev] = current_ctx_id();   // the context the address belongs to
  }
  *out = g_ptr[dev];
  return FDTD2D_OK;
}

}  // namespace

extern "C" int fdtd2d_check_finite_noalloc(const float* d_data, int64_t n, int64_t* nonfinite,
                                           void* stream) {
  if (nonfinite) *nonfinite = 0;
  if (n < 0 || (n > 0 && !d_data)) return FDTD2D_ERR_INVALID;
  if (n > kMaxValues) return FDTD2D_ERR_RANGE;  // more values than the fixed scratch covers
  if (n == 0) return FDTD2D_OK;
  unsigned long long* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = (int)((n + kChunk - 1) / kChunk);
  count_nonfinite_partial<<<blocks, kThreads, 0, s>>>(d_data, n, scratch);
  count_nonfinite_total<<<1, kThreads, 0, s>>>(scratch, blocks);
  unsigned long long total = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, scratch + kPartials, sizeof(total), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? FDTD2D_ERR_NOMEM : FDTD2D_ERR_CUDA;
  if (nonfinite) *nonfinite = (int64_t)total;
  return total ? FDTD2D_ERR_NONFINITE : FDTD2D_OK;
}
