/*
 * Host-side stand-in for the CUDA runtime, used ONLY to compile the
 * reference program's own sources for the CPU (oracle/ref_build.py).  TEST
 * INFRASTRUCTURE: kernels become plain functions that EMU_LAUNCH calls once
 * per emulated thread, serially, with blockIdx/threadIdx/blockDim/gridDim set
 * as CUDA would; "device" memory is host memory.  Nothing here is linked into
 * the product.
 */
#ifndef REF_SHIM_CUDA_RUNTIME_H
#define REF_SHIM_CUDA_RUNTIME_H

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <algorithm>

using std::abs;

#define __global__
#define __device__
#define __host__
#define __constant__ static
#define __shared__ static

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern thread_local uint3 blockIdx, threadIdx;
extern thread_local dim3 blockDim, gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3 };
struct cudaDeviceProp { int maxThreadsPerBlock; char name[256]; };

/* Buffers carry 64 KiB of zeroed slack: the reference writes one detector row
   past its nMax-row buffers and reads SourceP[nMax] (kernel.cu:802, 653). */
void *ref_shim_alloc(size_t bytes);
static inline cudaError_t cudaMalloc(void **p, size_t bytes) { *p = ref_shim_alloc(bytes); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
static inline cudaError_t cudaFree(void *) { return cudaSuccess; }  /* kept for the harness' final dump */
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return cudaSuccess; }
template <class T> cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n, size_t off = 0,
                                                  cudaMemcpyKind = cudaMemcpyHostToDevice) {
    std::memcpy(reinterpret_cast<char *>(&sym) + off, src, n);
    return cudaSuccess;
}
/* maxThreadsPerBlock drives the reference's launch shapes; REF_MAX_THREADS
   overrides the 1024 of every GPU since Fermi (used to show which cells the
   reference's floor-divided grids leave out). */
static inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
    const char *e = std::getenv("REF_MAX_THREADS");
    p->maxThreadsPerBlock = e ? std::atoi(e) : 1024;
    std::strcpy(p->name, "emulated");
    return cudaSuccess;
}
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
static inline cudaError_t cudaDeviceReset() { return cudaSuccess; }
static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }

/* Serial launch: every (block, thread) of the grid, x fastest, as one call. */
#define EMU_LAUNCH(grid, block, ...)                                                    \
    do {                                                                                \
        const dim3 emu_g(grid), emu_b(block);                                           \
        gridDim = emu_g; blockDim = emu_b;                                              \
        for (unsigned bz = 0; bz < emu_g.z; ++bz)                                       \
        for (unsigned by = 0; by < emu_g.y; ++by)                                       \
        for (unsigned bx = 0; bx < emu_g.x; ++bx)                                       \
        for (unsigned tz = 0; tz < emu_b.z; ++tz)                                       \
        for (unsigned ty = 0; ty < emu_b.y; ++ty)                                       \
        for (unsigned tx = 0; tx < emu_b.x; ++tx) {                                     \
            blockIdx = uint3{bx, by, bz}; threadIdx = uint3{tx, ty, tz};                \
            __VA_ARGS__;                                                                \
        }                                                                               \
    } while (0)

/* MSVC secure-CRT calls the reference uses. */
static inline int fopen_s(FILE **f, const char *name, const char *mode) { *f = std::fopen(name, mode); return *f ? 0 : 1; }
static inline int _strtime_s(char *b, size_t n) { std::snprintf(b, n, "00:00:00"); return 0; }
static inline int _strdate_s(char *b, size_t n) { std::snprintf(b, n, "01/01/00"); return 0; }
template <size_t N> int sprintf_s(char (&b)[N], const char *fmt, ...) { va_list a; va_start(a, fmt); int r = std::vsnprintf(b, N, fmt, a); va_end(a); return r; }
template <size_t N> int strcat_s(char (&b)[N], const char *s) { std::strncat(b, s, N - std::strlen(b) - 1); return 0; }

#endif
