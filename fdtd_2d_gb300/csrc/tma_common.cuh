// Device helpers shared by the staged step kernels (step_tma.cu: one row per
// ring stage, 1-D bulk copies; step_tmat.cu: several rows per stage, tensor
// copies): mbarrier waits bounded in time, bulk copies, and the loads and
// stores of the field storage types.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace fdtd2d {
namespace {

constexpr uint64_t kWaitNs = 1000000000ull;   // 1 s bound on any barrier wait

// Loads and stores of 4 consecutive stored elements (and of one), converted
// to / from FP32 with the array's power-of-two scale.
template <class T>
struct Sto;

template <>
struct Sto<float> {
  __device__ static __forceinline__ void lds4(float (&d)[4], const float* p, float) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
  }
  __device__ static __forceinline__ void ldg4(float (&d)[4], const float* p, float) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
  }
  __device__ static __forceinline__ float ld1(const float* p, float) { return *p; }
  __device__ static __forceinline__ float ldg1(const float* p, float) { return __ldg(p); }
  __device__ static __forceinline__ void stcs4(float* p, const float (&d)[4], float) {
    __stcs(reinterpret_cast<float4*>(p), make_float4(d[0], d[1], d[2], d[3]));
  }
  __device__ static __forceinline__ void st1(float* p, float v, float) { *p = v; }
  // The value a store followed by a load gives back (F32: the value itself).
  __device__ static __forceinline__ void rt4(float (&o)[4], const float (&d)[4], float, float) {
    o[0] = d[0]; o[1] = d[1]; o[2] = d[2]; o[3] = d[3];
  }
  __device__ static __forceinline__ float rt1(float v, float, float) { return v; }
  // The same in stored units (no scale).
  __device__ static __forceinline__ void lds4(float (&d)[4], const float* p) { lds4(d, p, 1.f); }
  __device__ static __forceinline__ void ldg4(float (&d)[4], const float* p) { ldg4(d, p, 1.f); }
  __device__ static __forceinline__ float ld1(const float* p) { return *p; }
  __device__ static __forceinline__ float ldg1(const float* p) { return __ldg(p); }
  __device__ static __forceinline__ void stcs4(float* p, const float (&d)[4]) { stcs4(p, d, 1.f); }
  __device__ static __forceinline__ void st1(float* p, float v) { *p = v; }
  __device__ static __forceinline__ void rt4(float (&o)[4], const float (&d)[4]) { rt4(o, d, 1.f, 1.f); }
  __device__ static __forceinline__ float rt1(float v) { return v; }
};

template <class T, class T2>
struct Sto16 {
  __device__ static __forceinline__ float2 to_f2(uint32_t w);
  __device__ static __forceinline__ uint32_t from_f2(float a, float b);
};

template <>
__device__ __forceinline__ float2 Sto16<__half, __half2>::to_f2(uint32_t w) {
  __half2 h;
  memcpy(&h, &w, 4);
  return __half22float2(h);
}
template <>
__device__ __forceinline__ uint32_t Sto16<__half, __half2>::from_f2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  uint32_t w;
  memcpy(&w, &h, 4);
  return w;
}
template <>
__device__ __forceinline__ float2 Sto16<__nv_bfloat16, __nv_bfloat162>::to_f2(uint32_t w) {
  __nv_bfloat162 h;
  memcpy(&h, &w, 4);
  return __bfloat1622float2(h);
}
template <>
__device__ __forceinline__ uint32_t Sto16<__nv_bfloat16, __nv_bfloat162>::from_f2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  uint32_t w;
  memcpy(&w, &h, 4);
  return w;
}

template <class T, class T2>
struct Sto16Ops {
  using B = Sto16<T, T2>;
  __device__ static __forceinline__ void cvt(float (&d)[4], uint2 v, float sc) {
    const float2 a = B::to_f2(v.x), b = B::to_f2(v.y);
    d[0] = a.x * sc; d[1] = a.y * sc; d[2] = b.x * sc; d[3] = b.y * sc;
  }
  __device__ static __forceinline__ void lds4(float (&d)[4], const T* p, float sc) {
    cvt(d, *reinterpret_cast<const uint2*>(p), sc);
  }
  __device__ static __forceinline__ void ldg4(float (&d)[4], const T* p, float sc) {
    cvt(d, __ldg(reinterpret_cast<const uint2*>(p)), sc);
  }
  __device__ static __forceinline__ float ld1(const T* p, float sc) {
    uint16_t u;
    memcpy(&u, p, 2);
    return B::to_f2((uint32_t)u).x * sc;
  }
  __device__ static __forceinline__ float ldg1(const T* p, float sc) {
    const uint16_t u = __ldg(reinterpret_cast<const unsigned short*>(p));
    return B::to_f2((uint32_t)u).x * sc;
  }
  __device__ static __forceinline__ void stcs4(T* p, const float (&d)[4], float isc) {
    uint2 v;
    v.x = B::from_f2(d[0] * isc, d[1] * isc);
    v.y = B::from_f2(d[2] * isc, d[3] * isc);
    __stcs(reinterpret_cast<uint2*>(p), v);
  }
  __device__ static __forceinline__ void st1(T* p, float v, float isc) {
    const uint16_t u = (uint16_t)(B::from_f2(v * isc, 0.f) & 0xffffu);
    memcpy(p, &u, 2);
  }
  // stcs4 then lds4 (st1 then ld1) of the same element, without the memory
  // round trip: the same conversions, so the same bits.
  __device__ static __forceinline__ void rt4(float (&o)[4], const float (&d)[4], float isc, float sc) {
    uint2 v;
    v.x = B::from_f2(d[0] * isc, d[1] * isc);
    v.y = B::from_f2(d[2] * isc, d[3] * isc);
    cvt(o, v, sc);
  }
  __device__ static __forceinline__ float rt1(float v, float isc, float sc) {
    return B::to_f2(B::from_f2(v * isc, 0.f) & 0xffffu).x * sc;
  }
  // The same in stored units: the value the element holds, no scale.
  __device__ static __forceinline__ void cvt(float (&d)[4], uint2 v) {
    const float2 a = B::to_f2(v.x), b = B::to_f2(v.y);
    d[0] = a.x; d[1] = a.y; d[2] = b.x; d[3] = b.y;
  }
  __device__ static __forceinline__ void lds4(float (&d)[4], const T* p) {
    cvt(d, *reinterpret_cast<const uint2*>(p));
  }
  __device__ static __forceinline__ void ldg4(float (&d)[4], const T* p) {
    cvt(d, __ldg(reinterpret_cast<const uint2*>(p)));
  }
  __device__ static __forceinline__ float ld1(const T* p) {
    uint16_t u;
    memcpy(&u, p, 2);
    return B::to_f2((uint32_t)u).x;
  }
  __device__ static __forceinline__ float ldg1(const T* p) {
    const uint16_t u = __ldg(reinterpret_cast<const unsigned short*>(p));
    return B::to_f2((uint32_t)u).x;
  }
  __device__ static __forceinline__ void stcs4(T* p, const float (&d)[4]) {
    uint2 v;
    v.x = B::from_f2(d[0], d[1]);
    v.y = B::from_f2(d[2], d[3]);
    __stcs(reinterpret_cast<uint2*>(p), v);
  }
  __device__ static __forceinline__ void st1(T* p, float v) {
    const uint16_t u = (uint16_t)(B::from_f2(v, 0.f) & 0xffffu);
    memcpy(p, &u, 2);
  }
  __device__ static __forceinline__ void rt4(float (&o)[4], const float (&d)[4]) {
    uint2 v;
    v.x = B::from_f2(d[0], d[1]);
    v.y = B::from_f2(d[2], d[3]);
    cvt(o, v);
  }
  __device__ static __forceinline__ float rt1(float v) { return B::to_f2(B::from_f2(v, 0.f) & 0xffffu).x; }
};

template <>
struct Sto<__half> : Sto16Ops<__half, __half2> {};
template <>
struct Sto<__nv_bfloat16> : Sto16Ops<__nv_bfloat16, __nv_bfloat162> {};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the barrier's phase `parity` to complete, for at most kWaitNs of
// wall time (a try_wait may itself suspend for a while, so the bound is on
// time, not on the number of polls).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  for (int it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (it == 0) {
      t0 = global_ns();
    } else if ((it & 15) == 0 && global_ns() - t0 > kWaitNs) {
      return false;
    }
  }
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void lds4f(float (&d)[4], const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}

}  // namespace
}  // namespace fdtd2d
