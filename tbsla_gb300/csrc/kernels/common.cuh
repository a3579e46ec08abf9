// Device helpers shared by the SpMV kernels: cache-policy loads, value
// widening, warp / block reductions.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace tbsla_gpu {

constexpr int kWarp = 32;

// L2 policy for data read exactly once (matrix values and indices): evict
// first, so the gathered vector x keeps the L2.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// Streaming loads: read-only path, no L1 allocation, L2 policy operand.
__device__ __forceinline__ double ld_stream(const double* p, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;"
               : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* p, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;"
               : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ __nv_bfloat16 ld_stream(const __nv_bfloat16* p, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;"
               : "=h"(v) : "l"(p), "l"(pol));
  __nv_bfloat16 r;
  *reinterpret_cast<unsigned short*>(&r) = v;
  return r;
}
__device__ __forceinline__ int ld_stream(const int* p, uint64_t pol) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;"
               : "=r"(v) : "l"(p), "l"(pol));
  return v;
}

// Gathered vector entries: read-only path with L1 allocation (the near-
// diagonal part of a row block hits L1).
__device__ __forceinline__ double ld_gather(const double* p) { return __ldg(p); }

// Narrowing to the storage precision, round to nearest even.  bfloat16 is
// rounded from the double's bits directly (no intermediate float rounding):
// add half an ulp of the 8-bit significand (ties to even), drop the low 45
// mantissa bits, and the result is exact in float.
template <class V>
__device__ __forceinline__ V narrow(double v);
template <>
__device__ __forceinline__ double narrow<double>(double v) { return v; }
template <>
__device__ __forceinline__ float narrow<float>(double v) { return __double2float_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 narrow<__nv_bfloat16>(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  if ((b & 0x7ff0000000000000ull) != 0x7ff0000000000000ull) {  // finite
    b += (1ull << 44) - 1 + ((b >> 45) & 1);
    b &= ~((1ull << 45) - 1);
  }
  const float f = (float)__longlong_as_double((long long)b);
  const unsigned u = __float_as_uint(f);
  unsigned short h = (unsigned short)(u >> 16);
  __nv_bfloat16 r;
  *reinterpret_cast<unsigned short*>(&r) = h;
  return r;
}

// Widening to double.  GB300's FP64 pipe is narrow (about 1/64 of FP32), so
// float -> double is done on the integer pipes for normal numbers and zero:
// re-bias the exponent (+896 = 1023 - 127) and move the mantissa up 29 bits,
// which is exact; subnormals, infinities and NaNs take the hardware path.
__device__ __forceinline__ double widen_bits(unsigned u) {
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0u) {
    if ((u & 0x7fffffu) == 0u) return __longlong_as_double((long long)sign);
    return (double)__uint_as_float(u);
  }
  if (e == 0xffu) return (double)__uint_as_float(u);
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return widen_bits(__float_as_uint(v)); }
__device__ __forceinline__ double widen(__nv_bfloat16 v) {
  return widen_bits((unsigned)(*reinterpret_cast<const unsigned short*>(&v)) << 16);
}

// Fused multiply-add, one FP64 instruction per matrix entry.
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// Product and sum with explicit rounding (no FMA contraction), so a row
// summed by one thread reproduces the reference loop's rounding exactly.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = add_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum over the whole CTA (NT threads); result valid in thread 0.
// `scratch` holds NT/32 doubles; the call ends with __syncthreads().
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* scratch) {
  v = warp_sum(v);
  const int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
  if (l == 0) scratch[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NT / kWarp; i++) r = add_rn(r, scratch[i]);
  }
  __syncthreads();
  return r;
}

// Opts `Kernel` in to `smem` bytes of dynamic shared memory on the current
// device.  The attribute belongs to each device's context, so it is set once
// per device ordinal and kernel instantiation (a bit per device; ordinals
// past 63 set it on every call).
template <auto Kernel>
cudaError_t smem_opt_in(size_t smem) {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

}  // namespace tbsla_gpu
