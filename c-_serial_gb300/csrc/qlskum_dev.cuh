// Device helpers shared by the mixed kernels and their reverse: conversions
// between FP32 and FP64 on the integer pipe (the hardware conversion issues
// on the FP64 pipe, which on this chip is the scarce one) and the cp.async
// copies of the staged neighbour gathers (global -> the thread's own shared
// memory; 16- and 8-byte copies need 16- / 8-byte aligned addresses).
#pragma once

#include <cuda_runtime.h>

namespace qlskum {

// float -> double: exact for normal numbers and zero, flushes subnormals to
// zero and keeps Inf / NaN.
__device__ __forceinline__ double f2d(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7fffffffu;
    const unsigned sign = b & 0x80000000u;
    unsigned hi = sign | (((mag >> 23) + 896u) << 20) | ((mag & 0x7fffffu) >> 3);
    unsigned lo = b << 29;
    if (mag < 0x00800000u) { hi = sign; lo = 0u; }
    if (mag >= 0x7f800000u) hi = sign | 0x7ff00000u | ((mag & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)lo);
}

// double -> float on the integer pipe, truncating the mantissa (< 1 ulp);
// underflow goes to zero, overflow and Inf to Inf, NaN stays NaN.
__device__ __forceinline__ float d2f(double x)
{
    const unsigned h = (unsigned)__double2hiint(x), l = (unsigned)__double2loint(x);
    const unsigned mag = h & 0x7fffffffu;
    const unsigned sign = h & 0x80000000u;
    const int e = (int)(mag >> 20) - 896;
    const unsigned m = ((mag & 0xfffffu) << 3) | (l >> 29);
    unsigned b = sign | ((unsigned)e << 23) | m;
    if (e <= 0) b = sign;
    if (e >= 255) b = sign | 0x7f800000u | ((mag >= 0x7ff00000u && (m | (mag & 0xfffffu) | l)) ? 0x400000u : 0u);
    return __uint_as_float(b);
}

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

}  // namespace qlskum
