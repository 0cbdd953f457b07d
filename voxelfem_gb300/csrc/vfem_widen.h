/* FP32 -> FP64 widening on the integer units. Shared by the CUDA vector kernels (where an
 * FP64-pipe conversion per degree of freedom costs as much as an FMA) and by the host test
 * that checks it against the C conversion for every float. */
#ifndef VFEM_WIDEN_H
#define VFEM_WIDEN_H

#include <stdint.h>

#if defined(__CUDACC__)
#define VFEM_WIDEN_FN __host__ __device__ __forceinline__
#else
#define VFEM_WIDEN_FN static inline
#endif

VFEM_WIDEN_FN int vfem_clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __clz((int)x);
#else
    return __builtin_clz(x);
#endif
}

/* IEEE-754 binary32 bit pattern -> the binary64 bit pattern of the same value.
 * Normal numbers rebias the exponent by 1023 - 127 = 896 and move the mantissa from 23 to 52
 * bits. A subnormal m * 2^-149 whose leading one is bit p becomes (1 + f) * 2^(p - 149):
 * exponent field p + 874, fraction (m - 2^p) << (52 - p). Zeros keep their sign; infinities
 * and NaNs keep sign and payload, NaNs with the quiet bit set. */
VFEM_WIDEN_FN uint64_t vfem_widen_bits(uint32_t b) {
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint32_t e = (b >> 23) & 0xffu;
    const uint32_t m = b & 0x7fffffu;
    if (e == 0xffu) return sign | (0x7ffull << 52) | ((uint64_t)m << 29) | (m ? (1ull << 51) : 0ull);
    if (e == 0u) {
        if (m == 0u) return sign;
        const int p = 31 - vfem_clz32(m);
        return sign | ((uint64_t)(p + 874) << 52) | ((uint64_t)(m ^ (1u << p)) << (52 - p));
    }
    return sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
}

#endif
