// Double-float arithmetic on the FP32 units: a value is an unevaluated pair hi + lo of floats.
#pragma once
#include <cuda_runtime.h>

namespace vfem {

__device__ __forceinline__ void df_split(double v, float &hi, float &lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// (sh, sl) += a*b with a = (ah, al), b = (bh, bl) (error-free product of the high parts)
__device__ __forceinline__ void df_fma_acc(float ah, float al, float bh, float bl, float &sh, float &sl) {
    const float p = ah * bh;
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = sh + p;
    const float bp = t - sh;
    const float err = (sh - (t - bp)) + (p - bp);
    sh = t;
    sl += err + e;
}

}  // namespace vfem
