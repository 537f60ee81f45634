// Small device helpers shared by the absorption, gridding and interpolation
// kernels.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace anacor {

// exp(-x) in FP32 after an FP64 reduction x = k ln2 + r, |r| <= ln2/2.
__device__ __forceinline__ float exp_neg(double x)
{
    const double kd = rint(__dmul_rn(x, 1.4426950408889634));
    const double r = __fma_rn(-kd, 0.6931471805599453, x);
    const float e = expf(-(float)r);
    const int k = (int)fmaxf(fminf((float)kd, 400.0f), -400.0f);
    return ldexpf(e, -k);
}

// Knuth's TwoSum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

}  // namespace anacor
