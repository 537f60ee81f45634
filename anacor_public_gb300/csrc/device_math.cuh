// Small device helpers shared by the absorption, gridding and interpolation
// kernels.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace anacor {

// exp(-x) = 2^-k exp(-r) with the additive range reduction of exp by
// multiples of ln 2 (Cody and Waite, "Software Manual for the Elementary
// Functions", 1980, the exp chapter): k = rint(x / ln2), r = x - k ln2 in FP64
// (one FP64 constant instead of their two-part split: the rounding of k ln2,
// ~1e-16 k, is far below FP32's resolution), then CUDA's expf on the FP32 r,
// |r| <= ln2/2, and an exact scaling by 2^-k.
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
