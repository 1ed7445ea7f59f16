// fr_device.cuh -- device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <limits.h>

namespace fr {

// float -> int as the reference's x86-64 build converts (cvttss2si):
// NaN and out-of-range values give INT_MIN.
__device__ __forceinline__ int f2i_ref(float v)
{
    return (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : INT_MIN;
}

// Clamped cell range of one component, GridLut.cpp:98-106:
//   start = max(ceil(c - kHW), 0), end = min(floor(c + kHW), G - 1)
// with the subtraction/addition rounded in float like the reference.
__device__ __forceinline__ void comp_range(float c, float hw, unsigned G, int &s, int &e)
{
    int st = f2i_ref(ceilf(__fsub_rn(c, hw)));
    int en = f2i_ref(floorf(__fadd_rn(c, hw)));
    s = st > 0 ? st : 0;
    int gm1 = (int)(G - 1u);
    e = en < gm1 ? en : gm1;
}

// Kernel LUT index of one tap, GridLut.cpp:120-136:
//   dk = sqrtf(dz^2 + dy^2 + dx^2) (summed in that order, no fused
//   multiply-add), valid when dk < kHW, index round(dk / kHW * (L - 1)).
// Returns -1 for taps outside the kernel radius.
__device__ __forceinline__ int tap_index(float dx, float dy2, float dz2, float hw, float inv_hw,
                                         bool hw_pow2, float lm1, int L)
{
    float s = __fadd_rn(__fadd_rn(dz2, dy2), __fmul_rn(dx, dx));
    float dk = __fsqrt_rn(s);
    if (!(dk < hw)) return -1;
    // x / 2^k and x * 2^-k are the same correctly rounded value.
    float q = hw_pow2 ? __fmul_rn(dk, inv_hw) : __fdiv_rn(dk, hw);
    int ki = (int)roundf(__fmul_rn(q, lm1));
    return ki < L ? ki : L - 1;
}

}  // namespace fr
