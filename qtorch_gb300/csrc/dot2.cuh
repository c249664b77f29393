// Compensated FP32 arithmetic shared by the reduction kernels (kernels.cu,
// permute.cu).
#pragma once
#include <cuda_runtime.h>

namespace qtg {

// Compensated FP32 dot product (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005, algorithm Dot2): the running sum
// is p + s, every product is split exactly into h + r with one FMA (TwoProduct)
// and every addition into p + q (Knuth's TwoSum); the errors q + r are summed
// in s.  The result is as accurate as an FP32 loop run in twice the working
// precision, and it runs on the FP32 pipe, which on GB300 is many times wider
// than the FP64 one.  The _rn intrinsics keep the compiler from fusing the
// error-free transformations into FMAs.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void dot2_acc(float &p, float &s, float x, float y) {
    const float h = __fmul_rn(x, y);
    const float r = __fmaf_rn(x, y, -h);
    float q, np;
    two_sum(p, h, np, q);
    p = np;
    s = __fadd_rn(s, __fadd_rn(q, r));
}

__device__ __forceinline__ void cmac_dot2(float &pre, float &sre, float &pim, float &sim, float2 a, float2 b) {
    dot2_acc(pre, sre, a.x, b.x);
    dot2_acc(pre, sre, -a.y, b.y);
    dot2_acc(pim, sim, a.x, b.y);
    dot2_acc(pim, sim, a.y, b.x);
}

// (p1 + s1) += (p2 + s2)
__device__ __forceinline__ void dot2_merge(float &p, float &s, float p2, float s2) {
    float np, q;
    two_sum(p, p2, np, q);
    p = np;
    s = __fadd_rn(s, __fadd_rn(s2, q));
}

}  // namespace qtg
