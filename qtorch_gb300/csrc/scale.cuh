// Per-tensor power-of-two scaling of the mixed form when a plan runs step by
// step (one whole-GPU launch per step).
//
// Every step output owns a ScaleWord in device memory: the float bits of the
// largest magnitude max(|re|, |im|) stored in it, and its exponent E (the
// tensor's true values are the stored ones times 2^E).  A consumer reads its
// producers' words, scales its sums by 2^-(mA + mB), where m is the exponent
// of a producer's stored maximum (max = f 2^m, f in [0.5, 1)), and records
// E_C = E_A + E_B + mA + mB.  Stored values therefore stay within a factor
// 4^K of 1 whatever the network's true magnitudes; leaves (null words) are
// used as they are.  The words are zeroed before the first step; the kernels
// of a step raise max with one atomicMax per warp (non-negative floats order
// as their bit patterns, so inf and NaN end up above every finite value and
// are seen by the host).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace qtg {

struct ScaleWord {
    uint32_t maxbits;
    int32_t expo;
};

struct StepScaleRef {
    const ScaleWord *a = nullptr;   // producer of A (null: a leaf or no scaling)
    const ScaleWord *b = nullptr;
    ScaleWord *c = nullptr;         // this step's output (null: not tracked)
};

#ifdef __CUDACC__
// exponent m of a stored maximum (0 for a leaf, an all-zero tensor, inf or NaN)
__device__ __forceinline__ int scale_word_exp(const ScaleWord *w) {
    if (!w) return 0;
    const uint32_t bits = w->maxbits;
    const uint32_t ex = (bits >> 23) & 0xffu;
    if (ex == 0xffu || bits == 0) return 0;
    if (ex == 0) {   // a subnormal maximum
        int e;
        frexpf(__uint_as_float(bits), &e);
        return e;
    }
    return (int) ex - 126;
}

// the shift a consumer applies to its sums: -(mA + mB)
__device__ __forceinline__ int scale_shift(const StepScaleRef &s) {
    return -(scale_word_exp(s.a) + scale_word_exp(s.b));
}

// exact multiplication by 2^e
__device__ __forceinline__ float scale_pow2(float x, int e) {
    return (e >= -126 && e <= 127) ? x * __int_as_float((127 + e) << 23) : ldexpf(x, e);
}

// Magnitudes are tracked as the bit patterns of |x|: an integer maximum keeps
// NaN (whose |x| bits lie above those of inf), which fmaxf would drop.
__device__ __forceinline__ uint32_t mag_bits(float2 v) {
    return max(__float_as_uint(fabsf(v.x)), __float_as_uint(fabsf(v.y)));
}

// Fold a thread's largest stored magnitude (mag_bits) into the step's word --
// the whole warp calls this together -- and, from thread 0 of the step's first
// CTA, write E_C.
__device__ __forceinline__ void scale_note(const StepScaleRef &s, uint32_t local_maxbits, int shift,
                                           bool first_cta) {
    if (!s.c) return;
    const uint32_t wmax = __reduce_max_sync(0xffffffffu, local_maxbits);
    if ((threadIdx.x & 31u) == 0 && wmax) atomicMax(&s.c->maxbits, wmax);
    if (first_cta && threadIdx.x == 0) {
        const int ea = s.a ? s.a->expo : 0, eb = s.b ? s.b->expo : 0;
        s.c->expo = ea + eb - shift;
    }
}
#endif

}  // namespace qtg
