// CUDA kernels of the contraction engine (sm_103a).
//
//  * pair_kernel<double>: one pairwise contraction over the whole GPU, FP64,
//    every output element accumulated sequentially over k in the reference's
//    order with separately rounded multiplies and adds (no FMA contraction),
//    which reproduces src/Network.h:876-971 bit for bit.
//  * pair_kernel<float>: the same contraction in complex64 with FP32 FMA.
//  * plan_kernel<Mode>: the grouped interpreter.  One CTA runs one plan
//    instance (a whole network) level by level: all steps of a dependency
//    level run concurrently across the CTA's threads, tiny outputs split their
//    k loop over lane groups that finish with warp shuffles (mixed mode), and
//    intermediates stay in a shared-memory (small plans) or global per-CTA
//    workspace.  Mixed mode keeps every intermediate normalised by a power of
//    two (per-tensor exponent) and accumulates the expectation-value
//    reductions with compensated FP32 dot products (no FP64 arithmetic).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "engine.cuh"
#include "dot2.cuh"
#include "kernels.h"
#include "scale.cuh"

namespace qtg {

// ---------------------------------------------------------------------------
// Exact complex128 multiply-accumulate, rounded like the reference's
// std::complex<double> loop on x86-64: p = (ar*br - ai*bi, ar*bi + ai*br), c += p.
// The _rn intrinsics are never fused into FMA by the compiler.
__device__ __forceinline__ void cmac_exact(double &cre, double &cim, double2 a, double2 b) {
    double pre = __dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y));
    double pim = __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x));
    cre = __dadd_rn(cre, pre);
    cim = __dadd_rn(cim, pim);
}

__device__ __forceinline__ void cmac_f32(float &cre, float &cim, float2 a, float2 b) {
    cre = fmaf(a.x, b.x, cre);
    cre = fmaf(-a.y, b.y, cre);
    cim = fmaf(a.x, b.y, cim);
    cim = fmaf(a.y, b.x, cim);
}

// ---------------------------------------------------------------------------
// Multi-CTA pairwise contraction.  The k-offset table of a chunk of the
// summation range is built in shared memory once per CTA and read as a
// broadcast by every thread; each thread owns whole output elements, so the
// summation order per element is the reference's.
constexpr int kPairThreads = 256;
constexpr int kPairChunk = 1024;

template <typename T>
struct Vec2;
template <>
struct Vec2<double> { using type = double2; };
template <>
struct Vec2<float> { using type = float2; };

// One contraction on CTAs blk = 0 .. nblk-1 of its launch.  complex64: the
// sums are scaled by 2^shift and the largest stored magnitude is returned
// (mag_bits) for the step's scale word.
template <typename T>
__device__ __forceinline__ uint32_t pair_body(const typename Vec2<T>::type *__restrict__ A,
                                              const typename Vec2<T>::type *__restrict__ B,
                                              typename Vec2<T>::type *__restrict__ C, const StepDesc &d,
                                              uint64_t n_out, uint64_t K, uint32_t blk, uint32_t nblk, int shift) {
    using V = typename Vec2<T>::type;
    uint32_t lmax = 0;
    __shared__ uint64_t s_oa[kPairChunk];
    __shared__ uint64_t s_ob[kPairChunk];
    const uint64_t stride = (uint64_t) nblk * blockDim.x;
    // every CTA walks the same number of outer iterations so that the
    // __syncthreads of the chunk loop stay uniform
    const uint64_t n_iter = (n_out + stride - 1) / stride;
    for (uint64_t it = 0; it < n_iter; it++) {
        const uint64_t c = it * stride + (uint64_t) blk * blockDim.x + threadIdx.x;
        const bool valid = c < n_out;
        uint64_t oa0 = 0, ob0 = 0;
        if (valid) scatter_c(c, d, oa0, ob0);
        T cre = 0, cim = 0;
        for (uint64_t k0 = 0; k0 < K; k0 += kPairChunk) {
            const int nk = (int) ((K - k0) < (uint64_t) kPairChunk ? (K - k0) : (uint64_t) kPairChunk);
            __syncthreads();
            for (int j = threadIdx.x; j < nk; j += blockDim.x) {
                s_oa[j] = scatter_digits(k0 + j, d.posAs, d.nSum);
                s_ob[j] = scatter_digits(k0 + j, d.posBs, d.nSum);
            }
            __syncthreads();
            if (valid) {
                for (int j = 0; j < nk; j++) {
                    V a = A[oa0 + s_oa[j]];
                    V b = B[ob0 + s_ob[j]];
                    if constexpr (sizeof(T) == 8) cmac_exact(cre, cim, a, b);
                    else cmac_f32(cre, cim, a, b);
                }
            }
        }
        if (valid) {
            V v;
            if constexpr (sizeof(T) == 8) {
                v.x = cre;
                v.y = cim;
            } else {
                v.x = scale_pow2(cre, shift);
                v.y = scale_pow2(cim, shift);
                lmax = max(lmax, mag_bits(v));
            }
            C[c] = v;
        }
    }
    return lmax;
}

template <typename T>
__global__ void __launch_bounds__(kPairThreads)
pair_kernel(const typename Vec2<T>::type *__restrict__ A, const typename Vec2<T>::type *__restrict__ B,
            typename Vec2<T>::type *__restrict__ C, const StepDesc d, uint64_t n_out, uint64_t K,
            const StepScaleRef sc) {
    const int shift = sizeof(T) == 4 ? scale_shift(sc) : 0;
    const uint32_t lmax = pair_body<T>(A, B, C, d, n_out, K, blockIdx.x, gridDim.x, shift);
    if constexpr (sizeof(T) == 4) scale_note(sc, lmax, shift, blockIdx.x == 0);
}

// Several independent small contractions (one dependency level of a plan run
// step by step) in one launch: job j owns CTAs [block_begin_j, block_begin_{j+1}).
template <typename T>
__global__ void __launch_bounds__(kPairThreads) pair_batch_kernel(const __grid_constant__ PairBatch pb) {
    using V = typename Vec2<T>::type;
    uint32_t j = 0;
    while (j + 1 < pb.n_jobs && blockIdx.x >= pb.job[j + 1].block_begin) j++;
    const PairJob &w = pb.job[j];
    const uint32_t end = j + 1 < pb.n_jobs ? pb.job[j + 1].block_begin : gridDim.x;
    const int shift = sizeof(T) == 4 ? scale_shift(w.sc) : 0;
    const uint32_t lmax = pair_body<T>(reinterpret_cast<const V *>(w.A), reinterpret_cast<const V *>(w.B),
                                       reinterpret_cast<V *>(w.C), w.d, w.n_out, w.K, blockIdx.x - w.block_begin,
                                       end - w.block_begin, shift);
    if constexpr (sizeof(T) == 4) scale_note(w.sc, lmax, shift, blockIdx.x == w.block_begin);
}

// ---------------------------------------------------------------------------
// Long reductions into a few outputs (steps run one at a time).

constexpr int kReduceThreads = 256;

// Dot2 partial sums of output c over a grid-strided share of the k range; one
// (p_re, s_re, p_im, s_im) per CTA and output.
__global__ void __launch_bounds__(kReduceThreads)
reduce_partial_f32(const float2 *__restrict__ A, const float2 *__restrict__ B, const StepDesc d, uint32_t n_out,
                   uint64_t K, float4 *__restrict__ partials) {
    __shared__ float4 s_part[kReduceThreads / 32];
    for (uint32_t c = 0; c < n_out; c++) {
        uint64_t oa0, ob0;
        scatter_c(c, d, oa0, ob0);
        float pre = 0.f, sre = 0.f, pim = 0.f, sim = 0.f;
        const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
        for (uint64_t k = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; k < K; k += stride)
            cmac_dot2(pre, sre, pim, sim, A[oa0 + scatter_digits(k, d.posAs, d.nSum)],
                      B[ob0 + scatter_digits(k, d.posBs, d.nSum)]);
        for (int off = 16; off >= 1; off >>= 1) {
            const float a = __shfl_xor_sync(0xffffffffu, pre, off), b = __shfl_xor_sync(0xffffffffu, sre, off);
            const float e = __shfl_xor_sync(0xffffffffu, pim, off), f = __shfl_xor_sync(0xffffffffu, sim, off);
            dot2_merge(pre, sre, a, b);
            dot2_merge(pim, sim, e, f);
        }
        if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = make_float4(pre, sre, pim, sim);
        __syncthreads();
        if (threadIdx.x == 0) {
            float4 t = s_part[0];
            for (int w = 1; w < kReduceThreads / 32; w++) {
                dot2_merge(t.x, t.y, s_part[w].x, s_part[w].y);
                dot2_merge(t.z, t.w, s_part[w].z, s_part[w].w);
            }
            partials[(uint64_t) c * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}

// one warp per output: merge the CTAs' partial sums, round once to complex64
// (scaled by 2^shift of the step's producers)
__global__ void reduce_final_f32(const float4 *__restrict__ partials, uint32_t n_parts, uint32_t n_out,
                                 float2 *__restrict__ C, const StepScaleRef sc) {
    const uint32_t c = blockIdx.x;
    if (c >= n_out) return;
    const int shift = scale_shift(sc);
    float pre = 0.f, sre = 0.f, pim = 0.f, sim = 0.f;
    for (uint32_t j = threadIdx.x; j < n_parts; j += 32) {
        const float4 t = partials[(uint64_t) c * n_parts + j];
        dot2_merge(pre, sre, t.x, t.y);
        dot2_merge(pim, sim, t.z, t.w);
    }
    for (int off = 16; off >= 1; off >>= 1) {
        const float a = __shfl_xor_sync(0xffffffffu, pre, off), b = __shfl_xor_sync(0xffffffffu, sre, off);
        const float e = __shfl_xor_sync(0xffffffffu, pim, off), f = __shfl_xor_sync(0xffffffffu, sim, off);
        dot2_merge(pre, sre, a, b);
        dot2_merge(pim, sim, e, f);
    }
    const float2 v = make_float2(scale_pow2((float) ((double) pre + (double) sre), shift),
                                 scale_pow2((float) ((double) pim + (double) sim), shift));
    if (threadIdx.x == 0) C[c] = v;
    scale_note(sc, threadIdx.x == 0 ? mag_bits(v) : 0u, shift, c == 0);
}

// Exact complex128 reduction: one CTA per output.  The products of a chunk of
// kReduceThreads consecutive k are formed in parallel (each rounded as the
// reference rounds it) into a double-buffered shared array; thread 0 adds them
// in increasing k, so the sum is the reference's sequential sum bit for bit.
__global__ void __launch_bounds__(kReduceThreads)
reduce_exact(const double2 *__restrict__ A, const double2 *__restrict__ B, const StepDesc d, uint64_t K,
             double2 *__restrict__ C) {
    __shared__ double2 prod[2][kReduceThreads];
    const uint32_t c = blockIdx.x;
    uint64_t oa0, ob0;
    scatter_c(c, d, oa0, ob0);
    double cre = 0.0, cim = 0.0;
    int buf = 0;
    for (uint64_t k0 = 0; k0 < K; k0 += kReduceThreads, buf ^= 1) {
        const uint64_t k = k0 + threadIdx.x;
        if (k < K) {
            const double2 a = A[oa0 + scatter_digits(k, d.posAs, d.nSum)];
            const double2 b = B[ob0 + scatter_digits(k, d.posBs, d.nSum)];
            prod[buf][threadIdx.x] = make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                                                  __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
        }
        // one barrier per chunk: thread 0 reaches the next one only after summing
        // this buffer, and the buffer is written again two chunks later
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t n = K - k0 < (uint64_t) kReduceThreads ? (uint32_t) (K - k0) : (uint32_t) kReduceThreads;
            // loads run ahead of the two dependent add chains
#pragma unroll 8
            for (uint32_t j = 0; j < n; j++) {
                const double2 p = prod[buf][j];
                cre = __dadd_rn(cre, p.x);
                cim = __dadd_rn(cim, p.y);
            }
        }
    }
    if (threadIdx.x == 0) C[c] = make_double2(cre, cim);
}

static uint32_t reduce_grid(const StepDesc &d) {
    const uint64_t K = 1ull << (2 * d.nSum);
    uint64_t g = K / (kReduceThreads * 64ull);   // >= 64 terms per thread
    const uint64_t cap = (uint64_t) persistent_sms() * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (uint32_t) g;
}

size_t reduce_scratch_bytes(const StepDesc &d) {
    return sizeof(float4) * (size_t) reduce_grid(d) * (size_t) (1ull << (2 * d.nFree));
}

cudaError_t launch_reduce_final_f32(const float4 *partials, uint32_t n_parts, uint32_t n_out, float2 *C,
                                    const StepScaleRef &sc, cudaStream_t stream) {
    reduce_final_f32<<<n_out, 32, 0, stream>>>(partials, n_parts, n_out, C, sc);
    return cudaGetLastError();
}

cudaError_t launch_reduce_f32(const StepDesc &d, const float2 *A, const float2 *B, float2 *C, void *scratch,
                              cudaStream_t stream, const StepScaleRef &sc) {
    const uint32_t n_out = (uint32_t) (1ull << (2 * d.nFree));
    const uint64_t K = 1ull << (2 * d.nSum);
    const uint32_t g = reduce_grid(d);
    float4 *parts = static_cast<float4 *>(scratch);
    reduce_partial_f32<<<g, kReduceThreads, 0, stream>>>(A, B, d, n_out, K, parts);
    reduce_final_f32<<<n_out, 32, 0, stream>>>(parts, g, n_out, C, sc);
    return cudaGetLastError();
}

cudaError_t launch_reduce_exact(const StepDesc &d, const double2 *A, const double2 *B, double2 *C,
                                cudaStream_t stream) {
    const uint32_t n_out = (uint32_t) (1ull << (2 * d.nFree));
    reduce_exact<<<n_out, kReduceThreads, 0, stream>>>(A, B, d, 1ull << (2 * d.nSum), C);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Grouped plan interpreter.

// The schedule of a level is precomputed on the host: every step carries the
// first work item it owns (item_start, relative to its level) and its lane
// group size, so a thread finds its step with a binary search and the CTA
// needs one barrier per level.
//
// Mixed precision keeps each intermediate as stored values S with a true value
// S * 2^E.  A step loads its operands as they are, scales the accumulated sum
// by 2^-(mA+mB) (m = the exponent of the producer's largest |S|, tracked with a
// shared-memory atomicMax while the producer ran) and records
// E_C = E_A + E_B + mA + mB.  Every stored tensor thus stays within a factor 4^K
// of 1 (no overflow, no underflow drift) without a separate normalisation pass.

struct PlanSmemHeader {
    uint32_t *maxbits;   // float bits of max |S| of each step's output
    int32_t *expo;       // E of each step's output
};

// exponent m of the producer's largest |S| (max = f 2^m, f in [0.5, 1)), from the float bits
__device__ __forceinline__ int step_scale(const PlanSmemHeader &h, int step) {
    if (step < 0) return 0;
    const uint32_t bits = h.maxbits[step];
    const uint32_t ex = (bits >> 23) & 0xffu;
    if (ex == 0xffu || bits == 0) return 0;        // inf/NaN or an all-zero tensor: no scaling
    if (ex == 0) {                                  // subnormal maximum
        int e;
        frexpf(__uint_as_float(bits), &e);
        return e;
    }
    return (int) ex - 126;
}

// exact multiplication by 2^e: one multiply while 2^e is a normal float, ldexp beyond
__device__ __forceinline__ float scale2f(float x, int e) {
    return (e >= -126 && e <= 127) ? x * __int_as_float((127 + e) << 23) : ldexpf(x, e);
}
__device__ __forceinline__ double scale2d(double x, int e) {
    return (e >= -1022 && e <= 1023) ? x * __longlong_as_double((long long) (1023 + e) << 52) : ldexp(x, e);
}

// Mixed plans run first without the power-of-two scaling.  A stored value
// above 2^60 -- or inf/NaN -- makes the CTA run the instance again with the
// scaling; with every magnitude <= 2^60 and sums of at most 4^8 terms no
// product or sum can overflow FP32.  On the small side what matters is a
// tensor's largest magnitude, not its smallest: a tensor whose largest
// magnitude is at least 2^-60 keeps the relative precision of FP32 (products
// of its entries underflow only where they are 2^-66 or more below the
// tensor's scale, far under FP32 rounding), whereas a tensor of small entries
// only could lose its products to underflow.  So a nonzero magnitude below
// 2^-60 only flags its step; at the end of the level the CTA looks at each
// flagged step's largest magnitude and reruns with scaling when it is below
// 2^-60.  (Cancellation residues next to O(1) entries are common in larger
// light cones and cost nothing this way.)
constexpr float kUnscaledMax = 1.152921504606847e18f;   // 2^60
constexpr float kUnscaledMin = 8.673617379884035e-19f;  // 2^-60

// range check of one stored magnitude (mag) / of a set with smallest nonzero
// magnitude tmin, in the unscaled pass
__device__ __forceinline__ void unscaled_check(float mag, float tmin, int si, PlanSmemHeader &h, int *bad,
                                               uint32_t &tiny) {
    if (!(mag <= kUnscaledMax)) {
        *bad = 1;
    } else if (tmin > 0.f && tmin < kUnscaledMin) {
        if (!(h.maxbits[si] & 1u)) atomicOr(&h.maxbits[si], 1u);
        tiny = 1;
    }
}

// End of a level of the unscaled pass: for every step of the level flagged
// by unscaled_check, whether its output has a magnitude of at least 2^-60
// (float values; the complex64 copy of a complex128 output).  Uniform across
// the CTA: the flags were written before the barrier that precedes this.
__device__ void unscaled_level_check(const StepDesc *__restrict__ steps, int s0, int s1, const char *ws,
                                     const PlanSmemHeader &h, int *bad, bool all = false) {
    for (int s = s0; s < s1; s++) {
        // all: steps carry no flags (the descriptor path); every step of the
        // level is scanned, and one holding a tiny magnitude but no normal one fails
        if (!all && !(h.maxbits[s] & 1u)) continue;
        const StepDesc &d = steps[s];
        const uint32_t n_out = 1u << (2 * d.nFree);
        const float2 *v = reinterpret_cast<const float2 *>(ws + d.c_off + ((d.flags & kCF64) ? 16ull * n_out : 0ull));
        int normal = 0, small = 0;
        for (uint32_t e = threadIdx.x; e < n_out; e += blockDim.x) {
            const float2 x = v[e];
            const float mag = fmaxf(fabsf(x.x), fabsf(x.y));
            normal |= mag >= kUnscaledMin;
            small |= mag > 0.f && mag < kUnscaledMin;
        }
        const bool any_normal = __syncthreads_or(normal) != 0;
        const bool any_small = all ? __syncthreads_or(small) != 0 : true;
        if (any_small && !any_normal && threadIdx.x == 0) *bad = 1;
    }
}

template <bool kMixed, bool kScaled>
__device__ void plan_level(const StepDesc *__restrict__ steps, const HotStep *__restrict__ hot, int s0, int s1,
                           uint32_t total, const char *leaves, char *ws, PlanSmemHeader &h,
                           const ushort2 *__restrict__ tables, const uint8_t *__restrict__ imap, int *bad,
                           uint32_t meta, uint32_t &tiny) {
    const int tid = threadIdx.x;
    for (uint32_t base = 0; base < total; base += blockDim.x) {
        // warps with no item this round skip it (the body has warp-level
        // collectives only, no CTA barrier)
        if (base + (tid & ~31) >= total) continue;
        const uint32_t item = base + tid;
        int si = s0;
        if (item < total && imap) {
            si = s0 + imap[item];
        } else if (item < total) {
            int lo = s0, hi = s1 - 1;   // last step whose first item is <= item
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (hot[mid].item_start <= item) lo = mid; else hi = mid - 1;
            }
            si = lo;
        }
        // the packed fields: two 16-byte shared-memory loads
        const uint4 w0 = reinterpret_cast<const uint4 *>(hot + si)[0];
        const uint4 w1 = reinterpret_cast<const uint4 *>(hot + si)[1];
        HotStep hs;
        hs.a_off = w0.x;
        hs.b_off = w0.y;
        hs.c_off = w0.z;
        hs.tab_off = w0.w;
        hs.item_start = w1.x;
        hs.a_step = (int16_t) (w1.y & 0xffffu);
        hs.b_step = (int16_t) (w1.y >> 16);
        hs.group_log2 = (uint8_t) (w1.z & 0xffu);
        hs.nFree = (uint8_t) ((w1.z >> 8) & 0xffu);
        hs.nSum = (uint8_t) ((w1.z >> 16) & 0xffu);
        hs.flags = (uint8_t) (w1.z >> 24);
        const uint32_t lg = hs.group_log2;
        const uint32_t g = 1u << lg;
        const uint32_t local = item - hs.item_start;
        const uint32_t c = local >> lg;
        const uint32_t lane_k = local & (g - 1);
        const int nFree = hs.nFree, nSum = hs.nSum;
        const uint32_t n_out = 1u << (2 * nFree);
        const bool valid = item < total && c < n_out;
        const uint32_t K = 1u << (2 * nSum);
        const uint32_t flags = hs.flags;
        const char *abase = ((flags & kALeaf) ? leaves : ws) + hs.a_off;
        const char *bbase = ((flags & kBLeaf) ? leaves : ws) + hs.b_off;
        const uint32_t tab = hs.tab_off;
        const StepDesc &d = steps[si];   // full maps, read only where there are no offset tables
        const ushort2 *ktab = tables + tab + n_out;   // used only when tab != kNoTable
        uint32_t oa0 = 0, ob0 = 0;
        if (valid) {
            if (tab != kNoTable) {
                const ushort2 o = tables[tab + c];
                oa0 = o.x;
                ob0 = o.y;
            } else {
                uint64_t oa, ob;
                scatter_c(c, d, oa, ob);
                oa0 = (uint32_t) oa;
                ob0 = (uint32_t) ob;
            }
        }
        if constexpr (!kMixed) {
            if (valid) {
                const double2 *A = reinterpret_cast<const double2 *>(abase) + oa0;
                const double2 *B = reinterpret_cast<const double2 *>(bbase) + ob0;
                double cre = 0.0, cim = 0.0;
                if (tab != kNoTable) {
                    // loads of four terms are issued together, the adds stay in k order
                    uint32_t k = 0;
                    for (; k + 4 <= K; k += 4) {
                        double2 a[4], b[4];
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const ushort2 kk = ktab[k + j];
                            a[j] = A[kk.x];
                            b[j] = B[kk.y];
                        }
#pragma unroll
                        for (int j = 0; j < 4; j++) cmac_exact(cre, cim, a[j], b[j]);
                    }
                    for (; k < K; k++) {
                        const ushort2 kk = ktab[k];
                        cmac_exact(cre, cim, A[kk.x], B[kk.y]);
                    }
                } else {
                    for (uint32_t k = 0; k < K; k++)
                        cmac_exact(cre, cim, A[scatter_digits(k, d.posAs, nSum)], B[scatter_digits(k, d.posBs, nSum)]);
                }
                reinterpret_cast<double2 *>(ws + hs.c_off)[c] = make_double2(cre, cim);
            }
        } else {
            // f64: a reduction where cancellation lives; accumulated with Dot2
            // (fre + ere, fim + eim) and stored as complex128
            // operands are complex64 (a complex128 producer leaves a complex64 copy)
            const bool f64 = (flags & kCF64) != 0;
            float fre = 0.f, fim = 0.f, ere = 0.f, eim = 0.f;
            if (valid) {
                if (!f64 && tab != kNoTable) {
                    // the common case: complex64 operands, tabled offsets
                    const float2 *A = reinterpret_cast<const float2 *>(abase) + oa0;
                    const float2 *B = reinterpret_cast<const float2 *>(bbase) + ob0;
                    // four terms in flight, two accumulators to break the FMA chain
                    float r1 = 0.f, i1 = 0.f;
                    uint32_t k = lane_k;
                    for (; k + 3 * g < K; k += 4 * g) {
                        float2 a[4], b[4];
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const ushort2 kk = ktab[k + j * g];
                            a[j] = A[kk.x];
                            b[j] = B[kk.y];
                        }
                        cmac_f32(fre, fim, a[0], b[0]);
                        cmac_f32(r1, i1, a[1], b[1]);
                        cmac_f32(fre, fim, a[2], b[2]);
                        cmac_f32(r1, i1, a[3], b[3]);
                    }
                    for (; k < K; k += g) {
                        const ushort2 kk = ktab[k];
                        cmac_f32(fre, fim, A[kk.x], B[kk.y]);
                    }
                    fre += r1;
                    fim += i1;
                } else {
                    for (uint32_t k = lane_k; k < K; k += g) {
                        uint32_t ka, kb;
                        if (tab != kNoTable) {
                            const ushort2 kk = ktab[k];
                            ka = kk.x;
                            kb = kk.y;
                        } else {
                            ka = (uint32_t) scatter_digits(k, d.posAs, nSum);
                            kb = (uint32_t) scatter_digits(k, d.posBs, nSum);
                        }
                        const float2 a = reinterpret_cast<const float2 *>(abase)[oa0 + ka];
                        const float2 b = reinterpret_cast<const float2 *>(bbase)[ob0 + kb];
                        if (f64) cmac_dot2(fre, ere, fim, eim, a, b);
                        else cmac_f32(fre, fim, a, b);
                    }
                }
            }
            // lane groups are aligned inside a warp; every lane takes part in the
            // shuffles, which run as far as the level's widest group needs (levels
            // of single-lane items skip them)
            const uint32_t gmax = 1u << (meta & 0xffu);
            const bool comp = (meta & 0x100u) != 0;
            for (uint32_t off = gmax >> 1; off >= 1; off >>= 1) {
                const float ore = __shfl_xor_sync(0xffffffffu, fre, (int) off);
                const float oim = __shfl_xor_sync(0xffffffffu, fim, (int) off);
                float oere = 0.f, oeim = 0.f;
                if (comp) {
                    oere = __shfl_xor_sync(0xffffffffu, ere, (int) off);
                    oeim = __shfl_xor_sync(0xffffffffu, eim, (int) off);
                }
                if (off < g) {
                    if (f64) {
                        dot2_merge(fre, ere, ore, oere);
                        dot2_merge(fim, eim, oim, oeim);
                    } else {
                        fre += ore;
                        fim += oim;
                    }
                }
            }
            const bool writer = valid && lane_k == 0;
            if constexpr (!kScaled) {
                if (writer) {
                    float mag;
                    if (f64) {
                        const double dre = (double) fre + (double) ere, dim = (double) fim + (double) eim;
                        reinterpret_cast<double2 *>(ws + hs.c_off)[c] = make_double2(dre, dim);
                        const float2 f = make_float2((float) dre, (float) dim);
                        reinterpret_cast<float2 *>(ws + hs.c_off + 16ull * n_out)[c] = f;
                        mag = fmaxf(fabsf(f.x), fabsf(f.y));
                    } else {
                        reinterpret_cast<float2 *>(ws + hs.c_off)[c] = make_float2(fre, fim);
                        mag = fmaxf(fabsf(fre), fabsf(fim));
                    }
                    // a complex value with one tiny part is fine; a tiny magnitude is flagged
                    unscaled_check(mag, mag, si, h, bad, tiny);
                }
                continue;
            }
            uint32_t magbits = 0;
            if (writer) {
                const int ma = step_scale(h, hs.a_step), mb = step_scale(h, hs.b_step);
                float mag;
                if (f64) {
                    const double dre = scale2d((double) fre + (double) ere, -(ma + mb));
                    const double dim = scale2d((double) fim + (double) eim, -(ma + mb));
                    reinterpret_cast<double2 *>(ws + hs.c_off)[c] = make_double2(dre, dim);
                    // the complex64 copy its consumers read
                    reinterpret_cast<float2 *>(ws + hs.c_off + 16ull * n_out)[c] = make_float2((float) dre, (float) dim);
                    mag = (float) fmax(fabs(dre), fabs(dim));
                } else {
                    fre = scale2f(fre, -(ma + mb));
                    fim = scale2f(fim, -(ma + mb));
                    reinterpret_cast<float2 *>(ws + hs.c_off)[c] = make_float2(fre, fim);
                    mag = fmaxf(fabsf(fre), fabsf(fim));
                }
                magbits = __float_as_uint(mag);
                if (c == 0) {
                    const int ea = hs.a_step >= 0 ? h.expo[hs.a_step] : 0;
                    const int eb = hs.b_step >= 0 ? h.expo[hs.b_step] : 0;
                    h.expo[si] = ea + eb + ma + mb;
                }
            }
            // one shared-memory atomic per (warp, step): the writers of a step
            // agree on the maximum first (non-negative floats order as their bits)
            const uint32_t key = writer ? (uint32_t) si : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, key);
            const uint32_t wmax = __reduce_max_sync(peers, magbits);
            if (writer && (threadIdx.x & 31) == (uint32_t) (__ffs(peers) - 1)) atomicMax(&h.maxbits[si], wmax);
        }
    }
}

// The unscaled mixed pass over one level's work items from their host-prepared
// descriptors (ItemDesc): the same arithmetic in the same order as the look-up
// path of plan_level, without the step look-up, the field unpacking and the
// output-offset table read.  A tiny magnitude only raises `tiny` (the level's
// outputs are then checked as a whole, unscaled_level_check with all = true).
__device__ void plan_level_items(const ItemDesc *__restrict__ items, uint32_t total, const char *leaves, char *ws,
                                 const ushort2 *__restrict__ tables, int *bad, uint32_t meta, uint32_t &tiny) {
    const uint32_t tid = threadIdx.x;
    const uint32_t gmax = 1u << (meta & 0xffu);
    const bool comp = (meta & 0x100u) != 0;
    for (uint32_t base = 0; base < total; base += blockDim.x) {
        if (base + (tid & ~31u) >= total) continue;   // warp-level collectives only below
        const uint32_t item = base + tid;
        uint4 w = make_uint4(0u, 0u, 0u, 0u);
        if (item < total) w = reinterpret_cast<const uint4 *>(items)[item];
        const uint32_t m = w.w;
        const uint32_t g = 1u << ((m >> 16) & 7u);
        const uint32_t K = 1u << (2 * ((m >> 19) & 15u));
        const bool valid = (m & kItemValid) != 0;
        const bool f64 = (m & kItemF64) != 0;
        const uint32_t lane_k = item & (g - 1);
        const float2 *A = reinterpret_cast<const float2 *>(((m & kItemLeafA) ? leaves : ws) + w.x);
        const float2 *B = reinterpret_cast<const float2 *>(((m & kItemLeafB) ? leaves : ws) + w.y);
        const ushort2 *ktab = tables + (m & 0xffffu);
        float fre = 0.f, fim = 0.f, ere = 0.f, eim = 0.f;
        if (valid) {
            if (!f64) {
                // four terms in flight, two accumulators to break the FMA chain
                float r1 = 0.f, i1 = 0.f;
                uint32_t k = lane_k;
                for (; k + 3 * g < K; k += 4 * g) {
                    float2 a[4], b[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const ushort2 kk = ktab[k + j * g];
                        a[j] = A[kk.x];
                        b[j] = B[kk.y];
                    }
                    cmac_f32(fre, fim, a[0], b[0]);
                    cmac_f32(r1, i1, a[1], b[1]);
                    cmac_f32(fre, fim, a[2], b[2]);
                    cmac_f32(r1, i1, a[3], b[3]);
                }
                for (; k < K; k += g) {
                    const ushort2 kk = ktab[k];
                    cmac_f32(fre, fim, A[kk.x], B[kk.y]);
                }
                fre += r1;
                fim += i1;
            } else {
                for (uint32_t k = lane_k; k < K; k += g) {
                    const ushort2 kk = ktab[k];
                    cmac_dot2(fre, ere, fim, eim, A[kk.x], B[kk.y]);
                }
            }
        }
        for (uint32_t off = gmax >> 1; off >= 1; off >>= 1) {
            const float ore = __shfl_xor_sync(0xffffffffu, fre, (int) off);
            const float oim = __shfl_xor_sync(0xffffffffu, fim, (int) off);
            float oere = 0.f, oeim = 0.f;
            if (comp) {
                oere = __shfl_xor_sync(0xffffffffu, ere, (int) off);
                oeim = __shfl_xor_sync(0xffffffffu, eim, (int) off);
            }
            if (off < g) {
                if (f64) {
                    dot2_merge(fre, ere, ore, oere);
                    dot2_merge(fim, eim, oim, oeim);
                } else {
                    fre += ore;
                    fim += oim;
                }
            }
        }
        if (valid && lane_k == 0) {
            float mag;
            if (f64) {
                const double dre = (double) fre + (double) ere, dim = (double) fim + (double) eim;
                *reinterpret_cast<double2 *>(ws + w.z) = make_double2(dre, dim);
                const float2 f = make_float2((float) dre, (float) dim);
                *reinterpret_cast<float2 *>(ws + w.z + 8u * ((m >> 27) & 15u)) = f;
                mag = fmaxf(fabsf(f.x), fabsf(f.y));
            } else {
                *reinterpret_cast<float2 *>(ws + w.z) = make_float2(fre, fim);
                mag = fmaxf(fabsf(fre), fabsf(fim));
            }
            if (!(mag <= kUnscaledMax)) *bad = 1;
            else if (mag > 0.f && mag < kUnscaledMin) tiny = 1;
        }
    }
}

// CTA-wide tiled step: the contraction as a product of the gathered matrices
// A~(m, k) = A[oa(m) + ka(k)] and B~(k, n) = B[ob(n) + kb(k)], C[m + M n].
// A tile of TM x TN outputs is split over 16 x 16 threads (MI x NJ outputs
// each, rows tx + 16 i, columns ty + 16 j; threads beyond 256, in the wide
// interpreter, only help gather); the summed range runs in chunks
// whose A~ and B~ slices are gathered into shared memory once and reused by
// every thread of the tile.  Each output still accumulates over k in
// increasing order, so the FP64 form keeps the reference's rounding.
template <bool kMixed, int MI, int NJ>
__device__ float tiled_tiles(const StepDesc &d, const typename std::conditional<kMixed, float2, double2>::type *A,
                             const typename std::conditional<kMixed, float2, double2>::type *B,
                             typename std::conditional<kMixed, float2, double2>::type *C, int shift,
                             unsigned char *tile, uint32_t t_first, uint32_t t_stride, float *tmin_out = nullptr) {
    using V = typename std::conditional<kMixed, float2, double2>::type;
    using T = typename std::conditional<kMixed, float, double>::type;
    constexpr uint32_t KC = kMixed ? kCtaTileChunk : kCtaTileChunk / 2;
    constexpr uint32_t TM = 16 * MI, TN = 16 * NJ;
    V *As = reinterpret_cast<V *>(tile);            // [KC][kCtaTileDim]
    V *Bs = As + KC * kCtaTileDim;                      // [KC][kCtaTileDim]
    uint32_t *s_oa = reinterpret_cast<uint32_t *>(tile + 2u * kCtaTileChunk * kCtaTileDim * 8u);
    uint32_t *s_ob = s_oa + kCtaTileDim;
    const uint32_t tid = threadIdx.x, tx = tid & 15u, ty = tid >> 4;
    const uint32_t fA = d.fA, fB = d.fB, nSum = d.nSum;
    const uint32_t M = 1u << (2 * fA), N = 1u << (2 * fB), K = 1u << (2 * nSum);
    const uint32_t kc = K < KC ? K : KC;
    const uint32_t tiles_m = M / TM, n_tiles = tiles_m * (N / TN);
    float tmax = 0.f, tmin = 0.f;   // tmin: smallest nonzero magnitude (0: none yet)
    for (uint32_t t = t_first; t < n_tiles; t += t_stride) {
        const uint32_t m0 = (t % tiles_m) * TM, n0 = (t / tiles_m) * TN;
        __syncthreads();   // readers of the previous tile's offsets and slices are done
        if (tid < TM) {
            const uint32_t x = m0 + tid;
            uint32_t o = 0;
            for (uint32_t i = 0; i < fA; i++) o += ((x >> (2 * i)) & 3u) << (2 * d.cA[i]);
            s_oa[tid] = o;
        } else if (tid >= 128 && tid - 128 < TN) {
            const uint32_t x = n0 + tid - 128;
            uint32_t o = 0;
            for (uint32_t i = 0; i < fB; i++) o += ((x >> (2 * i)) & 3u) << (2 * d.cB[fA + i]);
            s_ob[tid - 128] = o;
        }
        T cre[MI][NJ], cim[MI][NJ];
#pragma unroll
        for (int i = 0; i < MI; i++)
#pragma unroll
            for (int j = 0; j < NJ; j++) cre[i][j] = cim[i][j] = T(0);
        for (uint32_t k0 = 0; k0 < K; k0 += kc) {
            __syncthreads();   // offsets visible; the previous chunk's slices are consumed
            for (uint32_t e = tid; e < TM * kc; e += blockDim.x) {
                const uint32_t m = e % TM, kk = e / TM;
                As[kk * kCtaTileDim + m] = A[s_oa[m] + (uint32_t) scatter_digits(k0 + kk, d.posAs, (int) nSum)];
            }
            for (uint32_t e = tid; e < TN * kc; e += blockDim.x) {
                const uint32_t n = e % TN, kk = e / TN;
                Bs[kk * kCtaTileDim + n] = B[s_ob[n] + (uint32_t) scatter_digits(k0 + kk, d.posBs, (int) nSum)];
            }
            __syncthreads();
            for (uint32_t kk = 0; kk < kc && tid < 256u; kk++) {
                V a[MI];
#pragma unroll
                for (int i = 0; i < MI; i++) a[i] = As[kk * kCtaTileDim + tx + 16 * i];
#pragma unroll
                for (int j = 0; j < NJ; j++) {
                    const V b = Bs[kk * kCtaTileDim + ty + 16 * j];
#pragma unroll
                    for (int i = 0; i < MI; i++) {
                        if constexpr (kMixed) cmac_f32(cre[i][j], cim[i][j], a[i], b);
                        else cmac_exact(cre[i][j], cim[i][j], a[i], b);
                    }
                }
            }
        }
        if (tid >= 256u) continue;   // (the next tile starts with a barrier every thread reaches)
#pragma unroll
        for (int i = 0; i < MI; i++)
#pragma unroll
            for (int j = 0; j < NJ; j++) {
                const uint32_t c = (m0 + tx + 16 * i) + M * (n0 + ty + 16 * j);
                V v;
                if constexpr (kMixed) {
                    v.x = scale2f(cre[i][j], shift);
                    v.y = scale2f(cim[i][j], shift);
                    const float mag = fmaxf(fabsf(v.x), fabsf(v.y));
                    tmax = fmaxf(tmax, mag);
                    if (mag > 0.f) tmin = tmin > 0.f ? fminf(tmin, mag) : mag;
                } else {
                    v.x = cre[i][j];
                    v.y = cim[i][j];
                }
                C[c] = v;
            }
    }
    if (tmin_out) *tmin_out = tmin;
    return tmax;
}

template <bool kMixed, bool kScaled, int MI, int NJ>
__device__ void tiled_step(const StepDesc &d, int si, const char *leaves, char *ws, PlanSmemHeader &h,
                           unsigned char *tile, int *bad, uint32_t &tiny) {
    using V = typename std::conditional<kMixed, float2, double2>::type;
    const V *A = reinterpret_cast<const V *>(((d.flags & kALeaf) ? leaves : ws) + d.a_off);
    const V *B = reinterpret_cast<const V *>(((d.flags & kBLeaf) ? leaves : ws) + d.b_off);
    V *C = reinterpret_cast<V *>(ws + d.c_off);
    int ma = 0, mb = 0;
    if constexpr (kMixed && kScaled) {
        ma = step_scale(h, d.a_step);
        mb = step_scale(h, d.b_step);
    }
    float tmin = 0.f;
    const float tmax = tiled_tiles<kMixed, MI, NJ>(d, A, B, C, -(ma + mb), tile, 0, 1, &tmin);
    if constexpr (kMixed && !kScaled) unscaled_check(tmax, tmin, si, h, bad, tiny);
    if constexpr (kMixed && kScaled) {
        const uint32_t tid = threadIdx.x;
        const uint32_t wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(tmax));
        if ((tid & 31u) == 0) atomicMax(&h.maxbits[si], wmax);
        if (tid == 0) {
            const int ea = d.a_step >= 0 ? h.expo[d.a_step] : 0;
            const int eb = d.b_step >= 0 ? h.expo[d.b_step] : 0;
            h.expo[si] = ea + eb + ma + mb;
        }
    }
}

template <bool kMixed, bool kScaled>
__device__ __forceinline__ void run_tiled(const StepDesc &d, int si, const char *leaves, char *ws, PlanSmemHeader &h,
                                          unsigned char *tile, int *bad, uint32_t &tiny) {
    const bool wide_m = d.fA >= 3, wide_n = d.fB >= 3;
    if (wide_m && wide_n) tiled_step<kMixed, kScaled, 4, 4>(d, si, leaves, ws, h, tile, bad, tiny);
    else if (wide_m) tiled_step<kMixed, kScaled, 4, 1>(d, si, leaves, ws, h, tile, bad, tiny);
    else if (wide_n) tiled_step<kMixed, kScaled, 1, 4>(d, si, leaves, ws, h, tile, bad, tiny);
    else tiled_step<kMixed, kScaled, 1, 1>(d, si, leaves, ws, h, tile, bad, tiny);
}

// The same tiled product as a whole-GPU kernel for steps run one at a time:
// the CTAs stride over the output tiles; complex64 sums are scaled by the
// step's producers (scale.cuh).
template <bool kMixed, int MI, int NJ>
__global__ void __launch_bounds__(kPlanThreads)
tiled_pair_kernel(const typename std::conditional<kMixed, float2, double2>::type *A,
                  const typename std::conditional<kMixed, float2, double2>::type *B,
                  typename std::conditional<kMixed, float2, double2>::type *C, const StepDesc d,
                  const StepScaleRef sc) {
    extern __shared__ __align__(16) unsigned char tile_smem[];
    const int shift = kMixed ? scale_shift(sc) : 0;
    const float tmax = tiled_tiles<kMixed, MI, NJ>(d, A, B, C, shift, tile_smem, blockIdx.x, gridDim.x);
    if constexpr (kMixed) scale_note(sc, __float_as_uint(tmax), shift, blockIdx.x == 0);
}

// Rotation leaves rebuilt from an angle (mixed plans): the superoperators the
// host gate factory writes, T[in + 4 out] for one-qubit gates and the
// controlled phase's diagonal T[i1 + 4 i2 + 16 i1 + 64 i2] (src/Node.h
// RxNode .. CPhaseNode).  Rx/Ry/Rz angles are narrowed to float first, as the
// reference's parser does with std::stof (src/Network.h:342, 383, 402, 422);
// the trigonometry runs in FP32 (GB300's FP64 pipe is narrow and this is on
// every instance's critical path): one sincosf per gate, sin(th)/2 as
// sin(th/2) cos(th/2).  Entries agree with the host-built complex64 leaves to
// a few ulp.
__device__ void build_rotation(char *leaves, uint2 rot, double angle) {
    float2 *t = reinterpret_cast<float2 *>(leaves + rot.x);
    auto put = [&](int in, int out, float re, float im) { t[in + 4 * out] = make_float2(re, im); };
    if (rot.y == kRotCPhase) {
        float s, c;
        sincosf((float) angle, &s, &c);
        for (int i1 = 0; i1 < 4; i1++)
            for (int i2 = 0; i2 < 4; i2++) {
                const bool rowph = (i1 >> 1) && (i2 >> 1), colph = (i1 & 1) && (i2 & 1);
                float2 v = make_float2(1.f, 0.f);
                if (rowph && !colph) v = make_float2((float) c, (float) s);
                else if (!rowph && colph) v = make_float2((float) c, (float) -s);
                t[i1 + 4 * i2 + 16 * i1 + 64 * i2] = v;
            }
        return;
    }
    const float th = (float) angle;
    for (int e = 0; e < 16; e++) t[e] = make_float2(0.f, 0.f);
    if (rot.y == kRotRz) {
        float s, c;
        sincosf(th, &s, &c);
        put(0, 0, 1.f, 0.f);
        put(3, 3, 1.f, 0.f);
        put(1, 1, c, -s);
        put(2, 2, c, s);
        return;
    }
    float sh2, ch2;
    sincosf(0.5f * th, &sh2, &ch2);
    const float cc = ch2 * ch2, ss = sh2 * sh2, sh = sh2 * ch2;
    for (int i = 0; i < 4; i++) put(i, i, cc, 0.f);
    if (rot.y == kRotRx) {
        put(0, 3, ss, 0.f); put(1, 2, ss, 0.f); put(2, 1, ss, 0.f); put(3, 0, ss, 0.f);
        put(0, 1, 0.f, sh); put(1, 0, 0.f, sh); put(2, 3, 0.f, sh); put(3, 2, 0.f, sh);
        put(0, 2, 0.f, -sh); put(1, 3, 0.f, -sh); put(2, 0, 0.f, -sh); put(3, 1, 0.f, -sh);
    } else {
        put(0, 3, ss, 0.f); put(3, 0, ss, 0.f); put(1, 2, -ss, 0.f); put(2, 1, -ss, 0.f);
        put(0, 1, sh, 0.f); put(0, 2, sh, 0.f); put(1, 3, sh, 0.f); put(2, 3, sh, 0.f);
        put(1, 0, -sh, 0.f); put(2, 0, -sh, 0.f); put(3, 1, -sh, 0.f); put(3, 2, -sh, 0.f);
    }
}

// Staging: at the start of an instance one thread issues TMA bulk copies
// (cp.async.bulk, completion counted on an mbarrier) of the instance's plan
// block and leaf image into shared memory; the CTA waits once and then every
// level reads descriptors, leaves and intermediates from shared memory.

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(mbar), "r"(parity) : "memory");
    return ok != 0;
}

// Test hook of the staging failure path (qt_debug_staging_fault): with mode 1
// thread 0 issues no staging copies, so the wait below runs out after
// g_stage_fault_polls polls and the instances report the timeout value.
__device__ uint32_t g_stage_fault_mode = 0;
__device__ uint32_t g_stage_fault_polls = 0;

// Bounded wait: a bulk copy finishes in microseconds; after ~1 s of polling the
// wait gives up and the instance reports kStagingTimeoutBits instead of
// hanging the CTA.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity, uint32_t limit = 1u << 22) {
    for (uint32_t it = 0; it < limit; it++) {
        if (mbar_try_wait(mbar, parity)) return true;
        if (it > 64) __nanosleep(256);
    }
    return false;
}

constexpr uint32_t kBulkChunk = 32768;

__device__ __forceinline__ void bulk_copy_chunks(unsigned char *dst, const char *src, uint32_t bytes, uint32_t mbar) {
    for (uint32_t off = 0; off < bytes; off += kBulkChunk) {
        const uint32_t n = bytes - off < kBulkChunk ? bytes - off : kBulkChunk;
        bulk_g2s(smem_addr(dst + off), src + off, n, mbar);
    }
}

// The arrays of a plan block, in global memory or rebased into its staged copy
// in shared memory (stage != null).
struct PlanView {
    PlanDesc P;
    const StepDesc *steps;
    const int32_t *level_start, *rank0_steps, *level_cta;
    const uint32_t *level_items, *level_meta;
    const uint2 *rotations;
    const uint8_t *item_step;
    const HotStep *hot;
    const ushort2 *tables;
    const ItemDesc *items;   // null: the work items look their steps up
};

__device__ __forceinline__ PlanView plan_view(const PlanDesc *gplan, const unsigned char *stage) {
    PlanView v;
    v.P = stage ? *reinterpret_cast<const PlanDesc *>(stage) : *gplan;
    const char *gbase = reinterpret_cast<const char *>(gplan);
    const char *sbase = reinterpret_cast<const char *>(stage);
    auto at = [&](const void *p) -> const char * {
        return stage ? sbase + (reinterpret_cast<const char *>(p) - gbase) : reinterpret_cast<const char *>(p);
    };
    v.steps = reinterpret_cast<const StepDesc *>(at(v.P.steps));
    v.level_start = reinterpret_cast<const int32_t *>(at(v.P.level_start));
    v.rank0_steps = reinterpret_cast<const int32_t *>(at(v.P.rank0_steps));
    v.level_items = reinterpret_cast<const uint32_t *>(at(v.P.level_items));
    v.tables = reinterpret_cast<const ushort2 *>(at(v.P.tables));
    v.level_cta = reinterpret_cast<const int32_t *>(at(v.P.level_cta));
    v.rotations = reinterpret_cast<const uint2 *>(at(v.P.rotations));
    v.item_step = v.P.item_step ? reinterpret_cast<const uint8_t *>(at(v.P.item_step)) : nullptr;
    v.hot = reinterpret_cast<const HotStep *>(at(v.P.hot));
    v.level_meta = reinterpret_cast<const uint32_t *>(at(v.P.level_meta));
    v.items = v.P.items ? reinterpret_cast<const ItemDesc *>(at(v.P.items)) : nullptr;
    return v;
}

// Every level of a plan, one CTA; a barrier after each level.
template <bool kMixed, bool kScaled>
__device__ __forceinline__ void plan_levels(const PlanView &v, const char *leaves, char *ws, PlanSmemHeader &h,
                                            unsigned char *tile, int *bad) {
    uint32_t items_before = 0;
    uint32_t tiny = 0;   // this thread flagged a step of the level (unscaled pass)
    for (int L = 0; L < v.P.n_levels; L++) {
        const int sc = v.level_cta[L], s1 = v.level_start[L + 1];
        if (kMixed && !kScaled && v.items)
            plan_level_items(v.items + items_before, v.level_items[L], leaves, ws, v.tables, bad, v.level_meta[L],
                             tiny);
        else
            plan_level<kMixed, kScaled>(v.steps, v.hot, v.level_start[L], sc, v.level_items[L], leaves, ws, h,
                                        v.tables, v.item_step ? v.item_step + items_before : nullptr, bad,
                                        v.level_meta[L], tiny);
        items_before += v.level_items[L];
        for (int s = sc; s < s1; s++) run_tiled<kMixed, kScaled>(v.steps[s], s, leaves, ws, h, tile, bad, tiny);
        if constexpr (kMixed && !kScaled) {
            if (__syncthreads_or(tiny)) {
                unscaled_level_check(v.steps, v.level_start[L], s1, ws, h, bad, v.items != nullptr);
                tiny = 0;
            }
        } else {
            __syncthreads();
        }
    }
}

// One contraction of an instance: the header is clear, *bad is 0 and a barrier
// has passed.  The mixed form runs unscaled first and again with power-of-two
// scaling only when a value left the safe range.
template <bool kMixed>
__device__ __forceinline__ void plan_contract(const PlanView &v, const char *leaves, char *ws, PlanSmemHeader &h,
                                              unsigned char *tile, int *bad, uint32_t n_steps) {
    if constexpr (kMixed) {
        plan_levels<true, false>(v, leaves, ws, h, tile, bad);
        if (*bad) {
            for (uint32_t s = threadIdx.x; s < n_steps; s += blockDim.x) {
                h.maxbits[s] = 0;
                h.expo[s] = 0;
            }
            __syncthreads();
            plan_levels<true, true>(v, leaves, ws, h, tile, bad);
        }
    } else {
        plan_levels<false, true>(v, leaves, ws, h, tile, bad);
    }
}

// final-value rule of src/Network.h:961-965, applied in contraction order
// (one thread)
template <bool kMixed>
__device__ __forceinline__ double2 plan_final_value(const PlanView &v, const char *ws, const PlanSmemHeader &h) {
    double fre = 0.0, fim = 0.0;
    for (int r = 0; r < v.P.n_rank0; r++) {
        const int s = v.rank0_steps[r];
        const StepDesc &d = v.steps[s];
        double vre, vim;
        if (!kMixed || (d.flags & kCF64)) {
            const double2 x = *reinterpret_cast<const double2 *>(ws + d.c_off);
            vre = x.x; vim = x.y;
        } else {
            const float2 x = *reinterpret_cast<const float2 *>(ws + d.c_off);
            vre = x.x; vim = x.y;
        }
        if (kMixed) {
            vre = scale2d(vre, h.expo[s]);
            vim = scale2d(vim, h.expo[s]);
        }
        if ((fabs(fre) <= 1.0e-30 && fabs(fim) <= 1.0e-30) || (d.flags & kBothRank0)) {
            fre = vre;
            fim = vim;
        }
    }
    return make_double2(fre, fim);
}

// kMinCtas: the register budget -- the variant is compiled for that many
// resident CTAs per SM (2: up to 128 registers a thread; 3: 80, 4: 64 and
// 5: 48, with some spills), trading single-instance latency for warps per SM.
// kMinCtas = 1 is the wide variant: 512 threads, 128 registers, one CTA per SM.
template <bool kMixed, int kMinCtas>
__global__ void __launch_bounds__(plan_threads(kMinCtas), kMinCtas) plan_kernel(const PlanLaunch lp) {
    extern __shared__ __align__(256) unsigned char smem_raw[];
    const uint32_t header_bytes = plan_header_bytes(lp.header_steps);
    PlanSmemHeader h{reinterpret_cast<uint32_t *>(smem_raw), reinterpret_cast<int32_t *>(smem_raw + 4u * lp.header_steps)};
    uint64_t *mbar_slot = reinterpret_cast<uint64_t *>(smem_raw + header_bytes);
    unsigned char *region = smem_raw + header_bytes + 128;
    char *const ws_smem = reinterpret_cast<char *>(region);
    char *const ws_global = lp.ws_base ? lp.ws_base + (uint64_t) blockIdx.x * lp.ws_stride : nullptr;
    unsigned char *stage = region + lp.ws_smem_bytes;
    unsigned char *tile = stage + lp.stage_bytes;
    __shared__ int s_next;
    __shared__ int s_bad;   // the unscaled pass of the current instance left the safe range
    const uint32_t mbar = smem_addr(mbar_slot);
    if (lp.stage_bytes && threadIdx.x == 0) {
        mbar_init(mbar);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t parity = 0;
    for (int inst = blockIdx.x;;) {
        // dynamic schedule: instances come in the order the host sorted them
        // (longest first), each CTA takes the next one when it is free
        if (lp.next) {
            if (threadIdx.x == 0) s_next = (int) atomicAdd(lp.next, 1u);
            __syncthreads();
            inst = s_next;
        }
        if (inst >= lp.n_instances) break;
        const InstanceDesc I = lp.instances[inst];
        if constexpr (kMixed) {
            // the scale header is cleared while the plan block is in flight
            for (uint32_t s = threadIdx.x; s < I.n_steps; s += blockDim.x) {
                h.maxbits[s] = 0;
                h.expo[s] = 0;
            }
            if (threadIdx.x == 0) s_bad = 0;
        }
        char *const ws = I.ws_bytes <= lp.ws_smem_bytes ? ws_smem : ws_global;
        const bool staged = lp.stage_bytes && I.plan_bytes && I.plan_bytes + I.leaf_bytes <= lp.stage_bytes;
        if (staged) {
            const bool hook = g_stage_fault_mode == 1;
            if (threadIdx.x == 0 && !hook) {
                // the previous instance's generic reads of this region are ordered before the async writes
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(mbar, I.plan_bytes + I.leaf_bytes);
                bulk_copy_chunks(stage, reinterpret_cast<const char *>(I.plan), I.plan_bytes, mbar);
                bulk_copy_chunks(stage + I.plan_bytes, I.leaves, I.leaf_bytes, mbar);
            }
            const bool ok = mbar_wait_bounded(mbar, parity, hook ? g_stage_fault_polls : 1u << 22);
            parity ^= 1u;
            if (__syncthreads_or(!ok)) {
                // the copies never completed: this CTA's instances report the
                // timeout value instead of hanging
                if (threadIdx.x == 0) {
                    const double nan = __longlong_as_double((long long) kStagingTimeoutBits);
                    I.value[0] = I.value[1] = nan;
                    if (lp.next) {
                        for (int j = (int) atomicAdd(lp.next, 1u); j < lp.n_instances; j = (int) atomicAdd(lp.next, 1u))
                            lp.instances[j].value[0] = lp.instances[j].value[1] = nan;
                    } else {
                        for (int j = inst + (int) gridDim.x; j < lp.n_instances; j += gridDim.x)
                            lp.instances[j].value[0] = lp.instances[j].value[1] = nan;
                    }
                }
                return;
            }
        }
        const PlanView v = plan_view(I.plan, staged ? stage : nullptr);
        // the instance's own leaf image, or its staged copy
        char *const leaves = staged ? reinterpret_cast<char *>(stage) + I.plan_bytes : const_cast<char *>(I.leaves);
        if constexpr (kMixed) {
            // the step's angles arrive as numbers; the gate tensors are built here
            if (I.angles && v.P.n_rot) {
                for (int r = threadIdx.x; r < v.P.n_rot; r += blockDim.x)
                    build_rotation(leaves, v.rotations[r], I.angles[r]);
                __syncthreads();
            }
        }
        if (kMixed && !staged) __syncthreads();   // the cleared header (staging waited with a barrier)
        plan_contract<kMixed>(v, leaves, ws, h, tile, &s_bad, I.n_steps);
        if (threadIdx.x == 0) {
            const double2 val = plan_final_value<kMixed>(v, ws, h);
            I.value[0] = val.x;
            I.value[1] = val.y;
        }
        __syncthreads();   // the next instance reuses the header, the workspace and s_next
        if (ws == ws_global) {
            // The instance's intermediates are dead.  Their L2 lines are
            // dropped without being written back (discard is a weak write of
            // an indeterminate value; every intermediate of the next instance
            // is written before it is read), so a slab larger than L2 does not
            // turn every finished instance into DRAM writes.  The slab's stride
            // is a multiple of 256 bytes, so each line belongs to this CTA.
            const uint32_t lines = (I.ws_bytes + 127u) >> 7;
            for (uint32_t l = threadIdx.x; l < lines; l += blockDim.x)
                asm volatile("discard.global.L2 [%0], 128;" ::"l"(ws + ((uint64_t) l << 7)) : "memory");
            __syncthreads();   // ordered before the next instance's first writes
        }
        if (!lp.next) inst += gridDim.x;
    }
}

__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_sys(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_acquire_sys_u64(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(uint32_t *p, uint32_t v) {
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The resident engine (ResidentLaunch).  Every wait is bounded: the request
// poll gives up after idle_polls (the CTA leaves; the host relaunches it on the
// next request) and the staging wait after about a second.
template <int kMinCtas>
__global__ void __launch_bounds__(plan_threads(kMinCtas), kMinCtas) resident_kernel(const ResidentLaunch rl) {
    const PlanLaunch &lp = rl.lp;
    const int inst = blockIdx.x;
    if (inst >= lp.n_instances) return;
    extern __shared__ __align__(256) unsigned char smem_raw[];
    const uint32_t header_bytes = plan_header_bytes(lp.header_steps);
    PlanSmemHeader h{reinterpret_cast<uint32_t *>(smem_raw), reinterpret_cast<int32_t *>(smem_raw + 4u * lp.header_steps)};
    uint64_t *mbar_slot = reinterpret_cast<uint64_t *>(smem_raw + header_bytes);
    unsigned char *region = smem_raw + header_bytes + 128;
    char *const ws_smem = reinterpret_cast<char *>(region);
    char *const ws_global = lp.ws_base ? lp.ws_base + (uint64_t) blockIdx.x * lp.ws_stride : nullptr;
    unsigned char *stage = region + lp.ws_smem_bytes;
    unsigned char *tile = stage + lp.stage_bytes;
    __shared__ int s_bad;
    __shared__ uint32_t s_seq;
    const InstanceDesc I = lp.instances[inst];
    char *const ws = I.ws_bytes <= lp.ws_smem_bytes ? ws_smem : ws_global;
    const bool staged = lp.stage_bytes && I.plan_bytes && I.plan_bytes + I.leaf_bytes <= lp.stage_bytes;
    if (staged) {
        const uint32_t mbar = smem_addr(mbar_slot);
        if (threadIdx.x == 0) {
            mbar_init(mbar);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(mbar, I.plan_bytes + I.leaf_bytes);
            bulk_copy_chunks(stage, reinterpret_cast<const char *>(I.plan), I.plan_bytes, mbar);
            bulk_copy_chunks(stage + I.plan_bytes, I.leaves, I.leaf_bytes, mbar);
        }
        __syncthreads();   // the barrier is initialised before anyone waits on it
        const bool ok = mbar_wait_bounded(mbar, 0);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) st_release_sys(rl.done + inst, kResidentLeft);
            return;
        }
    }
    const PlanView v = plan_view(I.plan, staged ? stage : nullptr);
    char *const leaves = staged ? reinterpret_cast<char *>(stage) + I.plan_bytes : const_cast<char *>(I.leaves);
    uint32_t last = rl.first_seq;
    // Tagged angle words: each carries its request's number beside the angle,
    // so the poll that sees a request also brings the angles (one CPU-GPU
    // round trip instead of two).
    const bool tagged = rl.tagged && I.angles && v.P.n_rot > 0;
    const uint64_t *const words = reinterpret_cast<const uint64_t *>(I.angles);
    if (tagged && v.P.n_rot > (int) blockDim.x) {
        // one word per thread is the host's promise; without it, say so and leave
        if (threadIdx.x == 0) st_release_sys(rl.done + inst, kResidentLeft);
        return;
    }
    for (;;) {
        uint32_t s = last;
        float angle = 0.f;
        if (tagged) {
            // Every thread that owns an angle polls its word until the word
            // carries the next request's number; thread 0 also reads the
            // request word, which here only says whether to leave.  Both are
            // agreed CTA-wide, so every thread leaves the loop together.
            const uint32_t want = resident_next_request(last);
            bool have = threadIdx.x >= (uint32_t) v.P.n_rot;
            for (uint32_t it = 0; it < rl.idle_polls; it++) {
                const bool stop = threadIdx.x == 0 && ld_relaxed_sys(rl.seq) == kResidentStop;
                if (!have) {
                    // acquire: the host reset the value slots before it wrote
                    // this word, so the value written below lands after them
                    const uint64_t w = ld_acquire_sys_u64(words + threadIdx.x);
                    if ((uint32_t) (w >> 32) == want) {
                        have = true;
                        angle = __uint_as_float((uint32_t) w);
                    }
                }
                if (__syncthreads_and(have)) {
                    s = want;
                    break;
                }
                if (__syncthreads_or(stop)) {
                    s = kResidentStop;
                    break;
                }
                __nanosleep(it < 1024 ? 100 : 1000);   // a short spin after a request, then back off
            }
        } else if (threadIdx.x == 0) {
            for (uint32_t it = 0; it < rl.idle_polls; it++) {
                s = ld_acquire_sys(rl.seq);
                if (s != last) break;
                __nanosleep(it < 1024 ? 100 : 1000);   // a short spin after a request, then back off
            }
            s_seq = s;
        }
        for (uint32_t k = threadIdx.x; k < I.n_steps; k += blockDim.x) {
            h.maxbits[k] = 0;
            h.expo[k] = 0;
        }
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        if (!tagged) s = s_seq;
        if (s == kResidentStop) break;   // asked to leave
        if (s == last) {                 // idle for too long: tell the host, then leave
            if (threadIdx.x == 0) st_release_sys(rl.done + inst, kResidentLeft);
            break;
        }
        last = s;
        if (I.angles && v.P.n_rot) {
            if (tagged) {
                // the angle arrived narrowed to float, as build_rotation narrows it
                if (threadIdx.x < (uint32_t) v.P.n_rot) build_rotation(leaves, v.rotations[threadIdx.x], (double) angle);
            } else {
                // the request's angles, read through to host memory (never a stale cached copy)
                for (int r = threadIdx.x; r < v.P.n_rot; r += blockDim.x)
                    build_rotation(leaves, v.rotations[r], __ldcv(I.angles + r));
            }
            __syncthreads();
        }
        plan_contract<true>(v, leaves, ws, h, tile, &s_bad, I.n_steps);
        if (threadIdx.x == 0) {
            const double2 val = plan_final_value<true>(v, ws, h);
            I.value[0] = val.x;
            I.value[1] = val.y;
            st_release_sys(rl.done + inst, s);   // release: the value is visible to the host before the flag
        }
        __syncthreads();   // s_seq, the header and the workspace are reused
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.

static int g_num_sms = 0;

static int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

int persistent_sms() { return num_sms(); }

bool pair_batchable(const StepDesc &d, bool f64) {
    if (2 * (d.nFree + d.nSum) > kPairBatchMaxLog2Macs) return false;
    const bool small_out = (1ull << (2 * d.nFree)) <= kReduceMaxOut;
    // the steps run_contraction would hand to the reduction kernels keep them
    return !reduce_shaped(d) && (f64 || !small_out || d.nSum < 3);
}

cudaError_t launch_pair_batch(PairBatch &pb, bool f64, cudaStream_t stream) {
    if (pb.n_jobs == 0) return cudaSuccess;
    uint32_t blocks = 0;
    for (uint32_t j = 0; j < pb.n_jobs; j++) {
        PairJob &w = pb.job[j];
        w.n_out = 1ull << (2 * w.d.nFree);
        w.K = 1ull << (2 * w.d.nSum);
        w.block_begin = blocks;
        blocks += (uint32_t) ((w.n_out + kPairThreads - 1) / kPairThreads);
    }
    if (f64) pair_batch_kernel<double><<<blocks, kPairThreads, 0, stream>>>(pb);
    else pair_batch_kernel<float><<<blocks, kPairThreads, 0, stream>>>(pb);
    return cudaGetLastError();
}

cudaError_t launch_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64, cudaStream_t stream,
                        const StepScaleRef &sc) {
    const uint64_t n_out = 1ull << (2 * d.nFree);
    const uint64_t K = 1ull << (2 * d.nSum);
    uint64_t blocks = (n_out + kPairThreads - 1) / kPairThreads;
    const uint64_t cap = (uint64_t) persistent_sms() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (f64)
        pair_kernel<double><<<(unsigned) blocks, kPairThreads, 0, stream>>>(
            (const double2 *) A, (const double2 *) B, (double2 *) C, d, n_out, K, StepScaleRef{});
    else
        pair_kernel<float><<<(unsigned) blocks, kPairThreads, 0, stream>>>(
            (const float2 *) A, (const float2 *) B, (float2 *) C, d, n_out, K, sc);
    return cudaGetLastError();
}

// The dynamic shared-memory limit of a kernel is process-wide state.  It is
// raised once per device to the opt-in maximum and never lowered, so launches
// made from several threads at once (the server's lanes) never see another
// thread's smaller setting.
static std::mutex g_attr_mutex;
static bool g_attr_done[64];

using PlanKernelFn = void (*)(const PlanLaunch);

static PlanKernelFn plan_kernel_fn(bool mixed, int ctas) {
    switch (ctas) {
    case 1: return mixed ? plan_kernel<true, 1> : plan_kernel<false, 1>;
    case 3: return mixed ? plan_kernel<true, 3> : plan_kernel<false, 3>;
    case 4: return mixed ? plan_kernel<true, 4> : plan_kernel<false, 4>;
    case 5: return mixed ? plan_kernel<true, 5> : plan_kernel<false, 5>;
    default: return mixed ? plan_kernel<true, 2> : plan_kernel<false, 2>;
    }
}

template <typename Fn>
static cudaError_t raise_smem_limit(Fn fn, int dev);

// the resident engine comes in the default (256 threads, 2 CTAs per SM) and
// the wide (512 threads, 1 CTA per SM) form
static int resident_variant(int variant) { return variant == 1 ? 1 : kPlanDefaultVariant; }
using ResidentKernelFn = void (*)(const ResidentLaunch);
static ResidentKernelFn resident_kernel_fn(int variant) {
    return resident_variant(variant) == 1 ? resident_kernel<1> : resident_kernel<kPlanDefaultVariant>;
}

template <typename Fn>
static cudaError_t raise_smem_limit(Fn fn, int dev) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, fn);
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int) fa.sharedSizeBytes);
    return e;
}

static cudaError_t plan_attributes() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(g_attr_mutex);
    if (dev >= 0 && dev < 64 && g_attr_done[dev]) return cudaSuccess;
    for (int ctas : kPlanVariants)
        for (bool mixed : {true, false})
            if (e == cudaSuccess) e = raise_smem_limit(plan_kernel_fn(mixed, ctas), dev);
    if (e == cudaSuccess) e = raise_smem_limit(resident_kernel<kPlanDefaultVariant>, dev);
    if (e == cudaSuccess) e = raise_smem_limit(resident_kernel<1>, dev);
    if (e == cudaSuccess && dev >= 0 && dev < 64) g_attr_done[dev] = true;
    return e;
}

bool tiled_shaped(const StepDesc &d) {
    for (int i = 0; i < d.nFree; i++)
        if ((d.cA[i] != kNoWire) != (i < d.fA)) return false;   // A's free wires first
    return d.fA >= 2 && d.fB >= 2 && d.fA + d.fB >= 5 && d.nSum >= 1 && d.rA <= 15 && d.rB <= 15 && d.nFree <= 15;
}

template <bool kMixed>
static cudaError_t launch_tiled_t(const StepDesc &d, const void *A, const void *B, void *C, cudaStream_t stream,
                                  const StepScaleRef &sc) {
    using V = typename std::conditional<kMixed, float2, double2>::type;
    const bool wide_m = d.fA >= 3, wide_n = d.fB >= 3;
    const uint64_t tiles = (1ull << (2 * d.fA)) / (wide_m ? 64 : 16) * ((1ull << (2 * d.fB)) / (wide_n ? 64 : 16));
    uint64_t grid = tiles;
    const uint64_t cap = (uint64_t) persistent_sms() * 4;
    if (grid > cap) grid = cap;
    const V *a = static_cast<const V *>(A);
    const V *b = static_cast<const V *>(B);
    V *c = static_cast<V *>(C);
    const size_t smem = kCtaTileBytes;
    if (wide_m && wide_n) tiled_pair_kernel<kMixed, 4, 4><<<(unsigned) grid, kPlanThreads, smem, stream>>>(a, b, c, d, sc);
    else if (wide_m) tiled_pair_kernel<kMixed, 4, 1><<<(unsigned) grid, kPlanThreads, smem, stream>>>(a, b, c, d, sc);
    else tiled_pair_kernel<kMixed, 1, 4><<<(unsigned) grid, kPlanThreads, smem, stream>>>(a, b, c, d, sc);
    return cudaGetLastError();
}

cudaError_t launch_tiled_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64,
                              cudaStream_t stream, const StepScaleRef &sc) {
    return f64 ? launch_tiled_t<false>(d, A, B, C, stream, sc) : launch_tiled_t<true>(d, A, B, C, stream, sc);
}

int plan_num_sms() { return num_sms(); }

cudaError_t plan_set_staging_fault(int mode, uint32_t polls) {
    const uint32_t m = (uint32_t) mode, p = polls ? polls : 1u;
    cudaError_t e = cudaMemcpyToSymbol(g_stage_fault_mode, &m, sizeof m);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_stage_fault_polls, &p, sizeof p);
    return e;
}

int plan_max_grid(size_t smem_bytes, int per_sm_cap, int variant) {
    int per_sm = 0;
    plan_attributes();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plan_kernel_fn(true, variant), plan_threads(variant),
                                                  smem_bytes);
    cudaGetLastError();
    if (per_sm_cap > 0) per_sm = std::min(per_sm, per_sm_cap);
    if (per_sm < 1) per_sm = 1;
    return num_sms() * per_sm;
}

size_t plan_smem_limit() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    size_t static_max = 0;
    for (int ctas : kPlanVariants)
        for (bool mixed : {true, false}) {
            cudaFuncAttributes fa;
            if (cudaFuncGetAttributes(&fa, plan_kernel_fn(mixed, ctas)) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            static_max = std::max(static_max, fa.sharedSizeBytes);
        }
    for (ResidentKernelFn fn : {resident_kernel_fn(1), resident_kernel_fn(kPlanDefaultVariant)}) {
        cudaFuncAttributes fr;
        if (cudaFuncGetAttributes(&fr, fn) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        static_max = std::max(static_max, fr.sharedSizeBytes);
    }
    return (size_t) optin - static_max;
}

size_t plan_smem_bytes(const PlanLaunch &lp) {
    return plan_header_bytes(lp.header_steps) + 128 + lp.ws_smem_bytes + lp.stage_bytes + lp.tile_bytes;
}

cudaError_t launch_plan(const PlanLaunch &lp, bool mixed, int grid, cudaStream_t stream, int variant) {
    if (lp.n_instances <= 0) return cudaSuccess;
    const size_t smem = plan_smem_bytes(lp);
    cudaError_t e = plan_attributes();
    if (e != cudaSuccess) return e;
    if (grid <= 0 || grid > lp.n_instances) grid = lp.n_instances;
    plan_kernel_fn(mixed, variant)<<<grid, plan_threads(variant), smem, stream>>>(lp);
    return cudaGetLastError();
}

int resident_capacity(size_t smem_bytes, int variant) {
    int per_sm = 0;
    plan_attributes();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, resident_kernel_fn(variant), plan_threads(resident_variant(variant)),
                                                  smem_bytes);
    cudaGetLastError();
    return num_sms() * std::max(per_sm, 0);
}

cudaError_t launch_resident(const ResidentLaunch &rl, cudaStream_t stream, int variant) {
    if (rl.lp.n_instances <= 0) return cudaSuccess;
    cudaError_t e = plan_attributes();
    if (e != cudaSuccess) return e;
    resident_kernel_fn(variant)<<<rl.lp.n_instances, plan_threads(resident_variant(variant)), plan_smem_bytes(rl.lp),
                                  stream>>>(rl);
    return cudaGetLastError();
}

}  // namespace qtg
