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
//    intermediates stay in an L2-resident per-instance workspace.  Mixed mode
//    keeps every intermediate normalised by a power of two (per-tensor
//    exponent) and runs rank-0/1 outputs (the expectation-value reductions)
//    in FP64.
#include <cuda_runtime.h>
#include <cstdint>
#include "engine.cuh"
#include "kernels.h"

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

__device__ __forceinline__ void cmac_f64(double &cre, double &cim, double2 a, double2 b) {
    cre = fma(a.x, b.x, cre);
    cre = fma(-a.y, b.y, cre);
    cim = fma(a.x, b.y, cim);
    cim = fma(a.y, b.x, cim);
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

template <typename T>
__global__ void __launch_bounds__(kPairThreads)
pair_kernel(const typename Vec2<T>::type *__restrict__ A, const typename Vec2<T>::type *__restrict__ B,
            typename Vec2<T>::type *__restrict__ C, const StepDesc d, uint64_t n_out, uint64_t K) {
    using V = typename Vec2<T>::type;
    __shared__ uint64_t s_oa[kPairChunk];
    __shared__ uint64_t s_ob[kPairChunk];
    const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
    // every CTA walks the same number of outer iterations so that the
    // __syncthreads of the chunk loop stay uniform
    const uint64_t n_iter = (n_out + stride - 1) / stride;
    for (uint64_t it = 0; it < n_iter; it++) {
        const uint64_t c = it * stride + (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
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
            v.x = cre;
            v.y = cim;
            C[c] = v;
        }
    }
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
    uint32_t maxbits[kPlanMaxSteps];   // float bits of max |S| of each step's output
    int32_t expo[kPlanMaxSteps];       // E of each step's output
};

__device__ __forceinline__ int step_scale(const PlanSmemHeader &h, int step) {
    if (step < 0) return 0;
    const float mx = __uint_as_float(h.maxbits[step]);
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    return e;
}

template <bool kMixed>
__device__ void plan_level(const StepDesc *__restrict__ steps, int s0, int s1, uint32_t total, const char *leaves,
                           char *ws, PlanSmemHeader &h) {
    const int tid = threadIdx.x;
    for (uint32_t base = 0; base < total; base += blockDim.x) {
        const uint32_t item = base + tid;
        int si = s0;
        if (item < total) {
            int lo = s0, hi = s1 - 1;   // last step whose first item is <= item
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (steps[mid].item_start <= item) lo = mid; else hi = mid - 1;
            }
            si = lo;
        }
        const StepDesc &d = steps[si];
        const uint32_t g = d.group;
        const uint32_t local = item - d.item_start;
        const uint32_t c = local / g;
        const uint32_t lane_k = local % g;
        const int nFree = d.nFree, nSum = d.nSum;
        const uint32_t n_out = 1u << (2 * nFree);
        const bool valid = item < total && c < n_out;
        const uint32_t K = 1u << (2 * nSum);
        const uint32_t flags = d.flags;
        const char *abase = ((flags & kALeaf) ? leaves : ws) + d.a_off;
        const char *bbase = ((flags & kBLeaf) ? leaves : ws) + d.b_off;
        uint32_t oa0 = 0, ob0 = 0;
        if (valid) {
            uint64_t oa, ob;
            scatter_c(c, d, oa, ob);
            oa0 = (uint32_t) oa;
            ob0 = (uint32_t) ob;
        }
        if constexpr (!kMixed) {
            if (valid) {
                const double2 *A = reinterpret_cast<const double2 *>(abase);
                const double2 *B = reinterpret_cast<const double2 *>(bbase);
                double cre = 0.0, cim = 0.0;
                for (uint32_t k = 0; k < K; k++) {
                    const uint32_t ka = (uint32_t) scatter_digits(k, d.posAs, nSum);
                    const uint32_t kb = (uint32_t) scatter_digits(k, d.posBs, nSum);
                    cmac_exact(cre, cim, A[oa0 + ka], B[ob0 + kb]);
                }
                reinterpret_cast<double2 *>(ws + d.c_off)[c] = make_double2(cre, cim);
            }
        } else {
            const bool f64 = (flags & kCF64) != 0;
            const bool a64 = (flags & kAF64) != 0, b64 = (flags & kBF64) != 0;
            double dre = 0.0, dim = 0.0;
            float fre = 0.f, fim = 0.f;
            if (valid) {
                for (uint32_t k = lane_k; k < K; k += g) {
                    const uint32_t ka = (uint32_t) scatter_digits(k, d.posAs, nSum);
                    const uint32_t kb = (uint32_t) scatter_digits(k, d.posBs, nSum);
                    if (f64) {
                        double2 a, b;
                        if (a64) a = reinterpret_cast<const double2 *>(abase)[oa0 + ka];
                        else { const float2 t = reinterpret_cast<const float2 *>(abase)[oa0 + ka]; a = make_double2(t.x, t.y); }
                        if (b64) b = reinterpret_cast<const double2 *>(bbase)[ob0 + kb];
                        else { const float2 t = reinterpret_cast<const float2 *>(bbase)[ob0 + kb]; b = make_double2(t.x, t.y); }
                        cmac_f64(dre, dim, a, b);
                    } else {
                        float2 a, b;
                        if (a64) { const double2 t = reinterpret_cast<const double2 *>(abase)[oa0 + ka]; a = make_float2((float) t.x, (float) t.y); }
                        else a = reinterpret_cast<const float2 *>(abase)[oa0 + ka];
                        if (b64) { const double2 t = reinterpret_cast<const double2 *>(bbase)[ob0 + kb]; b = make_float2((float) t.x, (float) t.y); }
                        else b = reinterpret_cast<const float2 *>(bbase)[ob0 + kb];
                        cmac_f32(fre, fim, a, b);
                    }
                }
            }
            // lane groups are aligned inside a warp; every lane takes part in the shuffles
            for (int off = 8; off >= 1; off >>= 1) {
                const float ore = __shfl_xor_sync(0xffffffffu, fre, off);
                const float oim = __shfl_xor_sync(0xffffffffu, fim, off);
                if ((uint32_t) off < g) { fre += ore; fim += oim; }
            }
            if (valid && lane_k == 0) {
                const int ma = step_scale(h, d.a_step), mb = step_scale(h, d.b_step);
                const int shift = -(ma + mb);
                float mag;
                if (f64) {
                    dre = ldexp(dre, shift);
                    dim = ldexp(dim, shift);
                    reinterpret_cast<double2 *>(ws + d.c_off)[c] = make_double2(dre, dim);
                    mag = (float) fmax(fabs(dre), fabs(dim));
                } else {
                    fre = ldexpf(fre, shift);
                    fim = ldexpf(fim, shift);
                    reinterpret_cast<float2 *>(ws + d.c_off)[c] = make_float2(fre, fim);
                    mag = fmaxf(fabsf(fre), fabsf(fim));
                }
                atomicMax(&h.maxbits[si], __float_as_uint(mag));
                if (c == 0) {
                    const int ea = d.a_step >= 0 ? h.expo[d.a_step] : 0;
                    const int eb = d.b_step >= 0 ? h.expo[d.b_step] : 0;
                    h.expo[si] = ea + eb + ma + mb;
                }
            }
        }
    }
}

template <bool kMixed>
__global__ void __launch_bounds__(kPlanThreads)
plan_kernel(const InstanceDesc *__restrict__ instances, int n_instances, char *ws_base, uint64_t ws_stride,
            int ws_in_smem) {
    extern __shared__ __align__(256) unsigned char smem_raw[];
    PlanSmemHeader &h = *reinterpret_cast<PlanSmemHeader *>(smem_raw);
    char *ws = ws_in_smem ? reinterpret_cast<char *>(smem_raw) + kPlanHeaderBytes
                          : ws_base + (uint64_t) blockIdx.x * ws_stride;
    for (int inst = blockIdx.x; inst < n_instances; inst += gridDim.x) {
        const InstanceDesc I = instances[inst];
        const PlanDesc P = *I.plan;
        if (kMixed) {
            for (int s = threadIdx.x; s < P.n_steps; s += blockDim.x) {
                h.maxbits[s] = 0;
                h.expo[s] = 0;
            }
            __syncthreads();
        }
        for (int L = 0; L < P.n_levels; L++) {
            plan_level<kMixed>(P.steps, P.level_start[L], P.level_start[L + 1], P.level_items[L], I.leaves, ws, h);
            __syncthreads();
        }
        // final-value rule of src/Network.h:961-965, applied in contraction order
        if (threadIdx.x == 0) {
            double fre = 0.0, fim = 0.0;
            for (int r = 0; r < P.n_rank0; r++) {
                const int s = P.rank0_steps[r];
                const StepDesc &d = P.steps[s];
                double vre, vim;
                if (!kMixed || (d.flags & kCF64)) {
                    const double2 v = *reinterpret_cast<const double2 *>(ws + d.c_off);
                    vre = v.x; vim = v.y;
                } else {
                    const float2 v = *reinterpret_cast<const float2 *>(ws + d.c_off);
                    vre = v.x; vim = v.y;
                }
                if (kMixed) {
                    vre = ldexp(vre, h.expo[s]);
                    vim = ldexp(vim, h.expo[s]);
                }
                if ((fabs(fre) <= 1.0e-30 && fabs(fim) <= 1.0e-30) || (d.flags & kBothRank0)) {
                    fre = vre;
                    fim = vim;
                }
            }
            I.value[0] = fre;
            I.value[1] = fim;
        }
        __syncthreads();
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

cudaError_t launch_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64, cudaStream_t stream) {
    const uint64_t n_out = 1ull << (2 * d.nFree);
    const uint64_t K = 1ull << (2 * d.nSum);
    uint64_t blocks = (n_out + kPairThreads - 1) / kPairThreads;
    const uint64_t cap = (uint64_t) num_sms() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (f64)
        pair_kernel<double><<<(unsigned) blocks, kPairThreads, 0, stream>>>(
            (const double2 *) A, (const double2 *) B, (double2 *) C, d, n_out, K);
    else
        pair_kernel<float><<<(unsigned) blocks, kPairThreads, 0, stream>>>(
            (const float2 *) A, (const float2 *) B, (float2 *) C, d, n_out, K);
    return cudaGetLastError();
}

int plan_max_grid(size_t smem_bytes) {
    int per_sm = 0;
    cudaFuncSetAttribute(plan_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem_bytes);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plan_kernel<true>, kPlanThreads, smem_bytes);
    cudaGetLastError();
    if (per_sm < 1) per_sm = 1;
    return num_sms() * per_sm;
}

cudaError_t launch_plan(const InstanceDesc *instances, int n_instances, bool mixed, int grid, char *ws_base,
                        uint64_t ws_stride, bool ws_in_smem, cudaStream_t stream) {
    if (n_instances <= 0) return cudaSuccess;
    const size_t smem = kPlanHeaderBytes + (ws_in_smem ? ws_stride : 0);
    cudaError_t e = mixed ? cudaFuncSetAttribute(plan_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                          : cudaFuncSetAttribute(plan_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    if (grid <= 0 || grid > n_instances) grid = n_instances;
    if (mixed) plan_kernel<true><<<grid, kPlanThreads, smem, stream>>>(instances, n_instances, ws_base, ws_stride, ws_in_smem ? 1 : 0);
    else plan_kernel<false><<<grid, kPlanThreads, smem, stream>>>(instances, n_instances, ws_base, ws_stride, ws_in_smem ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace qtg
