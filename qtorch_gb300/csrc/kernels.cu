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

constexpr int kPlanThreads = 256;
constexpr int kMaxLevelSteps = 64;      // steps of one level staged in shared memory per sub-batch
constexpr int kTableEntries = 4096;     // shared k-offset table entries per sub-batch

struct PlanShared {
    StepDesc steps[kMaxLevelSteps];        // descriptors of the sub-batch
    uint32_t prefix[kMaxLevelSteps + 1];   // first work item of each step (aligned to its lane group)
    uint32_t tbl_start[kMaxLevelSteps];    // start of each step's k table (or kNoTable)
    int32_t group[kMaxLevelSteps];         // lanes per output (power of two, <= 16)
    uint32_t maxbits[kMaxLevelSteps];      // max |C| bits per step (mixed)
    uint32_t tbl_a[kTableEntries];
    uint32_t tbl_b[kTableEntries];
};

constexpr uint32_t kNoTable = 0xffffffffu;

template <bool kMixed>
__device__ void plan_level(const PlanDesc &P, const InstanceDesc &I, const CtaScratch &W, int s_begin, int s_end,
                           PlanShared &sh) {
    const int tid = threadIdx.x;
    const int ns = s_end - s_begin;
    // ---- stage descriptors
    {
        const uint64_t *src = reinterpret_cast<const uint64_t *>(P.steps + s_begin);
        uint64_t *dst = reinterpret_cast<uint64_t *>(sh.steps);
        const int words = ns * (int) (sizeof(StepDesc) / 8);
        for (int w = tid; w < words; w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
    // ---- per-step work sizes, lane groups, table layout
    if (tid == 0) {
        uint32_t acc = 0, tacc = 0;
        for (int i = 0; i < ns; i++) {
            const StepDesc &d = sh.steps[i];
            const uint32_t n_out = 1u << (2 * d.nFree);
            const uint32_t K = 1u << (2 * d.nSum);
            uint32_t g = 1;
            if (kMixed && !(d.flags & kCF64)) {
                // split the k loop of tiny outputs across up to 16 lanes
                while (g < 16 && g * 2 <= K && n_out * g * 2 <= (uint32_t) blockDim.x) g *= 2;
            }
            acc = (acc + g - 1) / g * g;   // lane groups start on a multiple of their size
            sh.group[i] = (int) g;
            sh.prefix[i] = acc;
            acc += n_out * g;
            if (tacc + K <= (uint32_t) kTableEntries) {
                sh.tbl_start[i] = tacc;
                tacc += K;
            } else {
                sh.tbl_start[i] = kNoTable;
            }
            sh.maxbits[i] = 0;
        }
        sh.prefix[ns] = acc;
    }
    __syncthreads();
    // ---- k-offset tables (element offsets; interpreter tensors are < 4^16 elements)
    for (int i = 0; i < ns; i++) {
        const uint32_t t0 = sh.tbl_start[i];
        if (t0 == kNoTable) continue;
        const StepDesc &d = sh.steps[i];
        const uint32_t K = 1u << (2 * d.nSum);
        for (uint32_t k = tid; k < K; k += blockDim.x) {
            sh.tbl_a[t0 + k] = (uint32_t) scatter_digits(k, d.posAs, d.nSum);
            sh.tbl_b[t0 + k] = (uint32_t) scatter_digits(k, d.posBs, d.nSum);
        }
    }
    __syncthreads();
    // ---- compute
    const uint32_t total = sh.prefix[ns];
    for (uint32_t base = 0; base < total; base += blockDim.x) {
        const uint32_t item = base + tid;
        int si = 0;
        if (item < total) {
            int lo = 0, hi = ns - 1;   // last step whose first item is <= item
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (sh.prefix[mid] <= item) lo = mid; else hi = mid - 1;
            }
            si = lo;
        }
        const StepDesc &d = sh.steps[si];
        const uint32_t g = (uint32_t) sh.group[si];
        const uint32_t local = item - sh.prefix[si];
        const uint32_t c = local / g;
        const uint32_t lane_k = local % g;
        const uint32_t n_out = 1u << (2 * d.nFree);
        const bool valid = item < total && c < n_out;
        const uint32_t K = 1u << (2 * d.nSum);
        const uint32_t flags = d.flags;
        const char *abase = ((flags & kALeaf) ? I.leaves : W.workspace) + d.a_off;
        const char *bbase = ((flags & kBLeaf) ? I.leaves : W.workspace) + d.b_off;
        uint32_t oa0 = 0, ob0 = 0;
        if (valid) {
            uint64_t oa, ob;
            scatter_c(c, d, oa, ob);
            oa0 = (uint32_t) oa;
            ob0 = (uint32_t) ob;
        }
        const uint32_t t0 = sh.tbl_start[si];
        if (!kMixed) {
            const double2 *A = reinterpret_cast<const double2 *>(abase);
            const double2 *B = reinterpret_cast<const double2 *>(bbase);
            if (valid) {
                double cre = 0.0, cim = 0.0;
                for (uint32_t k = 0; k < K; k++) {
                    uint32_t ka, kb;
                    if (t0 != kNoTable) { ka = sh.tbl_a[t0 + k]; kb = sh.tbl_b[t0 + k]; }
                    else { ka = (uint32_t) scatter_digits(k, d.posAs, d.nSum); kb = (uint32_t) scatter_digits(k, d.posBs, d.nSum); }
                    cmac_exact(cre, cim, A[oa0 + ka], B[ob0 + kb]);
                }
                reinterpret_cast<double2 *>(W.workspace + d.c_off)[c] = make_double2(cre, cim);
            }
        } else {
            const bool f64 = (flags & kCF64) != 0;
            const bool a64 = (flags & kAF64) != 0, b64 = (flags & kBF64) != 0;
            double dre = 0.0, dim = 0.0;
            float fre = 0.f, fim = 0.f;
            if (valid) {
                for (uint32_t k = lane_k; k < K; k += g) {
                    uint32_t ka, kb;
                    if (t0 != kNoTable) { ka = sh.tbl_a[t0 + k]; kb = sh.tbl_b[t0 + k]; }
                    else { ka = (uint32_t) scatter_digits(k, d.posAs, d.nSum); kb = (uint32_t) scatter_digits(k, d.posBs, d.nSum); }
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
                float mag;
                if (f64) {
                    reinterpret_cast<double2 *>(W.workspace + d.c_off)[c] = make_double2(dre, dim);
                    mag = (float) fmax(fabs(dre), fabs(dim));
                } else {
                    reinterpret_cast<float2 *>(W.workspace + d.c_off)[c] = make_float2(fre, fim);
                    mag = fmaxf(fabsf(fre), fabsf(fim));
                }
                atomicMax(&sh.maxbits[si], __float_as_uint(mag));
            }
        }
    }
    __syncthreads();
    if constexpr (!kMixed) return;
    // ---- power-of-two normalisation of every C of this sub-batch
    for (int i = 0; i < ns; i++) {
        const StepDesc &d = sh.steps[i];
        const float mx = __uint_as_float(sh.maxbits[i]);
        int e = 0;
        if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
        const uint32_t n_out = 1u << (2 * d.nFree);
        if (e != 0) {
            if (d.flags & kCF64) {
                double2 *Cp = reinterpret_cast<double2 *>(W.workspace + d.c_off);
                for (uint32_t c = tid; c < n_out; c += blockDim.x) {
                    const double2 v = Cp[c];
                    Cp[c] = make_double2(ldexp(v.x, -e), ldexp(v.y, -e));
                }
            } else {
                float2 *Cp = reinterpret_cast<float2 *>(W.workspace + d.c_off);
                for (uint32_t c = tid; c < n_out; c += blockDim.x) {
                    const float2 v = Cp[c];
                    Cp[c] = make_float2(ldexpf(v.x, -e), ldexpf(v.y, -e));
                }
            }
        }
        if (tid == 0) {
            const int ea = d.a_step >= 0 ? W.exps[d.a_step] : 0;
            const int eb = d.b_step >= 0 ? W.exps[d.b_step] : 0;
            W.exps[s_begin + i] = ea + eb + e;
        }
    }
    __syncthreads();
}

template <bool kMixed>
__global__ void __launch_bounds__(kPlanThreads)
plan_kernel(const InstanceDesc *__restrict__ instances, int n_instances, char *ws_base, uint64_t ws_stride,
            int32_t *exps_base, uint64_t exps_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PlanShared &sh = *reinterpret_cast<PlanShared *>(smem_raw);
    CtaScratch W;
    W.workspace = ws_base + (uint64_t) blockIdx.x * ws_stride;
    W.exps = exps_base ? exps_base + (uint64_t) blockIdx.x * exps_stride : nullptr;
    for (int inst = blockIdx.x; inst < n_instances; inst += gridDim.x) {
        const InstanceDesc I = instances[inst];
        const PlanDesc P = *I.plan;
        for (int L = 0; L < P.n_levels; L++) {
            const int s0 = P.level_start[L], s1 = P.level_start[L + 1];
            for (int sb = s0; sb < s1; sb += kMaxLevelSteps) {
                const int se = (s1 - sb) < kMaxLevelSteps ? s1 : sb + kMaxLevelSteps;
                plan_level<kMixed>(P, I, W, sb, se, sh);
            }
        }
        // final-value rule of src/Network.h:961-965, applied in contraction order
        if (threadIdx.x == 0) {
            double fre = 0.0, fim = 0.0;
            for (int r = 0; r < P.n_rank0; r++) {
                const StepDesc &d = P.steps[P.rank0_steps[r]];
                double vre, vim;
                if (!kMixed || (d.flags & kCF64)) {
                    const double2 v = *reinterpret_cast<const double2 *>(W.workspace + d.c_off);
                    vre = v.x; vim = v.y;
                } else {
                    const float2 v = *reinterpret_cast<const float2 *>(W.workspace + d.c_off);
                    vre = v.x; vim = v.y;
                }
                if (kMixed) {
                    const int e = W.exps[P.rank0_steps[r]];
                    vre = ldexp(vre, e);
                    vim = ldexp(vim, e);
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

size_t plan_smem_bytes() { return sizeof(PlanShared); }

int plan_max_grid() {
    // resident CTAs: 256 threads and ~41 KB of shared memory each
    return num_sms() * 4;
}

cudaError_t launch_plan(const InstanceDesc *instances, int n_instances, bool mixed, int grid, char *ws_base,
                        uint64_t ws_stride, int32_t *exps_base, uint64_t exps_stride, cudaStream_t stream) {
    if (n_instances <= 0) return cudaSuccess;
    const size_t smem = sizeof(PlanShared);
    static bool attr_done[2] = {false, false};
    if (!attr_done[mixed]) {
        cudaError_t e = mixed ? cudaFuncSetAttribute(plan_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                              : cudaFuncSetAttribute(plan_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
        if (e != cudaSuccess) return e;
        attr_done[mixed] = true;
    }
    if (grid <= 0 || grid > n_instances) grid = n_instances;
    if (mixed) plan_kernel<true><<<grid, kPlanThreads, smem, stream>>>(instances, n_instances, ws_base, ws_stride, exps_base, exps_stride);
    else plan_kernel<false><<<grid, kPlanThreads, smem, stream>>>(instances, n_instances, ws_base, ws_stride, exps_base, exps_stride);
    return cudaGetLastError();
}

}  // namespace qtg
