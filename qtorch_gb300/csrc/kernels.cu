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

template <bool kMixed>
__device__ void plan_level(const StepDesc *__restrict__ steps, int s0, int s1, uint32_t total, const char *leaves,
                           char *ws, PlanSmemHeader &h, const ushort2 *__restrict__ tables) {
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
        const uint32_t tab = d.tab_off;
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
                reinterpret_cast<double2 *>(ws + d.c_off)[c] = make_double2(cre, cim);
            }
        } else {
            const bool f64 = (flags & kCF64) != 0;
            const bool a64 = (flags & kAF64) != 0, b64 = (flags & kBF64) != 0;
            double dre = 0.0, dim = 0.0;
            float fre = 0.f, fim = 0.f;
            if (valid) {
                if (!f64 && !a64 && !b64 && tab != kNoTable) {
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
                        double2 a, b;
                        if (a64) a = reinterpret_cast<const double2 *>(abase)[oa0 + ka];
                        else { const float2 t = reinterpret_cast<const float2 *>(abase)[oa0 + ka]; a = make_double2(t.x, t.y); }
                        if (b64) b = reinterpret_cast<const double2 *>(bbase)[ob0 + kb];
                        else { const float2 t = reinterpret_cast<const float2 *>(bbase)[ob0 + kb]; b = make_double2(t.x, t.y); }
                        if (f64) {
                            cmac_f64(dre, dim, a, b);
                        } else {
                            cmac_f32(fre, fim, make_float2((float) a.x, (float) a.y), make_float2((float) b.x, (float) b.y));
                        }
                    }
                }
            }
            // lane groups are aligned inside a warp; every lane takes part in the shuffles,
            // which run only as far as the widest group of the warp needs
            const uint32_t gmax = __reduce_max_sync(0xffffffffu, valid ? g : 1u);
            const bool dbl = __any_sync(0xffffffffu, valid && f64 && g > 1);
            for (uint32_t off = gmax >> 1; off >= 1; off >>= 1) {
                const float ore = __shfl_xor_sync(0xffffffffu, fre, (int) off);
                const float oim = __shfl_xor_sync(0xffffffffu, fim, (int) off);
                if (off < g) { fre += ore; fim += oim; }
                if (dbl) {
                    const double dro = __shfl_xor_sync(0xffffffffu, dre, (int) off);
                    const double dio = __shfl_xor_sync(0xffffffffu, dim, (int) off);
                    if (off < g) { dre += dro; dim += dio; }
                }
            }
            if (valid && lane_k == 0) {
                const int ma = step_scale(h, d.a_step), mb = step_scale(h, d.b_step);
                float mag;
                if (f64) {
                    dre = scale2d(dre, -(ma + mb));
                    dim = scale2d(dim, -(ma + mb));
                    reinterpret_cast<double2 *>(ws + d.c_off)[c] = make_double2(dre, dim);
                    mag = (float) fmax(fabs(dre), fabs(dim));
                } else {
                    fre = scale2f(fre, -(ma + mb));
                    fim = scale2f(fim, -(ma + mb));
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

// Bounded wait: a bulk copy finishes in microseconds; after ~1 s of polling the
// wait gives up and the instance reports NaN instead of hanging the CTA.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
    for (uint32_t it = 0; it < (1u << 22); it++) {
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

template <bool kMixed>
__global__ void __launch_bounds__(kPlanThreads, 2) plan_kernel(const PlanLaunch lp) {
    extern __shared__ __align__(256) unsigned char smem_raw[];
    PlanSmemHeader &h = *reinterpret_cast<PlanSmemHeader *>(smem_raw);
    uint64_t *mbar_slot = reinterpret_cast<uint64_t *>(smem_raw + kPlanHeaderBytes);
    unsigned char *region = smem_raw + kPlanHeaderBytes + 128;
    char *const ws_smem = reinterpret_cast<char *>(region);
    char *const ws_global = lp.ws_base ? lp.ws_base + (uint64_t) blockIdx.x * lp.ws_stride : nullptr;
    unsigned char *stage = region + lp.ws_smem_bytes;
    const uint32_t mbar = smem_addr(mbar_slot);
    if (lp.stage_bytes && threadIdx.x == 0) {
        mbar_init(mbar);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t parity = 0;
    for (int inst = blockIdx.x; inst < lp.n_instances; inst += gridDim.x) {
        const InstanceDesc I = lp.instances[inst];
        char *const ws = I.ws_bytes <= lp.ws_smem_bytes ? ws_smem : ws_global;
        const bool staged = lp.stage_bytes && I.plan_bytes && I.plan_bytes + I.leaf_bytes <= lp.stage_bytes;
        const StepDesc *steps;
        const int32_t *level_start, *rank0_steps;
        const uint32_t *level_items;
        const ushort2 *tables;
        const char *leaves;
        PlanDesc P;
        if (staged) {
            if (threadIdx.x == 0) {
                // the previous instance's generic reads of this region are ordered before the async writes
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(mbar, I.plan_bytes + I.leaf_bytes);
                bulk_copy_chunks(stage, reinterpret_cast<const char *>(I.plan), I.plan_bytes, mbar);
                bulk_copy_chunks(stage + I.plan_bytes, I.leaves, I.leaf_bytes, mbar);
            }
            const bool ok = mbar_wait_bounded(mbar, parity);
            parity ^= 1u;
            if (__syncthreads_or(!ok)) {
                // the copies never completed: this CTA's instances report NaN instead of hanging
                if (threadIdx.x == 0)
                    for (int j = inst; j < lp.n_instances; j += gridDim.x)
                        lp.instances[j].value[0] = lp.instances[j].value[1] = __longlong_as_double(0x7ff8000000000000ll);
                return;
            }
            P = *reinterpret_cast<const PlanDesc *>(stage);
            const char *gbase = reinterpret_cast<const char *>(I.plan);
            const char *sbase = reinterpret_cast<const char *>(stage);
            steps = reinterpret_cast<const StepDesc *>(sbase + (reinterpret_cast<const char *>(P.steps) - gbase));
            level_start = reinterpret_cast<const int32_t *>(sbase + (reinterpret_cast<const char *>(P.level_start) - gbase));
            rank0_steps = reinterpret_cast<const int32_t *>(sbase + (reinterpret_cast<const char *>(P.rank0_steps) - gbase));
            level_items = reinterpret_cast<const uint32_t *>(sbase + (reinterpret_cast<const char *>(P.level_items) - gbase));
            tables = reinterpret_cast<const ushort2 *>(sbase + (reinterpret_cast<const char *>(P.tables) - gbase));
            leaves = sbase + I.plan_bytes;
        } else {
            P = *I.plan;
            steps = P.steps;
            level_start = P.level_start;
            rank0_steps = P.rank0_steps;
            level_items = P.level_items;
            tables = P.tables;
            leaves = I.leaves;
        }
        if (kMixed) {
            for (int s = threadIdx.x; s < P.n_steps; s += blockDim.x) {
                h.maxbits[s] = 0;
                h.expo[s] = 0;
            }
            __syncthreads();
        }
        for (int L = 0; L < P.n_levels; L++) {
            plan_level<kMixed>(steps, level_start[L], level_start[L + 1], level_items[L], leaves, ws, h, tables);
            __syncthreads();
        }
        // final-value rule of src/Network.h:961-965, applied in contraction order
        if (threadIdx.x == 0) {
            double fre = 0.0, fim = 0.0;
            for (int r = 0; r < P.n_rank0; r++) {
                const int s = rank0_steps[r];
                const StepDesc &d = steps[s];
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

size_t plan_smem_bytes(const PlanLaunch &lp) {
    return kPlanHeaderBytes + 128 + lp.ws_smem_bytes + lp.stage_bytes;
}

cudaError_t launch_plan(const PlanLaunch &lp, bool mixed, int grid, cudaStream_t stream) {
    if (lp.n_instances <= 0) return cudaSuccess;
    const size_t smem = plan_smem_bytes(lp);
    cudaError_t e = mixed ? cudaFuncSetAttribute(plan_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                          : cudaFuncSetAttribute(plan_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    if (grid <= 0 || grid > lp.n_instances) grid = lp.n_instances;
    if (mixed) plan_kernel<true><<<grid, kPlanThreads, smem, stream>>>(lp);
    else plan_kernel<false><<<grid, kPlanThreads, smem, stream>>>(lp);
    return cudaGetLastError();
}

}  // namespace qtg
