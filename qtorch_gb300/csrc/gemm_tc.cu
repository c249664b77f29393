// Tensor-core (tcgen05) path for contraction steps dense enough to be a GEMM.
//
// A step C[m + M n] = sum_k A[a(m,k)] B[b(n,k)] in complex64 becomes one real
// GEMM  D = X Y^T  with
//   X (M x 2K)  = [Ar | Ai]                       row m, K contiguous
//   Y (2N x 2K) row 2n   = [Br_n | -Bi_n]          -> D[m][2n]   = Re C
//               row 2n+1 = [Bi_n |  Br_n]          -> D[m][2n+1] = Im C
// or, when B has more free indices than A (N > M), the other way round, so
// that the larger operand is packed twice instead of four times:
//   X (2M x 2K) row 2m   = [Ar_m | -Ai_m]          -> D[2m][n]   = Re C
//               row 2m+1 = [Ai_m |  Ar_m]          -> D[2m+1][n] = Im C
//   Y (N x 2K)  = [Br | Bi]
// computed with three TF32 products per term (x_hi y_hi + x_hi y_lo + x_lo y_hi,
// FP32 accumulation in tensor memory); with both parts rounded to nearest the
// dropped x_lo y_lo and the rounding of the lo parts leave ~2^-21 per product,
// unbiased.
//
// pack_operand writes X and Y (hi and lo planes) already in the UMMA canonical
// K-major layout without swizzle, tile by tile (128 rows x 32 columns, 16 KB),
// so every shared-memory stage is filled by one TMA bulk copy per plane.
// Inside a tile the 8x4 "core matrices" (8 rows x 16 bytes) are stored row
// group major: byte offset of (r, k) = ((r/8)*8 + k/4)*128 + (r%8)*16 + (k%4)*4,
// i.e. LBO (next core matrix along K) = 128 B, SBO (next 8-row group) = 1024 B.
//
// gemm_tf32x3: one CTA per 128x128 tile of D, 128 threads.  Thread 0 runs the
// pipeline (bulk copies into 3 stages, 12 tcgen05.mma per stage, tcgen05.commit
// to release a stage); all four warps read the accumulator with tcgen05.ld and
// store complex pairs.  Every mbarrier wait is bounded; on a timeout the CTA
// raises an error flag, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.cuh"
#include "gemm_tc.h"

namespace qtg {

constexpr int kTileM = 128;          // rows of X per tile (UMMA M)
constexpr int kTileN = 128;          // rows of Y per tile (UMMA N, real columns of D)
constexpr int kTileK = 32;           // tf32 elements of K per stage (128 bytes)
constexpr int kTileBytes = kTileM * kTileK * 4;   // 16 KB, same for X and Y tiles
constexpr int kStages = 3;
constexpr uint64_t kGroupM = 8;      // row tiles per band of the CTA order
constexpr int kGemmThreads = 128;
// Accumulators in tensor memory (128 columns each): the hi*hi products rotate
// over kAccBig regions by k tile and the small hi*lo + lo*hi products have one
// of their own; the epilogue adds them in FP32.  Each region then takes a third
// of the big additions and the small terms are not absorbed by the big sum: on
// 1e8-MAC random circuits the error against FP64 fell from ~1e-6 (one shared
// accumulator) to 0.7-2e-7, at the same speed.
constexpr uint32_t kAccBig = 3;
constexpr uint32_t kTmemCols = 128 * (kAccBig + 1);

// Operand layout: tiles ordered [row tile][k tile], each kTileM x kTileK in the
// canonical core-matrix order, element (rr, kk) of a tile at
// ((rr / 8) * 8 + kk / 4) * 32 + (rr % 8) * 4 + kk % 4.

// x -> hi + lo, both exact TF32 values (10 explicit mantissa bits), each rounded
// to nearest (ties away from zero: add half an ulp of TF32, then clear the 13
// low bits).  Rounding both parts keeps the errors unbiased: truncation left
// x_lo with the sign of x, so the dropped x_lo * y_lo term had the sign of every
// product and accumulated along the summed range (~1e-6 on 1e8-MAC circuits).
__device__ __forceinline__ float round_tf32(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = round_tf32(x);
    lo = round_tf32(x - hi);   // x - hi is exact in FP32
}

// One operand (which: 0 = A into X, 1 = B into Y), `rows` rows, columns
// j < 2K (see the file comment); pairs: its rows come in (2e, 2e + 1) pairs.
// One CTA per (row tile, k tile of the first half of the columns):
// the tile's 128 row offsets and its column offsets into the gathered operand
// are computed once into shared memory, then every complex element the CTA
// covers is read once and written to all the places it goes -- single rows:
// (e, k) and (e, K + k); pairs: rows 2e and 2e + 1 at columns k and K + k -- split hi/lo, in
// the tiles' canonical core-matrix order (contiguous stores per warp).  The
// element-per-place version read X's elements twice and Y's four times.  With
// K = 16 a single k tile holds both halves (columns 0-15 and 16-31).
__global__ void __launch_bounds__(256) pack_tiles(const float2 *__restrict__ src, const StepDesc d, int which,
                                                  int pairs, uint64_t rows, uint64_t K, uint64_t k_tiles,
                                                  float *__restrict__ hi, float *__restrict__ lo) {
    __shared__ uint64_t row_off[kTileM];
    __shared__ uint64_t col_off[kTileK];
    const uint32_t tid = threadIdx.x;
    const uint64_t M = 1ull << (2 * d.fA);
    const bool one_tile = K < (uint64_t) kTileK;           // both halves in tile 0
    const uint64_t half_tiles = one_tile ? 0 : K / kTileK;  // tile of column K + k: tk + half_tiles
    // one-dimensional grid (a row-tile count can pass 65,535): k tile of the
    // first half fastest, then the row tile
    const uint64_t kt_half = one_tile ? 1 : half_tiles;
    const uint64_t tk = blockIdx.x % kt_half, tr = blockIdx.x / kt_half;
    const uint32_t kcols = one_tile ? (uint32_t) K : (uint32_t) kTileK;
    if (tid < (uint32_t) kTileM) {
        const uint64_t r = tr * kTileM + tid;
        uint64_t oa = 0, ob = 0;
        // X row m: A's free digits; Y rows 2n, 2n+1: the B digits of output column n
        const uint64_t e = pairs ? r >> 1 : r;   // the element's index along this operand's free digits
        if (r < rows) scatter_c(which == 0 ? e : e * M, d, oa, ob);
        row_off[tid] = which == 0 ? oa : ob;
    } else if (tid < (uint32_t) (kTileM + kTileK)) {
        const uint32_t kk = tid - kTileM;
        const uint64_t k = tk * kTileK + kk;
        col_off[kk] = kk < kcols && k < K ? scatter_digits(k, which == 0 ? d.posAs : d.posBs, d.nSum) : 0;
    }
    __syncthreads();
    const uint64_t tile_floats = kTileBytes / 4;
    float *const h0 = hi + (tr * k_tiles + tk) * tile_floats, *const l0 = lo + (tr * k_tiles + tk) * tile_floats;
    float *const h1 = hi + (tr * k_tiles + tk + half_tiles) * tile_floats;
    float *const l1 = lo + (tr * k_tiles + tk + half_tiles) * tile_floats;
    auto put = [](float *h, float *l, uint32_t p, float v) {
        float a, b;
        split_tf32(v, a, b);
        h[p] = a;
        l[p] = b;
    };
    for (uint32_t p = tid; p < (uint32_t) (kTileM * kTileK); p += blockDim.x) {
        // p = ((rr / 8) * 8 + kk / 4) * 32 + (rr % 8) * 4 + kk % 4 (tiled_offset inside a tile)
        const uint32_t kk = (p & 3u) | (((p >> 5) & 7u) << 2);
        const uint32_t rr = ((p >> 2) & 7u) | ((p >> 8) << 3);
        if (kk >= kcols) continue;             // the Im half of a one-tile operand: written below
        if (pairs && (rr & 1u)) continue;   // odd rows of a pair: written with the even one
        const uint64_t r = tr * kTileM + rr;
        float2 x = make_float2(0.f, 0.f);
        if (r < rows && tk * kTileK + kk < K) x = src[row_off[rr] + col_off[kk]];
        // the Im half's position: the same (rr, kk) in the second tile, or 16 columns on
        const uint32_t q = one_tile ? p + 128u : p;
        float *const hq = one_tile ? h0 : h1, *const lq = one_tile ? l0 : l1;
        if (!pairs) {
            put(h0, l0, p, x.x);
            put(hq, lq, q, x.y);
        } else {
            // row 2e = [re | -im], row 2e + 1 = [im | re]; row rr + 1 sits 4 floats on
            put(h0, l0, p, x.x);
            put(hq, lq, q, -x.y);
            put(h0, l0, p + 4u, x.y);
            put(hq, lq, q + 4u, x.x);
        }
    }
}

// ---------------------------------------------------------------------------
// PTX wrappers

__device__ __forceinline__ uint32_t sm_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init1(uint32_t mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Test hook of the pipeline's failure path (qt_debug_gemm_fault): with mode 1
// the producer issues no copies for the first k tile, so the MMA thread's wait
// for it (and the producer's for the stage it never frees) run out after
// g_gemm_fault_polls polls.
__device__ uint32_t g_gemm_fault_mode = 0;
__device__ uint32_t g_gemm_fault_polls = 0;

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t limit = 1u << 24) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(mbar), "r"(parity) : "memory");
        if (ok) return true;
        if (it > 128) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

// shared-memory matrix descriptor: K-major, no swizzle, LBO 128 B, SBO 1024 B
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t) ((addr >> 4) & 0x3fff);
    d |= (uint64_t) ((128 >> 4) & 0x3fff) << 16;
    d |= (uint64_t) ((1024 >> 4) & 0x3fff) << 32;
    d |= (uint64_t) 1 << 46;   // descriptor version of tcgen05
    return d;                  // base offset 0, layout type 0 = no swizzle
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 128
constexpr uint32_t kInstrDesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t) (kTileN >> 3) << 17) |
                                ((uint32_t) (kTileM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem_d), "l"(a), "l"(b), "r"(kInstrDesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__global__ void __launch_bounds__(kGemmThreads, 1)
gemm_tf32x3(const float *__restrict__ x_hi, const float *__restrict__ x_lo, const float *__restrict__ y_hi,
            const float *__restrict__ y_lo, uint64_t k_tiles, uint64_t M, uint64_t N2, int x_pairs,
            float2 *__restrict__ C, int *__restrict__ error_flag, const StepScaleRef sc) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // [stages x (x_hi, x_lo, y_hi, y_lo) tiles][full[stages], empty[stages], done][tmem address]
    unsigned char *tiles = smem;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kStages * 4 * kTileBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // Tile order for L2 reuse: CTAs run in bands of kGroupM row tiles, the
    // column tiles fastest within a band, so the CTAs resident at once share
    // the band's X tiles and the Y tiles they walk; X is read about once and Y
    // once per band (row-major order read all of X once per wave of columns).
    const uint64_t m_tiles = (M + kTileM - 1) / kTileM, n_tiles = (N2 + kTileN - 1) / kTileN;
    const uint64_t lin = blockIdx.x;
    const uint64_t band = lin / (kGroupM * n_tiles), first_m = band * kGroupM;
    const uint64_t rows_in_band = m_tiles - first_m < kGroupM ? m_tiles - first_m : kGroupM;
    const uint64_t within = lin - band * kGroupM * n_tiles;
    const uint64_t tm = first_m + within % rows_in_band, tn = within / rows_in_band;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(sm_addr(tmem_slot)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2 * kStages + 1; i++) mbar_init1(sm_addr(&bars[i]));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // Warp-specialised: lane 0 of warp 1 streams the operand tiles into the
    // stage ring (waiting for the MMAs that read a stage before refilling it),
    // thread 0 issues the MMAs as tiles land, so the tensor pipe always has the
    // next k tile queued.  Every wait is bounded; a timeout stops both roles,
    // the copies already issued are waited for, and the error flag is set.
    __shared__ uint64_t s_issued, s_consumed;
    const bool hook = g_gemm_fault_mode == 1;
    const uint32_t limit = hook ? g_gemm_fault_polls : 1u << 24;
    bool ok = true;
    auto stage_ptr = [&](int s, int plane) { return tiles + (s * 4 + plane) * kTileBytes; };
    if (warp == 1 && lane == 0) {
        const uint64_t tile_floats = kTileBytes / 4;
        uint32_t empty_phase[kStages] = {0, 0, 0};
        uint64_t kt = 0;
        for (; kt < k_tiles; kt++) {
            const int s = (int) (kt % kStages);
            if (kt >= (uint64_t) kStages) {
                if (!mbar_wait(sm_addr(&bars[kStages + s]), empty_phase[s], limit)) { ok = false; break; }
                empty_phase[s] ^= 1u;
            }
            if (hook && kt == 0) continue;   // the test hook: this tile never arrives
            const uint32_t full = sm_addr(&bars[s]);
            mbar_arrive_tx(full, 4 * kTileBytes);
            const uint64_t xt = (tm * k_tiles + kt) * tile_floats, yt = (tn * k_tiles + kt) * tile_floats;
            bulk_load(sm_addr(stage_ptr(s, 0)), x_hi + xt, kTileBytes, full);
            bulk_load(sm_addr(stage_ptr(s, 1)), x_lo + xt, kTileBytes, full);
            bulk_load(sm_addr(stage_ptr(s, 2)), y_hi + yt, kTileBytes, full);
            bulk_load(sm_addr(stage_ptr(s, 3)), y_lo + yt, kTileBytes, full);
        }
        s_issued = kt;
    }
    if (threadIdx.x == 0) {
        uint32_t full_phase[kStages] = {0, 0, 0};
        uint64_t kt = 0;
        for (; kt < k_tiles; kt++) {
            const int s = (int) (kt % kStages);
            if (!mbar_wait(sm_addr(&bars[s]), full_phase[s], limit)) { ok = false; break; }
            full_phase[s] ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t xh = sm_addr(stage_ptr(s, 0)), xl = sm_addr(stage_ptr(s, 1));
            const uint32_t yh = sm_addr(stage_ptr(s, 2)), yl = sm_addr(stage_ptr(s, 3));
            const uint32_t big = tmem + (uint32_t) (kt % kAccBig) * 128u, small = tmem + kAccBig * 128u;
            for (int j = 0; j < kTileK / 8; j++) {
                // 8 tf32 of K per instruction = two core matrices = 256 bytes along K
                const uint32_t o = (uint32_t) j * 256;
                const uint32_t acc_big = (kt >= kAccBig || j > 0) ? 1u : 0u;
                const uint32_t acc_small = (kt > 0 || j > 0) ? 1u : 0u;
                mma_tf32(big, smem_desc(xh + o), smem_desc(yh + o), acc_big);
                mma_tf32(small, smem_desc(xh + o), smem_desc(yl + o), acc_small);
                mma_tf32(small, smem_desc(xl + o), smem_desc(yh + o), 1u);
            }
            mma_commit(sm_addr(&bars[kStages + s]));   // the stage is free once these MMAs have read it
        }
        s_consumed = kt;
        mma_commit(sm_addr(&bars[2 * kStages]));
    }
    // every thread waits for the accumulator (bounded)
    ok = __syncthreads_and(ok) != 0;
    const int shift = scale_shift(sc);
    uint32_t lmax = 0;
    if (!ok && warp == 1 && lane == 0) {
        // after a timeout: the copies issued but never consumed land before the CTA leaves
        for (uint64_t kt = s_consumed; kt < s_issued; kt++) {
            if (hook && kt == 0) continue;   // never issued
            const int s = (int) (kt % kStages);
            mbar_wait(sm_addr(&bars[s]), (uint32_t) ((kt / kStages) & 1u));
        }
    }
    // the MMAs issued so far (all of them, or those before a timeout) finish
    // before the accumulator is read or released
    bool done = mbar_wait(sm_addr(&bars[2 * kStages]), 0);
    done = __syncthreads_and(ok && done) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done) {
        // row of D this thread holds (its TMEM lane); X's rows: M (single) or
        // 2 x the complex rows (pairs: the even row Re, the odd row Im)
        const uint64_t m = tm * kTileM + (uint64_t) warp * 32 + lane;
        const uint64_t Mc = x_pairs ? M >> 1 : M;   // complex rows of C
        const uint32_t n_big = k_tiles < kAccBig ? (uint32_t) k_tiles : kAccBig;
        for (int c0 = 0; c0 < kTileN; c0 += 16) {
            float v[16];
            // the small accumulator last: ((big0 + big1) + big2) + small
            for (uint32_t reg = 0; reg <= n_big; reg++) {
                const uint32_t region = reg < n_big ? reg : kAccBig;
                uint32_t r[16];
                const uint32_t taddr = tmem + ((uint32_t) (warp * 32) << 16) + region * 128u + (uint32_t) c0;
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                               "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                               "=r"(r[14]), "=r"(r[15])
                             : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = reg == 0 ? __uint_as_float(r[j]) : v[j] + __uint_as_float(r[j]);
            }
            if (x_pairs) {
                // lanes 2i and 2i + 1 hold Re and Im of complex row m >> 1 for
                // the same 16 columns: each takes its partner's values and
                // stores half of the columns (the even lane the even ones)
                float o[16];
#pragma unroll
                for (int j = 0; j < 16; j++) o[j] = __shfl_xor_sync(0xffffffffu, v[j], 1);
                const uint32_t odd = (uint32_t) (m & 1u);
                if (m < M) {
#pragma unroll
                    for (int j = 0; j < 16; j += 2) {
                        // even lane: column j, (v, o); odd lane: column j + 1, (o, v)
                        const uint64_t col = tn * kTileN + (uint64_t) (c0 + j) + odd;
                        if (col < N2) {
                            const float re = odd ? o[j + 1] : v[j], im = odd ? v[j + 1] : o[j];
                            const float2 out = make_float2(scale_pow2(re, shift), scale_pow2(im, shift));
                            lmax = max(lmax, mag_bits(out));
                            C[(m >> 1) + Mc * col] = out;
                        }
                    }
                }
            } else if (m < M) {
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    const uint64_t col = tn * kTileN + (uint64_t) (c0 + j);   // even: Re, odd: Im
                    if (col + 1 < N2 + 1 && col < N2) {
                        const float2 out = make_float2(scale_pow2(v[j], shift), scale_pow2(v[j + 1], shift));
                        lmax = max(lmax, mag_bits(out));
                        C[m + Mc * (col >> 1)] = out;
                    }
                }
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(error_flag, 1);
    }
    scale_note(sc, lmax, shift, blockIdx.x == 0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---------------------------------------------------------------------------

bool gemm_eligible(const StepDesc &d) {
    // A's free digits must be C's low digits and B's the high ones (what ContractNodes produces)
    for (int i = 0; i < d.nFree; i++) {
        const bool from_a = d.cA[i] != kNoWire;
        if (from_a != (i < d.fA)) return false;
    }
    const uint64_t M = 1ull << (2 * d.fA), N = 1ull << (2 * d.fB), K = 1ull << (2 * d.nSum);
    return M >= (uint64_t) kTileM && 2 * N >= 64 && 2 * K >= (uint64_t) kTileK && M * N * K >= (1ull << 26);
}

GemmSizes gemm_sizes(const StepDesc &d) {
    GemmSizes s;
    // the operand with more free indices is packed twice, the other four times
    s.x_pairs = d.fB > d.fA;
    const uint64_t Mc = 1ull << (2 * d.fA), Nc = 1ull << (2 * d.fB);
    s.M = s.x_pairs ? 2 * Mc : Mc;
    s.N2 = s.x_pairs ? Nc : 2 * Nc;
    s.K = 1ull << (2 * d.nSum);
    s.k_tiles = (2 * s.K + kTileK - 1) / kTileK;
    s.m_tiles = (s.M + kTileM - 1) / kTileM;
    s.n_tiles = (s.N2 + kTileN - 1) / kTileN;
    s.x_floats = s.m_tiles * kTileM * s.k_tiles * kTileK;
    s.y_floats = s.n_tiles * kTileN * s.k_tiles * kTileK;
    return s;
}

cudaError_t gemm_set_fault(int mode, uint32_t polls) {
    const uint32_t m = (uint32_t) mode, p = polls ? polls : 1u;
    cudaError_t e = cudaMemcpyToSymbol(g_gemm_fault_mode, &m, sizeof m);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_gemm_fault_polls, &p, sizeof p);
    return e;
}

size_t gemm_smem_bytes() { return (size_t) kStages * 4 * kTileBytes + (2 * kStages + 1) * 8 + 16; }

cudaError_t launch_gemm_step(const StepDesc &d, const float2 *A, const float2 *B, float2 *C, float *scratch,
                             int *error_flag, cudaStream_t stream, const StepScaleRef &sc) {
    const GemmSizes s = gemm_sizes(d);
    float *xh = scratch, *xl = xh + s.x_floats, *yh = xl + s.x_floats, *yl = yh + s.y_floats;
    // one CTA per k tile of the first half of the columns and row tile (the
    // second half's tiles are written by the same CTAs)
    const uint64_t kt_half = s.K < (uint64_t) kTileK ? 1 : s.K / kTileK;
    if (kt_half * s.m_tiles > 0x7fffffffull || kt_half * s.n_tiles > 0x7fffffffull) return cudaErrorInvalidValue;
    pack_tiles<<<(unsigned) (kt_half * s.m_tiles), 256, 0, stream>>>(A, d, 0, s.x_pairs ? 1 : 0, s.M, s.K, s.k_tiles,
                                                                      xh, xl);
    pack_tiles<<<(unsigned) (kt_half * s.n_tiles), 256, 0, stream>>>(B, d, 1, s.x_pairs ? 0 : 1, s.N2, s.K, s.k_tiles,
                                                                      yh, yl);
    const size_t smem = gemm_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(gemm_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    const uint64_t ctas = s.m_tiles * s.n_tiles;
    if (ctas > 0x7fffffffull) return cudaErrorInvalidValue;
    gemm_tf32x3<<<(unsigned) ctas, kGemmThreads, smem, stream>>>(xh, xl, yh, yl, s.k_tiles, s.M, s.N2,
                                                                 s.x_pairs ? 1 : 0, C, error_flag, sc);
    return cudaGetLastError();
}

}  // namespace qtg
