// Streaming contraction of complex64 steps with one small operand (see
// stream.h).  One persistent CTA of 256 threads loops over tiles of the large
// operand L:
//
//   * a producer warp streams the tiles into a ring of kStreamStages shared-
//     memory stages with TMA bulk copies (cp.async.bulk, one per contiguous
//     run, completion counted on the stage's "full" mbarrier); the eight
//     consumer warps release a stage on its "empty" mbarrier once they have
//     read it, so no block-wide barrier is needed in the steady state and up
//     to kStreamStages tiles are in flight per CTA;
//   * thread t owns element t of every 256-element stretch of the tile (L's
//     wires 0-3), so a warp's loads are consecutive and conflict-free; its
//     loop over the tile's other digits is unrolled at compile time (one
//     instantiation per shape class: free indices of S, looped free and
//     summed digits), with every element's tile and S offsets precomputed in
//     registers, and its sums stay in registers across a work item's chunks;
//   * after a work item's last tile, the summed digits among wires 0-3 are
//     reduced by warp shuffles (wires 0-1) or through shared memory (wires
//     2-3), and the sums are written to C.
//
// HBM traffic is one read of L and S and one write of C: the step's
// algorithmic bytes.  The mixed form's per-tensor power-of-two scaling
// (scale.cuh) is applied to every stored value.  Every mbarrier wait is
// bounded; after a timeout the warps stop, the CTA waits (bounded) for the
// copies it issued, raises the error flag and leaves.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "kernels.h"
#include "stream.h"

namespace qtg {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Test hook for the failure path (qt_debug_stream_fault): with mode 1 the
// producer leaves the first tile of every CTA unissued -- a wait that nothing
// will ever complete -- and the pipeline waits give up after `polls` polls.
// Waits for copies that were issued always use the full limit.
__device__ uint32_t g_stream_fault_mode = 0;
__device__ uint32_t g_stream_fault_polls = 0;

// at most `limit` polls (2^22: tens of milliseconds with the back-off), then false
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit = 1u << 22) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if (it > 64) __nanosleep(32);
    }
    return false;
}

// the 256 consumer threads agree on v (named barrier 1 with an AND reduction),
// so that none of them stops at a barrier the others have left
__device__ __forceinline__ bool consumers_all(bool v) {
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                 : "=r"(r) : "r"((uint32_t) v), "r"(kStreamThreads) : "memory");
    return r != 0;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ void cmac(float2 &c, float2 a, float2 b) {
    c.x = fmaf(a.x, b.x, c.x);
    c.x = fmaf(-a.y, b.y, c.x);
    c.y = fmaf(a.x, b.y, c.y);
    c.y = fmaf(a.y, b.x, c.y);
}

__host__ __device__ inline uint32_t round128(uint32_t x) { return (x + 127u) / 128u * 128u; }

// byte offsets of the shared-memory regions (host and device agree)
__host__ __device__ inline void stream_layout(const StreamStep &p, uint32_t off[5]) {
    const uint32_t tile = 1u << (2 * (4 + p.go + p.ho));
    const uint32_t staged = p.staged ? 1u << (2 * p.n_dout) : 0u;
    off[0] = 0;                                                  // kStreamStages tile buffers
    off[1] = kStreamStages * round128(8u * tile);                // staged outputs of a pass
    off[2] = off[1] + round128(8u * staged);                     // S
    off[3] = off[2] + round128(8u * p.s_store);                  // full[stages], empty[stages], issued count,
                                                                 // C offsets and staged indices of (g, f)
    off[4] = off[3] + round128(16u * kStreamStages + 8u + 20u * kStreamMaxStage);   // end
}

// producer warp: the bulk copies of (item, chunk) into tile buffer `dst`
__device__ __forceinline__ void issue_tile(const StreamStep &p, float2 *dst, uint64_t *bar_ptr, uint32_t item,
                                           uint32_t chunk, uint32_t lane) {
    uint64_t lbase = 0;
    for (uint32_t j = 0; j < p.n_item_d; j++) lbase += (uint64_t) ((item >> (2 * j)) & 3u) << (2 * p.item_lw[j]);
    for (uint32_t j = 0; j < p.n_chunk_d; j++) lbase += (uint64_t) ((chunk >> (2 * j)) & 3u) << (2 * p.chunk_lw[j]);
    const uint32_t bar = smem_u32(bar_ptr);
    const uint32_t run_bytes = 8u * p.run_elems;
    if (lane == 0) {
        // the buffer's previous contents were read by ordinary loads before
        // the CTA barrier that precedes this; order them before the async writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect(bar, run_bytes * p.n_runs);
    }
    __syncwarp();
    for (uint32_t r = lane; r < p.n_runs; r += 32) {
        uint64_t off = lbase;
        for (uint32_t j = 0; j < p.n_run_d; j++) off += (uint64_t) ((r >> (2 * j)) & 3u) << (2 * p.run_lw[j]);
        bulk_g2s(smem_u32(dst + (uint64_t) r * p.run_elems), p.L + off, run_bytes, bar);
    }
}

// C offset of the in-pass sum (g, f) of a work item, beyond the work item's
// and pass's bases and the thread's own free digits among wires 0-3
__device__ __forceinline__ uint64_t out_offset(const StreamStep &p, uint32_t g, uint32_t f) {
    uint64_t o = 0;
    for (uint32_t j = 0; j < p.go; j++) o += (uint64_t) ((g >> (2 * j)) & 3u) << (2 * p.g_cd[j]);
    for (uint32_t j = 0; j < p.nsfp; j++) o += (uint64_t) ((f >> (2 * j)) & 3u) << (2 * p.sf_cd[j]);
    return o;
}

// staged index of the in-pass sum (g, f)
__device__ __forceinline__ uint32_t staged_index(const StreamStep &p, uint32_t g, uint32_t f) {
    uint32_t o = 0;
    for (uint32_t j = 0; j < p.go; j++) o += ((g >> (2 * j)) & 3u) << (2 * p.g_rank[j]);
    for (uint32_t j = 0; j < p.nsfp; j++) o += ((f >> (2 * j)) & 3u) << (2 * p.sf_rank[j]);
    return o;
}

// Two CTAs per SM for every class but 4 g x 4 S-free sums over 4 summed
// combinations, which runs one CTA per SM instead of spilling (measured faster
// than looping its g digit over work items at two); 16 S-free sums keep
// their element loop rolled and fit two.
template <int NSF, int G, int H>
constexpr int stream_min_ctas() { return NSF == 4 && G == 4 && H == 4 ? 1 : 2; }
template <int NSF, int G, int H>
__global__ void __launch_bounds__(kStreamBlock, stream_min_ctas<NSF, G, H>())
    stream_kernel(const __grid_constant__ StreamStep p) {
    constexpr int E = G * H;
    constexpr int M = G * NSF;   // sums a thread keeps per pass
    constexpr int NS = kStreamStages;
    extern __shared__ __align__(128) unsigned char smem[];
    uint32_t off[5];
    stream_layout(p, off);
    const uint32_t tile_elems = 1u << (2 * (4 + p.go + p.ho));
    const uint32_t tile_stride = round128(8u * tile_elems) / 8u;
    float2 *const tiles = reinterpret_cast<float2 *>(smem + off[0]);
    float2 *const ostage = reinterpret_cast<float2 *>(smem + off[1]);
    float2 *const S = reinterpret_cast<float2 *>(smem + off[2]);
    uint64_t *const full = reinterpret_cast<uint64_t *>(smem + off[3]);
    uint64_t *const empty = full + NS;
    uint32_t *const issued_slot = reinterpret_cast<uint32_t *>(empty + NS);
    uint64_t *const out_off = reinterpret_cast<uint64_t *>(empty + NS + 1);      // [M]
    uint32_t *const st_gf = reinterpret_cast<uint32_t *>(out_off + kStreamMaxStage);   // [M]
    uint32_t *const eo_s = st_gf + kStreamMaxStage;     // [E]: element offsets for the rolled loop
    uint32_t *const so_s = eo_s + kStreamMaxStage;      // [E]
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t n_out = 1u << (2 * p.n_dout);

    for (uint32_t e = tid; e < p.s_elems; e += blockDim.x) {
        uint32_t dst = 0;
        for (int w = 0; w < kStreamMaxSmallRank; w++) dst += ((e >> (2 * w)) & 3u) * p.s_unit[w];
        S[dst] = p.S[e];
    }
    if (tid < (uint32_t) M) {
        out_off[tid] = out_offset(p, tid / NSF, tid % NSF);
        st_gf[tid] = staged_index(p, tid / NSF, tid % NSF);
    }
    if (p.staged && p.klo_mode == 2)   // sums from several warps meet there by atomic adds
        for (uint32_t u = tid; u < n_out; u += blockDim.x) ostage[u] = make_float2(0.f, 0.f);
    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), kStreamConsumerWarps);
        }
        *issued_slot = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // this CTA's tiles: work items blockIdx.x, + gridDim.x, ..., each in n_chunks chunks
    const uint32_t my_items = blockIdx.x < p.n_items ? (p.n_items - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t n_t = my_items * p.n_chunks;
    const int shift = scale_shift(p.sc);
    uint32_t lmax = 0;
    bool ok = true;
    const bool skip_first = g_stream_fault_mode == 1;
    const uint32_t limit = g_stream_fault_polls ? g_stream_fault_polls : (1u << 22);

    if (warp == kStreamConsumerWarps) {
        // producer: fill stage t % NS once its previous tile has been released
        uint32_t t = 0;
        for (; t < n_t; t++) {
            const uint32_t s = t % NS;
            if (t >= (uint32_t) NS && !mbar_wait(smem_u32(&empty[s]), ((t / NS) - 1) & 1u, limit)) {
                ok = false;
                break;
            }
            if (t == 0 && skip_first) continue;   // test hook: this tile never arrives
            const uint32_t item = blockIdx.x + (t / p.n_chunks) * gridDim.x, chunk = t % p.n_chunks;
            issue_tile(p, tiles + (uint64_t) s * tile_stride, &full[s], item, chunk, lane);
        }
        if (lane == 0) *issued_slot = t;
    } else {
        // consumers: thread tid owns element tid of every 256-element stretch
        uint32_t s_lo = 0, c_lo = 0, st_lo = 0;
        for (int w = 0; w < 4; w++) {
            const uint32_t dg = (tid >> (2 * w)) & 3u;
            if (p.lo_summed[w]) {
                s_lo += dg * p.s_unit[p.lo_other[w]];
            } else {
                c_lo += dg << (2 * p.lo_other[w]);
                st_lo += dg << (2 * p.lo_rank[w]);
            }
        }
        // each element's tile offset and S offset beyond the thread's own
        // (the g and h digits), and the free-index offsets of S: the same for
        // every thread of the CTA, so they stay out of the per-thread registers
        uint32_t eo[E], so[E];
#pragma unroll
        for (int g = 0; g < G; g++) {
            uint32_t tg = 0;
            if (G > 1)
                for (uint32_t j = 0; j < p.go; j++) tg += (((uint32_t) g >> (2 * j)) & 3u) << (2 * p.g_pos[j]);
#pragma unroll
            for (int h = 0; h < H; h++) {
                uint32_t th = tg, sh = 0;
                if (H > 1)
                    for (uint32_t j = 0; j < p.ho; j++) {
                        const uint32_t dg = ((uint32_t) h >> (2 * j)) & 3u;
                        th += dg << (2 * p.h_pos[j]);
                        sh += dg * p.s_unit[p.h_sw[j]];
                    }
                eo[g * H + h] = th;
                so[g * H + h] = sh;
            }
        }
        // with 16 free indices of S the element loop stays rolled (its body
        // is 64 FMAs already): the offsets then come from shared memory
        // (G == 1 there, so element tid is h digit combination tid)
        if constexpr (NSF >= 16) {
            if (tid < (uint32_t) E) {
                uint32_t th = 0, sh = 0;
                for (uint32_t j = 0; j < p.ho; j++) {
                    const uint32_t dg = (tid >> (2 * j)) & 3u;
                    th += dg << (2 * p.h_pos[j]);
                    sh += dg * p.s_unit[p.h_sw[j]];
                }
                eo_s[tid] = th;
                so_s[tid] = sh;
            }
            asm volatile("bar.sync 1, %0;" ::"r"(kStreamThreads) : "memory");
        }
        // the summed lane bits among wires 0/1 are consecutive: 0-1, 2-3 or 0-3
        const uint32_t b0 = p.lo_summed[0] ? 0u : 2u;
        const uint32_t nb = 2u * (p.lo_summed[0] + p.lo_summed[1]);
        constexpr int LM = M >= 16 ? 4 : M >= 4 ? 2 : 0;   // log2(M)
        float2 acc[G][NSF];
        float2 *flat = &acc[0][0];
        for (uint32_t t = 0; t < n_t; t++) {
            const uint32_t s = t % NS;
            const uint32_t item = blockIdx.x + (t / p.n_chunks) * gridDim.x, chunk = t % p.n_chunks;
            bool got = mbar_wait(smem_u32(&full[s]), (t / NS) & 1u, limit);
            // staged outputs use consumer barriers: all consumers leave together
            if (p.staged) got = consumers_all(got);
            if (!got) {
                ok = false;
                break;
            }
            const float2 *T = tiles + (uint64_t) s * tile_stride + tid;
            // S's share of the chunk's summed digits
            uint32_t s_c = 0;
            for (uint32_t j = 0; j < p.n_chunk_d; j++) s_c += ((chunk >> (2 * j)) & 3u) * p.s_unit[p.chunk_sw[j]];
            uint64_t cbase = 0;
            for (uint32_t j = 0; j < p.n_item_d; j++) cbase += (uint64_t) ((item >> (2 * j)) & 3u) << (2 * p.item_cd[j]);
            // a work item with several passes has one chunk (stream_plan), so
            // the sums never outlive a pass
            for (uint32_t pass = 0; pass < p.n_pass; pass++) {
                uint32_t s_p = s_c + s_lo;
                uint64_t cpass = cbase;
                for (uint32_t j = p.nsfp; j < p.nsf; j++) {
                    const uint32_t dg = (pass >> (2 * (j - p.nsfp))) & 3u;
                    s_p += dg * p.s_unit[p.sf_w[j]];
                    cpass += (uint64_t) dg << (2 * p.sf_cd[j]);
                }
                if (chunk == 0) {
#pragma unroll
                    for (int g = 0; g < G; g++)
#pragma unroll
                        for (int f = 0; f < NSF; f++) acc[g][f] = make_float2(0.f, 0.f);
                }
                const float2 *Sp = S + s_p;
                // a block of S's image holds an element's NSF values side by
                // side, 16-byte aligned (blocks are an even number of elements
                // apart): pairs of them load as one float4
                if constexpr (NSF >= 16) {
                    // G == 1 here: every element adds into acc[0]
#pragma unroll 1
                    for (int i = 0; i < E; i++) {
                        const float2 x = T[eo_s[i]];
                        const float4 *Si = reinterpret_cast<const float4 *>(Sp + so_s[i]);
#pragma unroll
                        for (int f = 0; f < NSF; f += 2) {
                            const float4 s2 = Si[f / 2];
                            cmac(acc[0][f], x, make_float2(s2.x, s2.y));
                            cmac(acc[0][f + 1], x, make_float2(s2.z, s2.w));
                        }
                    }
                } else if constexpr (NSF >= 4) {
#pragma unroll
                    for (int i = 0; i < E; i++) {
                        const float2 x = T[eo[i]];
                        const float4 *Si = reinterpret_cast<const float4 *>(Sp + so[i]);
#pragma unroll
                        for (int f = 0; f < NSF; f += 2) {
                            const float4 s2 = Si[f / 2];
                            cmac(acc[i / H][f], x, make_float2(s2.x, s2.y));
                            cmac(acc[i / H][f + 1], x, make_float2(s2.z, s2.w));
                        }
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < E; i++) cmac(acc[i / H][0], T[eo[i]], Sp[so[i]]);
                }
                if (pass + 1 == p.n_pass) {
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(&empty[s]));   // this warp is done with the stage
                }
                if (chunk + 1 < p.n_chunks) continue;

                // Summed wires among 0/1 (lane bits 0-3): a butterfly
                // reduce-scatter halves the sums a lane keeps at every step, so
                // the lanes sharing a sum each end up with a different part of
                // the outputs; bits beyond log2(M) finish as an all-reduce, the
                // lanes whose summed digits are 0 keeping the sum.
                uint32_t base = 0;
                bool owner = true;
#pragma unroll
                for (int k = 0; k < LM; k++) {
                    if ((uint32_t) k >= nb) break;
                    const uint32_t mask = 1u << (b0 + (uint32_t) k);
                    const bool hi = (tid & mask) != 0;
                    const int half = M >> (k + 1);
#pragma unroll
                    for (int i = 0; i < M / 2; i++) {
                        if (i >= half) break;
                        const float2 a = flat[i], c = flat[i + half];
                        const float2 send = hi ? a : c;
                        float2 keep = hi ? c : a;
                        keep.x += __shfl_xor_sync(0xffffffffu, send.x, mask);
                        keep.y += __shfl_xor_sync(0xffffffffu, send.y, mask);
                        flat[i] = keep;
                    }
                    if (hi) base += (uint32_t) half;
                }
                const uint32_t m_left = (uint32_t) M >> (nb < (uint32_t) LM ? nb : (uint32_t) LM);
                for (uint32_t k = LM; k < nb; k++) {
                    const uint32_t mask = 1u << (b0 + k);
                    flat[0].x += __shfl_xor_sync(0xffffffffu, flat[0].x, mask);
                    flat[0].y += __shfl_xor_sync(0xffffffffu, flat[0].y, mask);
                    owner = owner && (tid & mask) == 0;
                }
                if (!p.staged) {
                    if (owner) {
                        const uint64_t cb = cpass + c_lo;
#pragma unroll
                        for (int j = 0; j < M; j++) {
                            if ((uint32_t) j >= m_left) break;
                            const float2 v = make_float2(scale_pow2(flat[j].x, shift), scale_pow2(flat[j].y, shift));
                            lmax = max(lmax, mag_bits(v));
                            p.C[cb + out_off[base + j]] = v;
                        }
                    }
                    continue;
                }
                // staged: every output of the pass into shared memory in C's
                // digit order (added up there when summed wires 2/3 spread a
                // sum over warps), then stored along C's contiguous runs
                if (owner) {
#pragma unroll
                    for (int j = 0; j < M; j++) {
                        if ((uint32_t) j >= m_left) break;
                        float2 *dst = ostage + st_lo + st_gf[base + j];
                        if (p.klo_mode == 2) {
                            atomicAdd(&dst->x, flat[j].x);
                            atomicAdd(&dst->y, flat[j].y);
                        } else {
                            *dst = flat[j];
                        }
                    }
                }
                asm volatile("bar.sync 1, %0;" ::"r"(kStreamThreads) : "memory");
                const uint32_t run_log2 = 2 * p.out_run, run_mask = (1u << run_log2) - 1u;
                if (p.out_run >= 1) {
                    for (uint32_t u = 2 * tid; u < n_out; u += 2 * kStreamThreads) {
                        uint64_t coff = cpass + (u & run_mask);
                        uint32_t hi = u >> run_log2;
                        for (uint32_t r = p.out_run; r < p.n_dout; r++, hi >>= 2) coff += (uint64_t) (hi & 3u) << (2 * p.dout_cd[r]);
                        const float4 w = *reinterpret_cast<const float4 *>(ostage + u);
                        const float4 v = make_float4(scale_pow2(w.x, shift), scale_pow2(w.y, shift),
                                                     scale_pow2(w.z, shift), scale_pow2(w.w, shift));
                        lmax = max(lmax, max(mag_bits(make_float2(v.x, v.y)), mag_bits(make_float2(v.z, v.w))));
                        *reinterpret_cast<float4 *>(p.C + coff) = v;
                        if (p.klo_mode == 2) *reinterpret_cast<float4 *>(ostage + u) = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                } else {
                    for (uint32_t u = tid; u < n_out; u += kStreamThreads) {
                        uint64_t coff = cpass;
                        uint32_t hi = u;
                        for (uint32_t r = 0; r < p.n_dout; r++, hi >>= 2) coff += (uint64_t) (hi & 3u) << (2 * p.dout_cd[r]);
                        const float2 v = make_float2(scale_pow2(ostage[u].x, shift), scale_pow2(ostage[u].y, shift));
                        lmax = max(lmax, mag_bits(v));
                        p.C[coff] = v;
                        if (p.klo_mode == 2) ostage[u] = make_float2(0.f, 0.f);
                    }
                }
                asm volatile("bar.sync 1, %0;" ::"r"(kStreamThreads) : "memory");   // staging free again
            }
        }
    }
    // every wait above is bounded, so every thread gets here
    ok = __syncthreads_and(ok) != 0;
    if (!ok && tid == 0) {
        // the last copy issued into each stage lands before the CTA leaves
        const uint32_t issued = *issued_slot;
        for (uint32_t s = 0; s < (uint32_t) NS; s++)
            if (issued > s) {
                const uint32_t last = s + ((issued - 1 - s) / NS) * NS;
                if (!(last == 0 && skip_first)) mbar_wait(smem_u32(&full[s]), (last / NS) & 1u);
            }
        atomicExch(p.error_flag, 1);
    }
    scale_note(p.sc, lmax, shift, blockIdx.x == 0);
}

using StreamFn = void (*)(const StreamStep);

// the instantiation of a plan's shape class (G x NSF <= 16, G x H <= 16)
StreamFn stream_fn(uint32_t nsf, uint32_t go, uint32_t ho) {
    const uint32_t key = nsf * 9 + go * 3 + ho;
#define QT_STREAM_CASE(NS, GO, HO) \
    case (NS) * 9 + (GO) * 3 + (HO): return stream_kernel<1 << (2 * (NS)), 1 << (2 * (GO)), 1 << (2 * (HO))>;
    switch (key) {
        QT_STREAM_CASE(0, 0, 0) QT_STREAM_CASE(0, 0, 1) QT_STREAM_CASE(0, 0, 2)
        QT_STREAM_CASE(0, 1, 0) QT_STREAM_CASE(0, 1, 1) QT_STREAM_CASE(0, 2, 0)
        QT_STREAM_CASE(1, 0, 0) QT_STREAM_CASE(1, 0, 1) QT_STREAM_CASE(1, 0, 2)
        QT_STREAM_CASE(1, 1, 0) QT_STREAM_CASE(1, 1, 1)
        QT_STREAM_CASE(2, 0, 0) QT_STREAM_CASE(2, 0, 1) QT_STREAM_CASE(2, 0, 2)
    default: return nullptr;
    }
#undef QT_STREAM_CASE
}

std::mutex g_attr_lock;
bool g_attr_done[64];

cudaError_t stream_attributes() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(g_attr_lock);
    if (dev >= 0 && dev < 64 && g_attr_done[dev]) return cudaSuccess;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    for (uint32_t nsf = 0; nsf <= 2; nsf++)
        for (uint32_t go = 0; go <= 2; go++)
            for (uint32_t ho = 0; ho <= 2; ho++) {
                const StreamFn fn = stream_fn(nsf, go, ho);
                if (fn && e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            }
    if (e == cudaSuccess && dev >= 0 && dev < 64) g_attr_done[dev] = true;
    return e;
}

}  // namespace

cudaError_t stream_set_fault(int mode, uint32_t polls) {
    const uint32_t m = (uint32_t) mode;
    cudaError_t e = cudaMemcpyToSymbol(g_stream_fault_mode, &m, sizeof m);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_stream_fault_polls, &polls, sizeof polls);
    return e;
}

bool stream_plan(const StepDesc &d, StreamStep &p) {
    std::memset(&p, 0, sizeof p);
    const bool l_is_b = d.rB > d.rA;
    const int rL = l_is_b ? d.rB : d.rA, rS = l_is_b ? d.rA : d.rB;
    if (rS > kStreamMaxSmallRank || rL < 8 || d.nSum > kStreamMaxSmallRank) return false;
    const uint8_t *cL = l_is_b ? d.cB : d.cA;
    const uint8_t *cS = l_is_b ? d.cA : d.cB;
    const uint8_t *posL = l_is_b ? d.posBs : d.posAs;
    const uint8_t *posS = l_is_b ? d.posAs : d.posBs;
    int pair_s[kMaxWires], cdig[kMaxWires];
    bool summed[kMaxWires] = {false};
    for (int w = 0; w < kMaxWires; w++) pair_s[w] = cdig[w] = -1;
    for (int i = 0; i < d.nSum; i++) {
        summed[posL[i]] = true;
        pair_s[posL[i]] = posS[i];
    }
    int nsf = 0;
    for (int i = 0; i < d.nFree; i++) {
        if (cL[i] != kNoWire) {
            cdig[cL[i]] = i;
        } else {
            p.sf_cd[nsf] = (uint8_t) i;
            p.sf_w[nsf++] = cS[i];
        }
    }
    if (nsf > 3) return false;   // at most 64 free indices of S: 16 per pass
    p.l_is_b = l_is_b;
    p.nsf = (uint32_t) nsf;
    p.nsfp = (uint32_t) std::min(nsf, 2);
    p.n_pass = 1u << (2 * (nsf - (int) p.nsfp));
    p.s_elems = 1u << (2 * rS);
    {
        const uint32_t nblk = 1u << (2 * p.nsfp);
        const uint32_t bstride = nblk == 1 ? 1u : nblk + 2u;
        bool in_blk[kStreamMaxSmallRank] = {false};
        for (uint32_t j = 0; j < p.nsfp; j++) {
            in_blk[p.sf_w[j]] = true;
            p.s_unit[p.sf_w[j]] = 1u << (2 * j);
        }
        uint32_t rank = 0;
        for (int w = 0; w < rS; w++)
            if (!in_blk[w]) p.s_unit[w] = bstride << (2 * rank++);
        p.s_store = bstride << (2 * rank);
    }
    // wires 0-3: the thread's own digits
    int klo = 0;
    for (int w = 0; w < 4; w++) {
        p.lo_summed[w] = summed[w] ? 1 : 0;
        p.lo_other[w] = (uint8_t) (summed[w] ? pair_s[w] : cdig[w]);
        klo += summed[w];
    }
    p.n_klo = (uint32_t) klo;
    p.klo_mode = klo == 0 ? 0u : (summed[2] || summed[3]) ? 2u : 1u;
    // a thread's C offset over its free digits among wires 0-3 is 32-bit
    for (int w = 0; w < 4; w++)
        if (!summed[w] && cdig[w] >= 16) return false;
    int outer[kMaxWires], hi[kMaxWires], n_outer = 0, n_hi = 0;
    for (int w = 4; w < rL; w++) {
        if (summed[w]) hi[n_hi++] = w;
        else outer[n_outer++] = w;
    }
    // loop digits of a tile: up to 16 elements per thread and 16 sums per thread
    const int ho = std::min(n_hi, 2);
    int go = std::min(n_outer, 2 - ho);
    while (go > 0 && (1 << (2 * (go + (int) p.nsfp))) > (int) kStreamMaxStage) go--;
    // 16 sums over 16 elements (free and summed looped digits together) need
    // more registers than two CTAs per SM leave: loop the free digit over work
    // items instead
    if (n_outer - go > 15 || n_hi - ho > 15) return false;
    if (p.n_pass > 1 && n_hi > ho) return false;   // several passes keep no sums across chunks
    p.go = (uint32_t) go;
    p.ho = (uint32_t) ho;
    p.n_items = 1u << (2 * (n_outer - go));
    p.n_chunks = 1u << (2 * (n_hi - ho));
    p.n_item_d = (uint32_t) (n_outer - go);
    p.n_chunk_d = (uint32_t) (n_hi - ho);
    for (int j = go; j < n_outer; j++) {
        p.item_lw[j - go] = (uint8_t) outer[j];
        p.item_cd[j - go] = (uint8_t) cdig[outer[j]];
    }
    for (int j = ho; j < n_hi; j++) {
        p.chunk_lw[j - ho] = (uint8_t) hi[j];
        p.chunk_sw[j - ho] = (uint8_t) pair_s[hi[j]];
    }
    // in-tile wires in ascending order give the tile's local digits
    bool in_tile[kMaxWires] = {false};
    for (int w = 0; w < 4; w++) in_tile[w] = true;
    for (int j = 0; j < go; j++) in_tile[outer[j]] = true;
    for (int j = 0; j < ho; j++) in_tile[hi[j]] = true;
    int tpos[kMaxWires], nt = 0;
    for (int w = 0; w < rL; w++) tpos[w] = in_tile[w] ? nt++ : -1;
    for (int j = 0; j < go; j++) {
        p.g_pos[j] = (uint8_t) tpos[outer[j]];
        p.g_cd[j] = (uint8_t) cdig[outer[j]];
    }
    for (int j = 0; j < ho; j++) {
        p.h_pos[j] = (uint8_t) tpos[hi[j]];
        p.h_sw[j] = (uint8_t) pair_s[hi[j]];
    }
    // bulk copies: runs along the lowest in-tile wires that follow each other from wire 0
    int prefix = 0;
    while (prefix < rL && in_tile[prefix]) prefix++;
    p.run_elems = 1u << (2 * prefix);
    p.n_runs = 1u << (2 * (nt - prefix));
    int nr = 0;
    for (int w = prefix; w < rL; w++)
        if (in_tile[w]) p.run_lw[nr++] = (uint8_t) w;
    p.n_run_d = (uint32_t) nr;
    // the outputs of a pass: C digits of L's free wires 0-3, of the g digits
    // and of the in-pass free wires of S, ascending
    int nd = 0;
    for (int i = 0; i < d.nFree; i++) {
        if (cL[i] != kNoWire) {
            const int w = cL[i];
            if (w < 4) {
                p.lo_rank[w] = (uint8_t) nd;
            } else {
                int j = 0;
                while (j < go && outer[j] != w) j++;
                if (j == go) continue;   // a work-item digit
                p.g_rank[j] = (uint8_t) nd;
            }
        } else {
            int j = 0;
            while (j < nsf && p.sf_cd[j] != i) j++;
            if (j >= (int) p.nsfp) continue;   // a pass digit
            p.sf_rank[j] = (uint8_t) nd;
        }
        p.dout_cd[nd++] = (uint8_t) i;
    }
    p.n_dout = (uint32_t) nd;
    uint32_t run = 0;
    while ((int) run < nd && p.dout_cd[run] == run) run++;
    p.out_run = run;
    // Sums that summed wires 2/3 spread over warps meet in shared memory;
    // every other output is stored by the lane that owns it (staging those
    // too, for better-coalesced stores, measured slower: two consumer barriers
    // per tile cost more than the partly coalesced stores save).
    p.staged = p.klo_mode == 2 ? 1u : 0u;
    if (p.staged && (1u << (2 * nd)) > kStreamMaxOut) return false;
    uint32_t off[5];
    stream_layout(p, off);
    p.smem_bytes = off[4];
    return p.smem_bytes <= 200u * 1024u && stream_fn((uint32_t) p.nsfp, p.go, p.ho) != nullptr;
}

cudaError_t launch_stream(StreamStep &p, const StepDesc &d, const float2 *A, const float2 *B, float2 *C,
                          const StepScaleRef &sc, int *error_flag, cudaStream_t stream) {
    (void) d;
    p.L = p.l_is_b ? B : A;
    p.S = p.l_is_b ? A : B;
    p.C = C;
    p.sc = sc;
    p.error_flag = error_flag;
    cudaError_t e = stream_attributes();
    if (e != cudaSuccess) return e;
    const StreamFn fn = stream_fn(p.nsfp, p.go, p.ho);
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kStreamBlock, p.smem_bytes);
    if (e != cudaSuccess) return e;
    const int sms = persistent_sms();
    const uint32_t grid = std::min<uint32_t>(p.n_items, (uint32_t) (sms * std::max(per_sm, 1)));
    fn<<<grid, kStreamBlock, p.smem_bytes, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace qtg
