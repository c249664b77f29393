// Tiled index permutation and the permuted full contraction (permute.h).
//
// A tile holds 4^nu elements (nu <= 6 digits: X's lowest `a` digits and the X
// digits that become Y's lowest `b`, a = b = 3 where the rank allows).  Its
// element e numbers the tile digits in ascending X order, so e's low 2a bits
// are X's contiguous run; f numbers them in ascending Y order, so f's low 2b
// bits are Y's contiguous run.  A CTA reads the tile along e (coalesced),
// parks element e in shared memory at swz(e), and writes along f (coalesced)
// from swz(e(f)).  swz XORs e's low 4 bits with a hash of the higher ones, so
// the gathers along any single tile digit (stride 4^j) hit 16 different
// 8-byte slots in every half warp.  CTAs are persistent over the tiles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "dot2.cuh"
#include "kernels.h"
#include "permute.h"

namespace qtg {

namespace {

__device__ __forceinline__ uint32_t swz(uint32_t e) { return e ^ (((e >> 4) ^ (e >> 8)) & 15u); }

// base offsets of tile t in X and in Y
__device__ __forceinline__ void tile_base(const PermutePlan &p, uint64_t t, uint64_t &bi, uint64_t &bo) {
    bi = 0;
    bo = 0;
    for (uint32_t j = 0; j < p.n_rest; j++) {
        const uint64_t dg = (t >> (2 * j)) & 3ull;
        bi += dg << (2 * p.r_in[j]);
        bo += dg << (2 * p.r_out[j]);
    }
}

// the plan's index tables, copied to shared memory once per CTA (indexed by
// lane-varying values they would serialise in the parameter bank)
struct PermTables {
    uint32_t in_hi[64], out_hi[64], e_lo[64], e_hi[64];
};

__device__ __forceinline__ void load_tables(const PermutePlan &p, PermTables &t) {
    for (uint32_t i = threadIdx.x; i < 64; i += blockDim.x) {
        t.in_hi[i] = p.in_hi[i];
        t.out_hi[i] = p.out_hi[i];
        t.e_lo[i] = p.e_lo[i];
        t.e_hi[i] = p.e_hi[i];
    }
    __syncthreads();
}

// Loads the tile of X at base bi into shared memory (element e at swz(e)).
// 8-byte elements move in pairs: e and e + 1 are adjacent in X (a >= 1), so
// one 16-byte load brings both.
template <typename T>
__device__ __forceinline__ void load_tile(const PermutePlan &p, const PermTables &tb, const T *__restrict__ in,
                                          uint64_t bi, T *tile) {
    const uint32_t n = 1u << (2 * p.nu), ma = (1u << (2 * p.a)) - 1u;
    if (sizeof(T) == 8 && n >= 2) {
#pragma unroll 4
        for (uint32_t e = 2 * threadIdx.x; e < n; e += 2 * kPermThreads) {
            const uint4 v = *reinterpret_cast<const uint4 *>(in + bi + (e & ma) + tb.in_hi[e >> (2 * p.a)]);
            reinterpret_cast<uint2 *>(tile)[swz(e)] = make_uint2(v.x, v.y);
            reinterpret_cast<uint2 *>(tile)[swz(e + 1)] = make_uint2(v.z, v.w);
        }
    } else {
#pragma unroll 4
        for (uint32_t e = threadIdx.x; e < n; e += kPermThreads) tile[swz(e)] = in[bi + (e & ma) + tb.in_hi[e >> (2 * p.a)]];
    }
}

template <typename T>
__global__ void __launch_bounds__(kPermThreads) permute_kernel(const __grid_constant__ PermutePlan p,
                                                               const T *__restrict__ in, T *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ PermTables tb;
    T *tile = reinterpret_cast<T *>(smem_raw);
    load_tables(p, tb);
    const uint32_t n = 1u << (2 * p.nu);
    const uint32_t mb = (1u << (2 * p.b)) - 1u;
    for (uint64_t t = blockIdx.x; t < p.n_tiles; t += gridDim.x) {
        uint64_t bi, bo;
        tile_base(p, t, bi, bo);
        load_tile(p, tb, in, bi, tile);
        __syncthreads();
        if (sizeof(T) == 8 && n >= 2) {
            // f and f + 1 are adjacent in Y (b >= 1): one 16-byte store
#pragma unroll 4
            for (uint32_t f = 2 * threadIdx.x; f < n; f += 2 * kPermThreads) {
                const uint32_t hi = tb.e_hi[f >> (2 * p.b)];
                const uint2 v0 = reinterpret_cast<const uint2 *>(tile)[swz(tb.e_lo[f & mb] + hi)];
                const uint2 v1 = reinterpret_cast<const uint2 *>(tile)[swz(tb.e_lo[(f & mb) + 1] + hi)];
                *reinterpret_cast<uint4 *>(out + bo + (f & mb) + tb.out_hi[f >> (2 * p.b)]) =
                    make_uint4(v0.x, v0.y, v1.x, v1.y);
            }
        } else {
#pragma unroll 4
            for (uint32_t f = threadIdx.x; f < n; f += kPermThreads) {
                const uint32_t e = tb.e_lo[f & mb] + tb.e_hi[f >> (2 * p.b)];
                out[bo + (f & mb) + tb.out_hi[f >> (2 * p.b)]] = tile[swz(e)];
            }
        }
        __syncthreads();   // the tile's buffer is refilled next
    }
}

// sum_k A[k] B[pi(k)]: A is the plan's input side, B its output side
__global__ void __launch_bounds__(kPermThreads) permuted_dot_kernel(const __grid_constant__ PermutePlan p,
                                                                    const float2 *__restrict__ A,
                                                                    const float2 *__restrict__ B,
                                                                    float4 *__restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ PermTables tb;
    __shared__ float4 s_part[kPermThreads / 32];
    load_tables(p, tb);
    const uint32_t n = 1u << (2 * p.nu);
    float2 *ta = reinterpret_cast<float2 *>(smem_raw);
    float2 *tbuf = ta + n;
    const uint32_t mb = (1u << (2 * p.b)) - 1u;
    float pre = 0.f, sre = 0.f, pim = 0.f, sim = 0.f;
    for (uint64_t t = blockIdx.x; t < p.n_tiles; t += gridDim.x) {
        uint64_t bi, bo;
        tile_base(p, t, bi, bo);
        load_tile(p, tb, A, bi, ta);
        if (n >= 2) {
#pragma unroll 4
            for (uint32_t f = 2 * threadIdx.x; f < n; f += 2 * kPermThreads) {
                const float4 v = *reinterpret_cast<const float4 *>(B + bo + (f & mb) + tb.out_hi[f >> (2 * p.b)]);
                const uint32_t hi = tb.e_hi[f >> (2 * p.b)];
                tbuf[swz(tb.e_lo[f & mb] + hi)] = make_float2(v.x, v.y);
                tbuf[swz(tb.e_lo[(f & mb) + 1] + hi)] = make_float2(v.z, v.w);
            }
        } else if (threadIdx.x == 0) {
            tbuf[0] = B[bo];
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < n; e += kPermThreads) cmac_dot2(pre, sre, pim, sim, ta[e], tbuf[e]);
        __syncthreads();
    }
    for (int off = 16; off >= 1; off >>= 1) {
        const float a = __shfl_xor_sync(0xffffffffu, pre, off), b = __shfl_xor_sync(0xffffffffu, sre, off);
        const float c = __shfl_xor_sync(0xffffffffu, pim, off), d = __shfl_xor_sync(0xffffffffu, sim, off);
        dot2_merge(pre, sre, a, b);
        dot2_merge(pim, sim, c, d);
    }
    if ((threadIdx.x & 31u) == 0) s_part[threadIdx.x >> 5] = make_float4(pre, sre, pim, sim);
    __syncthreads();
    if (threadIdx.x == 0) {
        float4 t = s_part[0];
        for (int w = 1; w < kPermThreads / 32; w++) {
            dot2_merge(t.x, t.y, s_part[w].x, s_part[w].y);
            dot2_merge(t.z, t.w, s_part[w].z, s_part[w].w);
        }
        partials[blockIdx.x] = t;
    }
}

template <typename K>
uint32_t persistent_grid(K kernel, size_t smem, uint64_t n_tiles) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPermThreads, smem) != cudaSuccess) per_sm = 1;
    const uint64_t cap = (uint64_t) persistent_sms() * (uint64_t) std::max(per_sm, 1);
    return (uint32_t) std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, cap));
}

template <typename K>
cudaError_t allow_smem(K kernel, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
}

}  // namespace

cudaError_t launch_permute(const PermutePlan &p, const void *in, void *out, cudaStream_t stream) {
    // element pairs move as 16-byte accesses
    if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) return cudaErrorInvalidValue;
    const size_t smem = (size_t) p.elem_bytes << (2 * p.nu);
    if (p.elem_bytes == 8) {
        cudaError_t e = allow_smem(permute_kernel<uint2>, smem);
        if (e != cudaSuccess) return e;
        const uint32_t grid = persistent_grid(permute_kernel<uint2>, smem, p.n_tiles);
        permute_kernel<uint2><<<grid, kPermThreads, smem, stream>>>(p, static_cast<const uint2 *>(in),
                                                                    static_cast<uint2 *>(out));
    } else {
        cudaError_t e = allow_smem(permute_kernel<uint4>, smem);
        if (e != cudaSuccess) return e;
        const uint32_t grid = persistent_grid(permute_kernel<uint4>, smem, p.n_tiles);
        permute_kernel<uint4><<<grid, kPermThreads, smem, stream>>>(p, static_cast<const uint4 *>(in),
                                                                    static_cast<uint4 *>(out));
    }
    return cudaGetLastError();
}

uint32_t dot_grid(const PermutePlan &p) {
    const size_t smem = (size_t) 2 * 8 << (2 * p.nu);
    if (allow_smem(permuted_dot_kernel, smem) != cudaSuccess) return 1;
    return persistent_grid(permuted_dot_kernel, smem, p.n_tiles);
}

cudaError_t launch_permuted_dot(const PermutePlan &p, const float2 *A, const float2 *B, float2 *C, void *partials,
                                const StepScaleRef &sc, cudaStream_t stream) {
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15u) return cudaErrorInvalidValue;
    const size_t smem = (size_t) 2 * 8 << (2 * p.nu);
    cudaError_t e = allow_smem(permuted_dot_kernel, smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid = dot_grid(p);
    permuted_dot_kernel<<<grid, kPermThreads, smem, stream>>>(p, A, B, static_cast<float4 *>(partials));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_reduce_final_f32(static_cast<const float4 *>(partials), grid, 1, C, sc, stream);
}

}  // namespace qtg
