// Tiled index permutation of base-4 tensors (permute.cu), and the full
// contraction of two tensors whose wires are in different orders built on the
// same tiling.
//
// A tensor of rank r holds 4^r elements, digit i of the flat index being wire
// i (the reference's index map, src/Network.h:912-916: offset = sum of
// digit_i * 4^i).  Permuting it writes Y with digit i of Y's index equal to
// digit perm[i] of X's.  Read straight, one side of such a copy is strided;
// here a CTA moves one tile at a time through shared memory: the tile spans
// the lowest `a` digits of X and the digits that become Y's lowest `b` (at
// most 6 digits, 4096 elements), so the tile is read along X's contiguous
// runs and written along Y's.  The rest of the digits number the tiles.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "scale.cuh"

namespace qtg {

constexpr int kPermMaxRank = 24;
constexpr int kPermMaxTileDigits = 6;
constexpr int kPermLowDigits = 3;      // contiguous digits each side of a tile copies in a row (64 elements)
constexpr int kPermThreads = 256;

struct PermutePlan {
    uint32_t rank = 0;
    uint32_t elem_bytes = 8;           // 8 (complex64) or 16 (complex128)
    uint32_t nu = 0;                   // digits of a tile
    uint32_t a = 0, b = 0;             // the tile's low input / low output digits
    uint32_t n_rest = 0;               // digits numbering the tiles
    uint64_t n_tiles = 1;
    uint8_t u_in[kPermMaxTileDigits];  // tile digit j (ascending input order) -> input digit
    uint8_t r_in[kPermMaxRank];        // tile-number digit j -> input digit
    uint8_t r_out[kPermMaxRank];       //                     -> output digit
    // offsets of the tile's high digits, and the tile element of each output-order index
    uint32_t in_hi[64];                // input offset of e >> 2a
    uint32_t out_hi[64];               // output offset of f >> 2b
    uint16_t e_lo[64];                 // tile element of (f & (4^b - 1))
    uint16_t e_hi[64];                 //              and of f >> 2b
};

// perm[i]: the input digit that becomes output digit i (a permutation of
// 0..rank-1).  False when perm is not one or rank is out of range.
bool permute_plan(int rank, const int32_t *perm, uint32_t elem_bytes, PermutePlan &p);
// in and out 16-byte aligned (cudaErrorInvalidValue otherwise, nothing launched)
cudaError_t launch_permute(const PermutePlan &p, const void *in, void *out, cudaStream_t stream);

// Full contraction C = sum_k A[k] B[pi(k)] of two complex64 tensors of the
// same rank: digit j of A's index pairs with digit perm[j] of B's.  Tiles of A
// and of B (each read along its own contiguous runs) meet in shared memory;
// every CTA keeps compensated (Dot2) partial sums, merged by reduce_final_f32.
// partials: dot_grid(p) float4 values of scratch.  A and B 16-byte aligned
// (cudaErrorInvalidValue otherwise, nothing launched).
uint32_t dot_grid(const PermutePlan &p);
cudaError_t launch_permuted_dot(const PermutePlan &p, const float2 *A, const float2 *B, float2 *C, void *partials,
                                const StepScaleRef &sc, cudaStream_t stream);

}  // namespace qtg
