// Tensor-core path (gemm_tc.cu) for GEMM-shaped contraction steps in complex64.
#pragma once
#include <cuda_runtime.h>

#include "engine.cuh"

namespace qtg {

struct GemmSizes {
    bool x_pairs;                   // X's rows come in (Re, Im) pairs: B has more free indices than A
    uint64_t M, N2, K;              // rows of X, rows of Y (the paired one: 2 x complex rows), summed range
    uint64_t k_tiles, m_tiles, n_tiles;
    uint64_t x_floats, y_floats;    // one plane of packed X / Y
};

// A step qualifies when A's free wires are C's low digits (as ContractNodes
// orders them) and the GEMM is large enough to fill 128x128 tiles.
bool gemm_eligible(const StepDesc &d);
GemmSizes gemm_sizes(const StepDesc &d);
inline uint64_t gemm_scratch_floats(const StepDesc &d) {
    const GemmSizes s = gemm_sizes(d);
    return 2 * (s.x_floats + s.y_floats);
}
size_t gemm_smem_bytes();
// test hook of the pipeline's bounded waits (qt_debug_gemm_fault)
cudaError_t gemm_set_fault(int mode, uint32_t polls);
// pack X and Y (hi/lo TF32 planes) into scratch, then the tcgen05 GEMM writes C.
// error_flag (device int, zero on entry) becomes 1 if a pipeline wait timed out.
// sc: the mixed form's per-tensor scaling (scale.cuh), applied in the epilogue
cudaError_t launch_gemm_step(const StepDesc &d, const float2 *A, const float2 *B, float2 *C, float *scratch,
                             int *error_flag, cudaStream_t stream, const StepScaleRef &sc = StepScaleRef{});

}  // namespace qtg
