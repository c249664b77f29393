// Launchers of the device kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include "engine.cuh"

namespace qtg {

// One pairwise contraction over the whole GPU.  f64: complex128, reference
// rounding; otherwise complex64 with FP32 FMA.
cudaError_t launch_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64, cudaStream_t stream);

// Grouped interpreter over plan instances; workspace and exponent buffers are
// per CTA (ws_base + blockIdx.x * ws_stride).
cudaError_t launch_plan(const InstanceDesc *instances, int n_instances, bool mixed, int grid,
                        char *ws_base, uint64_t ws_stride, int32_t *exps_base, uint64_t exps_stride,
                        cudaStream_t stream);
size_t plan_smem_bytes();
int plan_max_grid();

}  // namespace qtg
