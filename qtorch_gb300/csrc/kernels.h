// Launchers of the device kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include "engine.cuh"

namespace qtg {

// One pairwise contraction over the whole GPU.  f64: complex128, reference
// rounding; otherwise complex64 with FP32 FMA.
cudaError_t launch_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64, cudaStream_t stream);

// Grouped interpreter over plan instances.  The workspace of a CTA is either
// its shared memory (ws_in_smem; ws_stride bytes after the header) or
// ws_base + blockIdx.x * ws_stride in global memory; with stage_bytes > 0 each
// instance's plan block and leaf image are copied into shared memory first.
cudaError_t launch_plan(const PlanLaunch &lp, bool mixed, int grid, cudaStream_t stream);
// dynamic shared memory of one interpreter CTA for these parameters
size_t plan_smem_bytes(const PlanLaunch &lp);
// resident CTAs of the interpreter for a given dynamic shared memory size
int plan_max_grid(size_t smem_bytes);

}  // namespace qtg
