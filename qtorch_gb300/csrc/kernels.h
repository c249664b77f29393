// Launchers of the device kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include "engine.cuh"
#include "scale.cuh"

namespace qtg {

// One pairwise contraction over the whole GPU.  f64: complex128, reference
// rounding; otherwise complex64 with FP32 FMA.
// sc: the mixed form's per-tensor scaling (scale.cuh); empty: none
cudaError_t launch_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64, cudaStream_t stream,
                        const StepScaleRef &sc = StepScaleRef{});
// a small step that run_contraction would give to a pair or tiled kernel: it
// may join a PairBatch of its dependency level
bool pair_batchable(const StepDesc &d, bool f64);
// fills n_out, K and block_begin of every job and launches them together
cudaError_t launch_pair_batch(PairBatch &pb, bool f64, cudaStream_t stream);

// Wide steps (C = A~ B~ with both gathered sides >= 16 and >= 1024 outputs,
// A's free wires first, ranks <= 15) as tiled products over the whole GPU;
// each output sums over k in increasing order (FP64: the reference's rounding).
bool tiled_shaped(const StepDesc &d);
cudaError_t launch_tiled_pair(const StepDesc &d, const void *A, const void *B, void *C, bool f64,
                              cudaStream_t stream, const StepScaleRef &sc = StepScaleRef{});

// Steps with at most kReduceMaxOut outputs and a sum of at least kReduceMinK
// terms (the final expectation values of large networks).
constexpr uint64_t kReduceMaxOut = 16;
constexpr uint64_t kReduceMinK = 1ull << 16;
inline bool reduce_shaped(const StepDesc &d) {
    return (1ull << (2 * d.nFree)) <= kReduceMaxOut && (1ull << (2 * d.nSum)) >= kReduceMinK;
}
// complex64: the sum split over the whole GPU, compensated (Dot2) partial sums
// merged in a second kernel; scratch holds reduce_scratch_bytes(d) bytes
size_t reduce_scratch_bytes(const StepDesc &d);
cudaError_t launch_reduce_f32(const StepDesc &d, const float2 *A, const float2 *B, float2 *C, void *scratch,
                              cudaStream_t stream, const StepScaleRef &sc = StepScaleRef{});
// merges n_parts compensated partial sums per output (float4: p_re, s_re,
// p_im, s_im; output-major) into n_out complex64 outputs
cudaError_t launch_reduce_final_f32(const float4 *partials, uint32_t n_parts, uint32_t n_out, float2 *C,
                                    const StepScaleRef &sc, cudaStream_t stream);
// complex128 with the reference's rounding: every thread of a CTA forms the
// products of a chunk of k, one thread adds them in the reference's order
cudaError_t launch_reduce_exact(const StepDesc &d, const double2 *A, const double2 *B, double2 *C,
                                cudaStream_t stream);

// Grouped interpreter over plan instances.  The workspace of a CTA is either
// its shared memory (ws_in_smem; ws_stride bytes after the header) or
// ws_base + blockIdx.x * ws_stride in global memory; with stage_bytes > 0 each
// instance's plan block and leaf image are copied into shared memory first.
// variant: the register budget, one of kPlanVariants (CTAs per SM it is built
// for; 1 is the wide form, 512 threads a CTA)
constexpr int kPlanVariants[] = {1, 2, 3, 4, 5};
constexpr int kPlanDefaultVariant = 2;
cudaError_t launch_plan(const PlanLaunch &lp, bool mixed, int grid, cudaStream_t stream,
                        int variant = kPlanDefaultVariant);
// dynamic shared memory of one interpreter CTA for these parameters
size_t plan_smem_bytes(const PlanLaunch &lp);
// CTAs of a grouped launch with this much dynamic shared memory: all SMs times
// the CTAs of the variant that fit one SM, at most per_sm_cap when positive
int plan_max_grid(size_t smem_bytes, int per_sm_cap = 0, int variant = kPlanDefaultVariant);
int plan_num_sms();
// test hook of the interpreter's staging waits (qt_debug_staging_fault)
cudaError_t plan_set_staging_fault(int mode, uint32_t polls);
// SMs the persistent whole-GPU kernels (streaming, tiled, pair, reduction
// and permutation kernels) size their grids by
int persistent_sms();
// largest dynamic shared memory an interpreter CTA may have on this device
size_t plan_smem_limit();
// The resident engine (one CTA per instance, 128-register budget; variant 1:
// the wide 512-thread form, otherwise 256 threads); returns once launched.
// resident_capacity: how many CTAs of that shared-memory size are resident at once.
cudaError_t launch_resident(const ResidentLaunch &rl, cudaStream_t stream, int variant);
int resident_capacity(size_t smem_bytes, int variant);

}  // namespace qtg
