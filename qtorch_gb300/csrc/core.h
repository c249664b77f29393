// Internal structures of the C ABI: context, caching device allocator, tensors.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qtorch_gb300.h"
#include "engine.cuh"

struct qt_ctx {
    // references: the owner's (dropped by qt_ctx_destroy) plus one per plan,
    // batch, network and server made on it; the context is torn down when the
    // last one goes, so objects freed after qt_ctx_destroy stay valid
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::recursive_mutex lock;
    std::string last_error;
    std::mutex err_lock;
    // caching allocator: size class (bytes, power of two >= 256) -> free blocks;
    // its state has a lock of its own (held briefly), so that an allocation
    // that runs out of device memory can empty other contexts' caches while
    // their owners run
    std::mutex alloc_lock;
    // smallest size class of both caching allocators: a context that serves
    // many short batches of varying size (a server's light lane) rounds its
    // blocks up so that every batch after the first finds them cached -- a
    // cudaMalloc or cudaMallocHost can wait behind other threads' large ones
    size_t min_class = 256;
    std::map<size_t, std::vector<void *>> free_blocks;
    std::map<void *, size_t> block_size;
    uint64_t bytes_in_use = 0;
    uint64_t bytes_cached = 0;
    uint64_t memory_budget = 0;          // 0 = unlimited
    // stream-ordered pool (null: the caching allocator above): blocks are
    // taken with cudaMallocFromPoolAsync and returned with cudaFreeAsync, both
    // on this context's stream (a server's heavy lanes; device_pool())
    cudaMemPool_t pool = nullptr;
    std::atomic<uint64_t> launches{0};
    std::atomic<uint64_t> device_allocs{0};   // cudaMalloc calls made by the caching allocator
    std::atomic<uint64_t> tc_steps{0};        // contraction steps run on the tcgen05 GEMM
    std::atomic<uint64_t> stream_steps{0};    // contraction steps run by the streaming kernel
    bool has_deadline = false;
    std::chrono::steady_clock::time_point deadline;
    // pinned staging buffer for small host<->device transfers
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    // caching allocator of pinned host memory (batch staging buffers): a
    // server forms a batch per wave, and cudaMallocHost costs far more than a wave
    std::map<size_t, std::vector<void *>> free_pinned;
    std::map<void *, size_t> pinned_size;
};

struct qt_tensor {
    void *ptr = nullptr;
    int rank = 0;
    qt_dtype dtype = QT_C128;
    size_t bytes = 0;
};

namespace qtg {

void ctx_retain(qt_ctx *ctx);
// a context with its own stream at the device's highest or lowest priority
qt_status ctx_create_prioritised(int device, bool high_priority, qt_ctx **out);
void ctx_release(qt_ctx *ctx);
qt_status set_error(qt_ctx *ctx, qt_status s, const std::string &msg);
qt_status cuda_error(qt_ctx *ctx, cudaError_t e, const char *what);
// allocate from the context cache (bytes rounded up to a size class)
qt_status dev_alloc(qt_ctx *ctx, size_t bytes, void **out);
void dev_free(qt_ctx *ctx, void *p);
// The stream-ordered memory pool of a device, created on first use and kept
// for the life of the process (see core.cpp).
qt_status device_pool(int device, cudaMemPool_t *out);
qt_status ensure_pinned(qt_ctx *ctx, size_t bytes);
// pinned host memory from the context cache (bytes rounded up to a size class)
qt_status host_alloc(qt_ctx *ctx, size_t bytes, void **out);
void host_free(qt_ctx *ctx, void *p);
bool deadline_passed(qt_ctx *ctx);
inline size_t elem_bytes(qt_dtype d) { return d == QT_C128 ? 16 : 8; }

// One contraction step over the whole GPU: complex128 with the reference's
// rounding, or complex64 -- through the tcgen05 tensor-core GEMM when the step
// is GEMM-shaped and large (gemm_tc.cu), the tiled kernel when both sides are
// wide, the streaming kernel when one operand is small (stream.cu), else the
// SIMT pair kernel.
// gemm_flag: a zeroed device int the caller checks after its last step (the
// tensor-core pipeline's timeout flag); null: checked here, with a stream
// synchronisation after every tensor-core step
// sc: the mixed form's per-tensor scale words of the step (scale.cuh); empty: no scaling
qt_status run_contraction(qt_ctx *ctx, const StepDesc &d, const void *A, const void *B, void *C, bool f64,
                          int *gemm_flag = nullptr, const StepScaleRef &sc = StepScaleRef{});
// whether complex64 steps may use the tensor cores (QT_DISABLE_TCGEN05=1 turns it off)
bool tensor_cores_enabled();
// whether complex64 steps with a small operand may use the streaming kernel
// (QT_DISABLE_STREAM=1 turns it off)
bool stream_enabled();

// Fill a StepDesc from the reference's index lists (toNotSumOn, toSumOn).
qt_status make_step(int rank_a, int rank_b, int n_free, const uint8_t *free_from_a, const int32_t *free_idx,
                    int n_sum, const int32_t *sum_a, const int32_t *sum_b, StepDesc *d);

}  // namespace qtg
