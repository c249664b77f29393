// C ABI: contexts, the caching device allocator, tensors and the pairwise
// contraction entry points (the drop-in for Network::ContractIndices,
// src/Network.h:876-971).
#include "core.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>

#include "gemm_tc.h"
#include "kernels.h"
#include "permute.h"
#include "stream.h"

namespace qtg {

qt_status set_error(qt_ctx *ctx, qt_status s, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->err_lock);
        ctx->last_error = msg;
    }
    return s;
}

qt_status cuda_error(qt_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return QT_OK;
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_error(ctx, QT_ERR_OUT_OF_MEMORY, msg);
    return set_error(ctx, QT_ERR_CUDA, msg);
}

// largest ratio of a cached block's class to the requested class that a
// request may take instead of allocating (twice for blocks above 64 MB)
static size_t cache_stretch(size_t cls) { return cls <= (64ull << 20) ? 4 : 2; }

static size_t size_class(size_t bytes) {
    size_t c = 256;
    while (c < bytes) c <<= 1;
    return c;
}

// every live context, for the allocator's last resort (dev_alloc)
static std::mutex g_ctx_list_lock;
static std::vector<qt_ctx *> g_ctx_list;

// Frees a context's cached blocks (caller holds its alloc_lock).  cudaFree
// waits for the device, so blocks that in-flight work on the owner's stream
// released in stream order are idle by then.
static void trim_cache(qt_ctx *c) {
    for (auto &kv : c->free_blocks)
        for (void *q : kv.second) {
            cudaFree(q);
            c->block_size.erase(q);
        }
    c->free_blocks.clear();
    c->bytes_cached = 0;
}

void ctx_retain(qt_ctx *ctx) {
    if (ctx) ctx->refs.fetch_add(1);
}

void ctx_release(qt_ctx *ctx) {
    if (!ctx || ctx->refs.fetch_sub(1) != 1) return;
    {
        std::lock_guard<std::mutex> g(g_ctx_list_lock);
        g_ctx_list.erase(std::remove(g_ctx_list.begin(), g_ctx_list.end(), ctx), g_ctx_list.end());
    }
    cudaSetDevice(ctx->device);
    // a caller's stream may be gone by now; cudaFree waits for the device anyway
    if (ctx->pool && ctx->own_stream) {
        // blocks still held go back to the pool; then the pool returns what no
        // context uses to the device (a server that closes leaves nothing mapped)
        for (auto &kv : ctx->block_size) cudaFreeAsync(kv.first, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        cudaMemPoolTrimTo(ctx->pool, 0);
    }
    if (ctx->own_stream) cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->free_blocks)
        for (void *p : kv.second) cudaFree(p);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    for (auto &kv : ctx->free_pinned)
        for (void *p : kv.second) cudaFreeHost(p);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

qt_status host_alloc(qt_ctx *ctx, size_t bytes, void **out) {
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    const size_t cls = size_class(std::max<size_t>(bytes, ctx->min_class));
    // a cached block of this class, or of a somewhat larger class (cache_stretch)
    for (auto it = ctx->free_pinned.lower_bound(cls); it != ctx->free_pinned.end() && it->first <= cls * cache_stretch(cls);
         ++it)
        if (!it->second.empty()) {
            *out = it->second.back();
            it->second.pop_back();
            return QT_OK;
        }
    void *p = nullptr;
    cudaError_t e = cudaMallocHost(&p, cls);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaMallocHost");
    ctx->pinned_size[p] = cls;
    *out = p;
    return QT_OK;
}

void host_free(qt_ctx *ctx, void *p) {
    if (!p) return;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    auto it = ctx->pinned_size.find(p);
    if (it == ctx->pinned_size.end()) return;
    ctx->free_pinned[it->second].push_back(p);
}

// One stream-ordered pool per device, for the contexts that allocate from one
// (a server's heavy lanes).  A heavy request's intermediates come in sizes
// that change from request to request; per-context caches of size classes
// kept every lane's blocks apart, outgrew the device and were emptied with
// cudaFree, which waits for the whole device (a serving run measured 1.8 k
// cudaMalloc and 2.3 k cudaFree calls, single calls up to 0.2 s, while light
// requests waited behind them).  The pool splits and merges its own blocks,
// keeps the memory it has mapped (release threshold: never), gives a lane a
// block another lane freed once that free has completed on the GPU, and
// never makes one lane's stream wait for another's (no internal
// dependencies); cudaFreeAsync synchronises nothing.
qt_status device_pool(int device, cudaMemPool_t *out) {
    static std::mutex m;
    static cudaMemPool_t pools[64] = {};
    std::lock_guard<std::mutex> g(m);
    if (device < 0 || device >= 64) return QT_ERR_INVALID_ARGUMENT;
    if (!pools[device]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        uint64_t keep = UINT64_MAX;
        int no = 0, yes = 1;
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowInternalDependencies, &no);
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowOpportunistic, &yes);
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(p, cudaMemPoolReuseFollowEventDependencies, &yes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (p) cudaMemPoolDestroy(p);
            return QT_ERR_CUDA;
        }
        pools[device] = p;
    }
    *out = pools[device];
    return QT_OK;
}

// Empties the caches of the device's other contexts (the allocators' last
// resort; cudaFree waits for the device).
static void trim_other_caches(qt_ctx *ctx) {
    std::lock_guard<std::mutex> lg(g_ctx_list_lock);
    for (qt_ctx *o : g_ctx_list) {
        if (o == ctx || o->device != ctx->device) continue;
        std::unique_lock<std::mutex> og(o->alloc_lock, std::try_to_lock);
        if (og.owns_lock()) trim_cache(o);
    }
}

// A block from the context's pool, in its stream's order.
static qt_status pool_alloc(qt_ctx *ctx, std::unique_lock<std::mutex> &g, size_t bytes, void **out) {
    const size_t sz = std::max<size_t>((bytes + 255) / 256 * 256, 256);
    if (ctx->memory_budget && ctx->bytes_in_use + sz > ctx->memory_budget)
        return set_error(ctx, QT_ERR_OUT_OF_MEMORY, "device memory budget exceeded");
    void *p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, sz, ctx->pool, ctx->stream);
    if (e == cudaErrorMemoryAllocation) {
        // the other contexts' cached blocks go back to the device, then once more
        cudaGetLastError();
        g.unlock();
        trim_other_caches(ctx);
        g.lock();
        e = cudaMallocFromPoolAsync(&p, sz, ctx->pool, ctx->stream);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_error(ctx, e, "cudaMallocFromPoolAsync");
    }
    ctx->block_size[p] = sz;
    ctx->bytes_in_use += sz;
    *out = p;
    return QT_OK;
}

qt_status dev_alloc(qt_ctx *ctx, size_t bytes, void **out) {
    std::unique_lock<std::mutex> g(ctx->alloc_lock);
    if (ctx->pool) return pool_alloc(ctx, g, bytes, out);
    const size_t cls = size_class(std::max<size_t>(bytes, ctx->min_class));
    // a cached block of this class, or of a somewhat larger class
    // (cache_stretch): a cudaMalloc can wait tens of milliseconds behind other threads'
    // large allocations, a somewhat larger block costs nothing
    for (auto it = ctx->free_blocks.lower_bound(cls); it != ctx->free_blocks.end() && it->first <= cls * cache_stretch(cls);
         ++it)
        if (!it->second.empty()) {
            *out = it->second.back();
            it->second.pop_back();
            ctx->bytes_cached -= it->first;
            ctx->bytes_in_use += it->first;
            return QT_OK;
        }
    if (ctx->memory_budget && ctx->bytes_in_use + cls > ctx->memory_budget)
        return set_error(ctx, QT_ERR_OUT_OF_MEMORY, "device memory budget exceeded");
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, cls);
    if (e == cudaErrorMemoryAllocation) {
        // give the cached blocks back and retry once
        cudaGetLastError();
        trim_cache(ctx);
        e = cudaMalloc(&p, cls);
    }
    if (e == cudaErrorMemoryAllocation) {
        // then the other contexts' caches on this device (the lanes of a
        // server each keep their own): each is taken only if its allocator is
        // free right now, so two contexts doing this at once cannot deadlock
        cudaGetLastError();
        g.unlock();
        trim_other_caches(ctx);
        g.lock();
        e = cudaMalloc(&p, cls);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_error(ctx, e, "cudaMalloc");
    }
    ctx->block_size[p] = cls;
    ctx->bytes_in_use += cls;
    ctx->device_allocs++;
    *out = p;
    return QT_OK;
}

void dev_free(qt_ctx *ctx, void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(ctx->alloc_lock);
    auto it = ctx->block_size.find(p);
    if (it == ctx->block_size.end()) return;
    if (ctx->pool) {
        // back to the pool once the stream has passed its last use
        cudaFreeAsync(p, ctx->stream);
        ctx->bytes_in_use -= it->second;
        ctx->block_size.erase(it);
        return;
    }
    ctx->free_blocks[it->second].push_back(p);
    ctx->bytes_in_use -= it->second;
    ctx->bytes_cached += it->second;
}

qt_status ensure_pinned(qt_ctx *ctx, size_t bytes) {
    if (ctx->pinned_bytes >= bytes) return QT_OK;
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    size_t want = 1 << 20;
    while (want < bytes) want <<= 1;
    cudaError_t e = cudaMallocHost(&ctx->pinned, want);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaMallocHost");
    ctx->pinned_bytes = want;
    return QT_OK;
}

bool deadline_passed(qt_ctx *ctx) {
    return ctx->has_deadline && std::chrono::steady_clock::now() > ctx->deadline;
}

bool tensor_cores_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("QT_DISABLE_TCGEN05");
        return !(v && v[0] == '1');
    }();
    return on;
}

bool stream_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("QT_DISABLE_STREAM");
        return !(v && v[0] == '1');
    }();
    return on;
}

// QT_STREAM_FIRST=1 offers every complex64 step to the streaming kernel before
// the tensor-core and tiled kernels (for measuring one against the other)
static bool stream_first() {
    static const bool on = [] {
        const char *v = std::getenv("QT_STREAM_FIRST");
        return v && v[0] == '1';
    }();
    return on;
}

qt_status run_contraction(qt_ctx *ctx, const StepDesc &d, const void *A, const void *B, void *C, bool f64,
                          int *gemm_flag, const StepScaleRef &sc) {
    // a long sum into a few outputs: the whole GPU on one sum.  In complex64
    // every such reduction (rank <= 2, >= 64 terms) takes the compensated kernel:
    // these are the expectation values where cancellation lives.
    const bool small_out = (1ull << (2 * d.nFree)) <= kReduceMaxOut;
    if (reduce_shaped(d) || (!f64 && small_out && d.nSum >= 3)) {
        if (f64) {
            cudaError_t e = launch_reduce_exact(d, (const double2 *) A, (const double2 *) B, (double2 *) C, ctx->stream);
            ctx->launches++;
            return cuda_error(ctx, e, "reduction launch");
        }
        const bool aligned = ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15u) == 0;
        if (d.nFree == 0 && d.rA == d.rB && d.nSum == d.rA && d.rA >= 4 && aligned) {
            // a full contraction (the expectation value of a large network):
            // tiles of A and B, each read along its own contiguous runs, meet in
            // shared memory (permute.cu) instead of one side being gathered
            int32_t perm[kPermMaxRank];
            for (int j = 0; j < d.nSum; j++) perm[d.posBs[j]] = d.posAs[j];   // B digit <- A digit
            PermutePlan pp;
            if (permute_plan(d.rA, perm, 8, pp)) {
                void *partials = nullptr;
                qt_status s = dev_alloc(ctx, sizeof(float4) * (size_t) dot_grid(pp), &partials);
                if (s != QT_OK) return s;
                cudaError_t e = launch_permuted_dot(pp, (const float2 *) A, (const float2 *) B, (float2 *) C, partials, sc,
                                                    ctx->stream);
                ctx->launches += 2;
                dev_free(ctx, partials);
                return cuda_error(ctx, e, "reduction launch");
            }
        }
        void *scratch = nullptr;
        qt_status s = dev_alloc(ctx, reduce_scratch_bytes(d), &scratch);
        if (s != QT_OK) return s;
        cudaError_t e = launch_reduce_f32(d, (const float2 *) A, (const float2 *) B, (float2 *) C, scratch, ctx->stream, sc);
        ctx->launches += 2;
        dev_free(ctx, scratch);   // stream-ordered: the next user of the block runs after these kernels
        return cuda_error(ctx, e, "reduction launch");
    }
    // Complex64 steps with one small operand stream the large one (stream.cu)
    // unless the tiled or tensor-core kernel does better for the shape:
    // measured per shape, the streaming kernel wins whenever it is the only
    // candidate (1.5-5.7x the pair kernel), and among wide or GEMM-shaped steps
    // when the large operand is A -- C's low digits are then its free wires and
    // the owning lanes store consecutive elements -- except with exactly 16
    // free indices of the small operand; when the large operand is B the
    // tiled kernel's output tiles store better.  Dense steps of two large
    // operands take the tensor cores (gemm_tc.cu), other wide ones the tiled
    // kernel.  The TMA-fed kernels report pipeline timeouts through a device
    // flag: the caller's, read once after its last step, or one checked here.
    StreamStep sp;
    const bool can_stream = !f64 && stream_enabled() && stream_plan(d, sp);
    const bool gemm_ok = !f64 && tensor_cores_enabled() && gemm_eligible(d);
    const bool use_stream = can_stream && (stream_first() || (!sp.l_is_b && sp.nsf != 2) ||
                                           (!gemm_ok && !tiled_shaped(d)));
    const bool use_gemm = !use_stream && gemm_ok;
    if (use_stream || use_gemm) {
        void *scratch = nullptr, *flag = gemm_flag;
        qt_status s = QT_OK;
        if (use_gemm) s = dev_alloc(ctx, sizeof(float) * gemm_scratch_floats(d), &scratch);
        if (s == QT_OK && !gemm_flag) s = dev_alloc(ctx, 256, &flag);
        if (s == QT_OK) {
            cudaError_t e = gemm_flag ? cudaSuccess : cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream);
            if (e == cudaSuccess) {
                if (use_stream) {
                    e = launch_stream(sp, d, (const float2 *) A, (const float2 *) B, (float2 *) C, sc, (int *) flag,
                                      ctx->stream);
                    ctx->launches += 1;
                    ctx->stream_steps++;
                } else {
                    e = launch_gemm_step(d, (const float2 *) A, (const float2 *) B, (float2 *) C, (float *) scratch,
                                         (int *) flag, ctx->stream, sc);
                    ctx->launches += 3;
                    ctx->tc_steps++;
                }
            }
            int h = 0;
            if (!gemm_flag) {
                if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            }
            s = cuda_error(ctx, e, use_stream ? "streaming contraction" : "tensor-core contraction");
            if (s == QT_OK && h) s = set_error(ctx, QT_ERR_CUDA, "TMA pipeline wait timed out");
        }
        dev_free(ctx, scratch);   // stream-ordered: the next user of the block runs after this step
        if (!gemm_flag) dev_free(ctx, flag);
        return s;
    }
    if (tiled_shaped(d)) {
        cudaError_t e = launch_tiled_pair(d, A, B, C, f64, ctx->stream, sc);
        ctx->launches++;
        return cuda_error(ctx, e, "tiled kernel launch");
    }
    cudaError_t e = launch_pair(d, A, B, C, f64, ctx->stream, sc);
    ctx->launches++;
    return cuda_error(ctx, e, "pair kernel launch");
}

qt_status make_step(int rank_a, int rank_b, int n_free, const uint8_t *free_from_a, const int32_t *free_idx,
                    int n_sum, const int32_t *sum_a, const int32_t *sum_b, StepDesc *d) {
    if (rank_a < 0 || rank_b < 0 || rank_a > kMaxWires || rank_b > kMaxWires || n_free < 0 || n_sum < 0 ||
        n_free > kMaxWires || n_sum > kMaxWires)
        return QT_ERR_INVALID_ARGUMENT;
    if (n_free + 2 * n_sum != rank_a + rank_b) return QT_ERR_INVALID_ARGUMENT;
    std::memset(d, 0, sizeof(*d));
    d->rA = (uint8_t) rank_a;
    d->rB = (uint8_t) rank_b;
    d->nFree = (uint8_t) n_free;
    d->nSum = (uint8_t) n_sum;
    int seenA[kMaxWires] = {0}, seenB[kMaxWires] = {0};
    int fa = 0, fb = 0;
    for (int i = 0; i < n_free; i++) {
        const int w = free_idx[i];
        if (free_from_a[i]) {
            if (w < 0 || w >= rank_a || seenA[w]++) return QT_ERR_INVALID_ARGUMENT;
            d->cA[i] = (uint8_t) w;
            d->cB[i] = kNoWire;
            fa++;
        } else {
            if (w < 0 || w >= rank_b || seenB[w]++) return QT_ERR_INVALID_ARGUMENT;
            d->cB[i] = (uint8_t) w;
            d->cA[i] = kNoWire;
            fb++;
        }
    }
    for (int j = 0; j < n_sum; j++) {
        const int wa = sum_a[j], wb = sum_b[j];
        if (wa < 0 || wa >= rank_a || seenA[wa]++) return QT_ERR_INVALID_ARGUMENT;
        if (wb < 0 || wb >= rank_b || seenB[wb]++) return QT_ERR_INVALID_ARGUMENT;
        // digit i of k <-> pair n_sum-1-i (src/Network.h:912-916)
        d->posAs[n_sum - 1 - j] = (uint8_t) wa;
        d->posBs[n_sum - 1 - j] = (uint8_t) wb;
    }
    d->fA = (uint8_t) fa;
    d->fB = (uint8_t) fb;
    d->a_step = d->b_step = -1;
    return QT_OK;
}

}  // namespace qtg

using namespace qtg;

extern "C" {

const char *qt_status_string(qt_status s) {
    switch (s) {
        case QT_OK: return "ok";
        case QT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case QT_ERR_INVALID_FILE: return "Invalid Input or Output File Path";
        case QT_ERR_INVALID_FILE_FORMAT: return "Invalid File Format.";
        case QT_ERR_CONTRACTION_FAILURE: return "Contraction Failed.";
        case QT_ERR_INVALID_USER_SEQUENCE: return "Invalid User Defined Contraction Sequence.";
        case QT_ERR_INVALID_FUNCTION_INPUT: return "Input to Function Invalid.";
        case QT_ERR_INVALID_CONTRACTION_METHOD: return "Invalid Contraction Method.";
        case QT_ERR_REFUSED: return "contraction refused";
        case QT_ERR_OUT_OF_MEMORY: return "out of device memory or over the memory budget";
        case QT_ERR_CUDA: return "CUDA error";
        case QT_ERR_DEADLINE: return "deadline expired";
        case QT_ERR_NO_DEVICE: return "no usable CUDA device";
        case QT_ERR_BUSY: return "not enough free budget right now";
    }
    return "unknown status";
}

qt_status qt_ctx_create(int device, void *stream, qt_ctx **out) {
    if (!out) return QT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
        cudaGetLastError();
        return QT_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return QT_ERR_NO_DEVICE;
    // the kernels are built for sm_103a only
    if (prop.major != 10 || prop.minor != 3) return QT_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return QT_ERR_NO_DEVICE;
    qt_ctx *ctx = new (std::nothrow) qt_ctx();
    if (!ctx) return QT_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    if (stream) {
        ctx->stream = (cudaStream_t) stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return QT_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    {
        std::lock_guard<std::mutex> g(g_ctx_list_lock);
        g_ctx_list.push_back(ctx);
    }
    *out = ctx;
    return QT_OK;
}



qt_status qt_ctx_destroy(qt_ctx *ctx) {
    if (!ctx) return QT_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::recursive_mutex> g(ctx->lock);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    ctx_release(ctx);
    return QT_OK;
}

qt_status qt_ctx_synchronize(qt_ctx *ctx) {
    if (!ctx) return QT_ERR_INVALID_ARGUMENT;
    return cuda_error(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
}

size_t qt_last_error(qt_ctx *ctx, char *buf, size_t cap) {
    if (!ctx) return 0;
    std::lock_guard<std::mutex> g(ctx->err_lock);
    if (buf && cap) {
        size_t n = ctx->last_error.size() < cap - 1 ? ctx->last_error.size() : cap - 1;
        std::memcpy(buf, ctx->last_error.data(), n);
        buf[n] = 0;
    }
    return ctx->last_error.size();
}

qt_status qt_ctx_set_memory_budget(qt_ctx *ctx, uint64_t bytes) {
    if (!ctx) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    ctx->memory_budget = bytes;
    return QT_OK;
}

qt_status qt_ctx_set_deadline(qt_ctx *ctx, double seconds) {
    if (!ctx) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (seconds <= 0) {
        ctx->has_deadline = false;
    } else {
        ctx->has_deadline = true;
        ctx->deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration_cast<std::chrono::steady_clock::duration>(std::chrono::duration<double>(seconds));
    }
    return QT_OK;
}

uint64_t qt_ctx_kernel_launches(const qt_ctx *ctx) { return ctx ? ctx->launches.load() : 0; }

uint64_t qt_ctx_tensor_core_steps(const qt_ctx *ctx) { return ctx ? ctx->tc_steps.load() : 0; }

uint64_t qt_ctx_stream_steps(const qt_ctx *ctx) { return ctx ? ctx->stream_steps.load() : 0; }

qt_status qt_debug_stream_fault(qt_ctx *ctx, int mode, uint32_t polls) {
    if (!ctx || mode < 0 || mode > 1) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = stream_set_fault(mode, polls);
    return cuda_error(ctx, e, "stream fault hook");
}

qt_status qt_debug_gemm_fault(qt_ctx *ctx, int mode, uint32_t polls) {
    if (!ctx || mode < 0 || mode > 1) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = gemm_set_fault(mode, polls);
    return cuda_error(ctx, e, "GEMM fault hook");
}

qt_status qt_debug_staging_fault(qt_ctx *ctx, int mode, uint32_t polls) {
    if (!ctx || mode < 0 || mode > 1) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = plan_set_staging_fault(mode, polls);
    return cuda_error(ctx, e, "staging fault hook");
}

qt_status qt_ctx_memory_stats(qt_ctx *ctx, uint64_t *bytes_in_use, uint64_t *bytes_cached, uint64_t *device_allocations) {
    if (!ctx) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(ctx->alloc_lock);
    if (bytes_in_use) *bytes_in_use = ctx->bytes_in_use;
    if (bytes_cached) *bytes_cached = ctx->bytes_cached;
    if (device_allocations) *device_allocations = ctx->device_allocs.load();
    return QT_OK;
}

qt_status qt_tensor_create(qt_ctx *ctx, int rank, qt_dtype dtype, qt_tensor **out) {
    if (!ctx || !out || rank < 0 || rank > kMaxWires || (dtype != QT_C128 && dtype != QT_C64)) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    qt_tensor *t = new (std::nothrow) qt_tensor();
    if (!t) return QT_ERR_OUT_OF_MEMORY;
    t->rank = rank;
    t->dtype = dtype;
    t->bytes = (size_t) elem_bytes(dtype) << (2 * rank);
    qt_status s = dev_alloc(ctx, t->bytes, &t->ptr);
    if (s != QT_OK) {
        delete t;
        return s;
    }
    cudaError_t e = cudaMemsetAsync(t->ptr, 0, t->bytes, ctx->stream);
    if (e != cudaSuccess) {
        dev_free(ctx, t->ptr);
        delete t;
        return cuda_error(ctx, e, "cudaMemsetAsync");
    }
    *out = t;
    return QT_OK;
}

qt_status qt_tensor_free(qt_ctx *ctx, qt_tensor *t) {
    if (!ctx || !t) return QT_ERR_INVALID_ARGUMENT;
    // blocks go back to the cache; stream order keeps later reuse safe
    dev_free(ctx, t->ptr);
    delete t;
    return QT_OK;
}

qt_status qt_tensor_upload(qt_ctx *ctx, qt_tensor *t, const void *host, size_t bytes) {
    if (!ctx || !t || !host || bytes != t->bytes) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaError_t e = cudaMemcpyAsync(t->ptr, host, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_error(ctx, e, "upload");
}

qt_status qt_tensor_download(qt_ctx *ctx, const qt_tensor *t, void *host, size_t bytes) {
    if (!ctx || !t || !host || bytes != t->bytes) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaError_t e = cudaMemcpyAsync(host, t->ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_error(ctx, e, "download");
}

int qt_tensor_rank(const qt_tensor *t) { return t ? t->rank : -1; }
qt_dtype qt_tensor_dtype(const qt_tensor *t) { return t ? t->dtype : QT_C128; }
void *qt_tensor_device_ptr(const qt_tensor *t) { return t ? t->ptr : nullptr; }

qt_status qt_contract_pair_device(qt_ctx *ctx, const void *a, int rank_a, const void *b, int rank_b, int n_free,
                                  const uint8_t *free_from_a, const int32_t *free_idx, int n_sum,
                                  const int32_t *sum_a, const int32_t *sum_b, void *c) {
    if (!ctx || !a || !b || !c) return QT_ERR_INVALID_ARGUMENT;
    if ((n_free && (!free_from_a || !free_idx)) || (n_sum && (!sum_a || !sum_b))) return QT_ERR_INVALID_ARGUMENT;
    StepDesc d;
    qt_status s = make_step(rank_a, rank_b, n_free, free_from_a, free_idx, n_sum, sum_a, sum_b, &d);
    if (s != QT_OK) return set_error(ctx, s, "index maps do not describe a contraction of these ranks");
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
    cudaError_t e = launch_pair(d, a, b, c, true, ctx->stream);
    ctx->launches++;
    return cuda_error(ctx, e, "pair kernel launch");
}

qt_status qt_contract_pair(qt_ctx *ctx, const qt_tensor *a, const qt_tensor *b, int n_free,
                           const uint8_t *free_from_a, const int32_t *free_idx, int n_sum,
                           const int32_t *sum_a, const int32_t *sum_b, qt_tensor **c_out) {
    if (!ctx || !a || !b || !c_out) return QT_ERR_INVALID_ARGUMENT;
    // an operand without data is the reference's InvalidFunctionInput (Network.h:938-940)
    if (!a->ptr || !b->ptr) return set_error(ctx, QT_ERR_INVALID_FUNCTION_INPUT, "operand holds no data");
    if (a->dtype != b->dtype) return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "operand dtypes differ");
    if ((n_free && (!free_from_a || !free_idx)) || (n_sum && (!sum_a || !sum_b))) return QT_ERR_INVALID_ARGUMENT;
    StepDesc d;
    qt_status s = make_step(a->rank, b->rank, n_free, free_from_a, free_idx, n_sum, sum_a, sum_b, &d);
    if (s != QT_OK) return set_error(ctx, s, "index maps do not describe a contraction of these ranks");
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
    qt_tensor *c = new (std::nothrow) qt_tensor();
    if (!c) return QT_ERR_OUT_OF_MEMORY;
    c->rank = n_free;
    c->dtype = a->dtype;
    c->bytes = (size_t) elem_bytes(c->dtype) << (2 * n_free);
    s = dev_alloc(ctx, c->bytes, &c->ptr);
    if (s != QT_OK) {
        delete c;
        return s;
    }
    // every output element is written by the kernel; no zero fill needed
    s = run_contraction(ctx, d, a->ptr, b->ptr, c->ptr, a->dtype == QT_C128);
    if (s != QT_OK) {
        dev_free(ctx, c->ptr);
        delete c;
        return s;
    }
    *c_out = c;
    return QT_OK;
}

qt_status qt_permute_device(qt_ctx *ctx, const void *in, int rank, qt_dtype dtype, const int32_t *perm, void *out) {
    if (!ctx || !in || !out || (dtype != QT_C64 && dtype != QT_C128)) return QT_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
    PermutePlan p;
    if (!permute_plan(rank, perm, (uint32_t) elem_bytes(dtype), p))
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "perm is not a permutation of the tensor's wires");
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
    cudaError_t e = launch_permute(p, in, out, ctx->stream);
    ctx->launches++;
    return cuda_error(ctx, e, "permute launch");
}

qt_status qt_tensor_permute(qt_ctx *ctx, const qt_tensor *in, const int32_t *perm, qt_tensor **out) {
    if (!ctx || !in || !out) return QT_ERR_INVALID_ARGUMENT;
    if (!in->ptr) return set_error(ctx, QT_ERR_INVALID_FUNCTION_INPUT, "tensor holds no data");
    PermutePlan p;
    if (!permute_plan(in->rank, perm, (uint32_t) elem_bytes(in->dtype), p))
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "perm is not a permutation of the tensor's wires");
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    qt_tensor *t = new (std::nothrow) qt_tensor();
    if (!t) return QT_ERR_OUT_OF_MEMORY;
    t->rank = in->rank;
    t->dtype = in->dtype;
    t->bytes = in->bytes;
    qt_status s = dev_alloc(ctx, t->bytes, &t->ptr);
    if (s == QT_OK) s = qt_permute_device(ctx, in->ptr, in->rank, in->dtype, perm, t->ptr);
    if (s != QT_OK) {
        if (t->ptr) dev_free(ctx, t->ptr);
        delete t;
        return s;
    }
    *out = t;
    return QT_OK;
}

qt_status qt_contract_pair_host(qt_ctx *ctx, const double *a, int rank_a, const double *b, int rank_b, int n_free,
                                const uint8_t *free_from_a, const int32_t *free_idx, int n_sum, const int32_t *sum_a,
                                const int32_t *sum_b, double *c) {
    if (!ctx || !a || !b || !c) return QT_ERR_INVALID_ARGUMENT;
    if (rank_a < 0 || rank_b < 0 || n_free < 0 || rank_a > kMaxWires || rank_b > kMaxWires || n_free > kMaxWires)
        return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    const size_t ba = (size_t) 16 << (2 * rank_a), bb = (size_t) 16 << (2 * rank_b), bc = (size_t) 16 << (2 * n_free);
    void *da = nullptr, *db = nullptr, *dc = nullptr;
    qt_status s = dev_alloc(ctx, ba, &da);
    if (s == QT_OK) s = dev_alloc(ctx, bb, &db);
    if (s == QT_OK) s = dev_alloc(ctx, bc, &dc);
    if (s == QT_OK) {
        cudaError_t e = cudaMemcpyAsync(da, a, ba, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, bb, cudaMemcpyHostToDevice, ctx->stream);
        s = cuda_error(ctx, e, "upload");
    }
    if (s == QT_OK)
        s = qt_contract_pair_device(ctx, da, rank_a, db, rank_b, n_free, free_from_a, free_idx, n_sum, sum_a, sum_b, dc);
    if (s == QT_OK) {
        cudaError_t e = cudaMemcpyAsync(c, dc, bc, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        s = cuda_error(ctx, e, "download");
    }
    dev_free(ctx, da);
    dev_free(ctx, db);
    dev_free(ctx, dc);
    return s;
}

}  // extern "C"

namespace qtg {

// A context whose own stream has the device's highest (or lowest) priority:
// CTAs of kernels on a high-priority stream are dispatched before waiting CTAs
// of lower-priority kernels, so short launches do not queue behind long ones.
qt_status ctx_create_prioritised(int device, bool high_priority, qt_ctx **out) {
    qt_status s = qt_ctx_create(device, nullptr, out);
    if (s != QT_OK) return s;
    int least = 0, greatest = 0;
    cudaStream_t st = nullptr;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
        cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, high_priority ? greatest : least) == cudaSuccess) {
        cudaStreamDestroy((*out)->stream);
        (*out)->stream = st;
    }
    cudaGetLastError();
    return QT_OK;
}

}  // namespace qtg
