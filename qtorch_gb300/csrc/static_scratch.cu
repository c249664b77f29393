// qt_plan_execute_static: the grouped interpreter with its scratch memory in a
// statically reserved device array, for callers that cannot allocate device
// memory themselves -- code that runs inside a framework that owns every byte
// of the device (a custom call or an operator whose allocator belongs to the
// host framework), or a latency-bound loop that must never pay cudaMalloc's
// implicit device synchronisation.  The caller passes the inputs (the leaf
// tensors) and the output (two doubles) in device memory it already owns;
// the entry point itself calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// The array holds the plan's descriptors, the instance descriptor and the
// workspace of the intermediates.  It is QT_STATIC_SCRATCH_BYTES large, and
// every GPU that loads this library keeps it until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "kernels.h"
#include "plan.h"

namespace qtg {
namespace {

static __device__ __align__(256) unsigned char g_static_scratch[QT_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

uint64_t align256(uint64_t x) { return (x + 255) / 256 * 256; }

// Host code cannot use g_static_scratch as a device address: its name here is
// a host-side stand-in.  The address comes from the runtime, once per device,
// with that device current.
qt_status scratch_address(qt_ctx *ctx, void **out) {
    std::lock_guard<std::mutex> g(g_setup_lock);
    if (ctx->device < 0 || ctx->device >= kMaxDevices) return QT_ERR_INVALID_ARGUMENT;
    if (!g_scratch_ptr[ctx->device]) {
        int cur = -1;
        cudaError_t e = cudaGetDevice(&cur);
        if (e == cudaSuccess && cur != ctx->device) e = cudaSetDevice(ctx->device);
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (cur >= 0 && cur != ctx->device) cudaSetDevice(cur);
        if (e != cudaSuccess) return cuda_error(ctx, e, "cudaGetSymbolAddress of the static scratch");
        g_scratch_ptr[ctx->device] = p;
    }
    *out = g_scratch_ptr[ctx->device];
    return QT_OK;
}

}  // namespace
}  // namespace qtg

using namespace qtg;

extern "C" qt_status qt_plan_execute_static(qt_ctx *ctx, const qt_plan *p, qt_precision prec, const void *d_leaves,
                                            double *d_value) {
    if (!ctx || !p || !d_leaves || !d_value || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED))
        return QT_ERR_INVALID_ARGUMENT;
    if (!p->grouped)
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT,
                         "plan exceeds the grouped interpreter's limits; qt_plan_execute_static takes grouped plans only");
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    // layout inside the static array: plan descriptor, steps, level starts,
    // rank-0 list, level work items, first tiled step per level, offset tables,
    // instance descriptor, workspace
    const uint64_t steps_bytes = sizeof(StepDesc) * p->steps[prec].size();
    const uint64_t lvl_bytes = sizeof(int32_t) * p->level_start.size();
    const uint64_t r0_bytes = sizeof(int32_t) * p->rank0_steps.size();
    const uint64_t items_bytes = sizeof(uint32_t) * p->level_items[prec].size();
    const uint64_t off_steps = align256(sizeof(PlanDesc));
    const uint64_t off_lvl = align256(off_steps + steps_bytes);
    const uint64_t off_r0 = align256(off_lvl + lvl_bytes);
    const uint64_t off_items = align256(off_r0 + r0_bytes);
    const uint64_t cta_bytes = sizeof(int32_t) * p->level_cta.size();
    const uint64_t off_cta = align256(off_items + items_bytes);
    const uint64_t map_bytes = p->item_step[prec].size();
    const uint64_t off_map = align256(off_cta + cta_bytes);
    const uint64_t hot_bytes = sizeof(HotStep) * p->hot[prec].size();
    const uint64_t off_hot = align256(off_map + map_bytes);
    const uint64_t meta_bytes = sizeof(uint32_t) * p->level_meta[prec].size();
    const uint64_t off_meta = align256(off_hot + hot_bytes);
    const uint64_t tab_bytes = sizeof(ushort2) * p->tables.size();
    const uint64_t off_tab = align256(off_meta + meta_bytes);
    const uint64_t off_inst = align256(off_tab + tab_bytes);
    const uint64_t off_ws = align256(off_inst + sizeof(InstanceDesc));
    const uint64_t total = off_ws + align256(p->ws_bytes[prec]);
    if (total > QT_STATIC_SCRATCH_BYTES)
        return set_error(ctx, QT_ERR_OUT_OF_MEMORY,
                         "plan needs " + std::to_string(total) + " bytes of scratch; the static scratch holds " +
                             std::to_string((unsigned long long) QT_STATIC_SCRATCH_BYTES));
    void *base = nullptr;
    qt_status s = scratch_address(ctx, &base);
    if (s != QT_OK) return s;
    char *b = static_cast<char *>(base);
    PlanDesc pd;
    std::memset(&pd, 0, sizeof pd);
    pd.steps = reinterpret_cast<const StepDesc *>(b + off_steps);
    pd.level_start = reinterpret_cast<const int32_t *>(b + off_lvl);
    pd.rank0_steps = reinterpret_cast<const int32_t *>(b + off_r0);
    pd.level_items = reinterpret_cast<const uint32_t *>(b + off_items);
    pd.tables = reinterpret_cast<const ushort2 *>(b + off_tab);
    pd.level_cta = reinterpret_cast<const int32_t *>(b + off_cta);
    pd.item_step = map_bytes ? reinterpret_cast<const uint8_t *>(b + off_map) : nullptr;
    pd.hot = reinterpret_cast<const HotStep *>(b + off_hot);
    pd.level_meta = reinterpret_cast<const uint32_t *>(b + off_meta);
    pd.n_steps = p->n_steps;
    pd.n_levels = p->n_levels;
    pd.n_rank0 = (int32_t) p->rank0_steps.size();
    InstanceDesc inst{};
    inst.plan = reinterpret_cast<const PlanDesc *>(b);
    inst.leaves = static_cast<const char *>(d_leaves);
    inst.value = d_value;
    inst.plan_bytes = 0;   // read in place from the static array, never staged
    inst.leaf_bytes = 0;
    inst.ws_bytes = (uint32_t) align256(p->ws_bytes[prec]);
    inst.n_steps = (uint32_t) p->n_steps;
    inst.angles = nullptr;   // the caller's leaves are used as they are
    // the descriptors of the previous call are overwritten; the workspace needs
    // no clearing (every intermediate is written before it is read)
    cudaError_t e = cudaMemcpyAsync(b, &pd, sizeof pd, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && steps_bytes)
        e = cudaMemcpyAsync(b + off_steps, p->steps[prec].data(), steps_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && lvl_bytes)
        e = cudaMemcpyAsync(b + off_lvl, p->level_start.data(), lvl_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && r0_bytes)
        e = cudaMemcpyAsync(b + off_r0, p->rank0_steps.data(), r0_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && items_bytes)
        e = cudaMemcpyAsync(b + off_items, p->level_items[prec].data(), items_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && cta_bytes)
        e = cudaMemcpyAsync(b + off_cta, p->level_cta.data(), cta_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && meta_bytes)
        e = cudaMemcpyAsync(b + off_meta, p->level_meta[prec].data(), meta_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && hot_bytes)
        e = cudaMemcpyAsync(b + off_hot, p->hot[prec].data(), hot_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && map_bytes)
        e = cudaMemcpyAsync(b + off_map, p->item_step[prec].data(), map_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && tab_bytes)
        e = cudaMemcpyAsync(b + off_tab, p->tables.data(), tab_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b + off_inst, &inst, sizeof inst, cudaMemcpyHostToDevice, ctx->stream);
    // Copies from pageable host memory: each returns once its source has been
    // staged by the driver, so pd and inst may go out of scope afterwards and
    // the host never waits for earlier work on the stream.
    if (e != cudaSuccess) return cuda_error(ctx, e, "static scratch upload");
    PlanLaunch lp{};
    lp.instances = reinterpret_cast<const InstanceDesc *>(b + off_inst);
    lp.n_instances = 1;
    lp.ws_smem_bytes = 0;   // the workspace is the static array's tail
    lp.ws_base = b + off_ws;
    lp.ws_stride = align256(p->ws_bytes[prec]);
    lp.stage_bytes = 0;
    lp.tile_bytes = p->n_tiled ? kCtaTileBytes : 0;
    lp.next = nullptr;
    lp.header_steps = (uint32_t) p->n_steps;
    e = launch_plan(lp, prec == QT_PREC_MIXED, 1, ctx->stream);
    ctx->launches++;
    return cuda_error(ctx, e, "plan kernel launch");
}
