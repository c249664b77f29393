// Host-side plan and batch objects of the C ABI.
#pragma once
#include <atomic>
#include <complex>
#include <string>
#include <vector>

#include "../../include/qtorch/qtorch.hpp"
#include "core.h"

namespace qtg {

// Mixed plans accumulate the reductions where cancellation lives with
// compensated (twice-FP32) dot products and store them as complex128: every
// rank-0 output, and outputs of rank <= kMixedTailRank summed over at least
// 4^kMixedTailMinSum terms.  Everything else is complex64 with FP32 FMA.
constexpr int kMixedTailRank = 1;
constexpr int kMixedTailMinSum = 3;
// limits of the grouped interpreter (one CTA per instance)
constexpr int kGroupedMaxRank = 11;
constexpr int kGroupedMaxSum = 8;
constexpr uint64_t kGroupedMaxWorkspace = 96ull << 20;
// Shared memory of an interpreter CTA: instances whose workspace is at most
// kSmemWorkspaceMax keep it in shared memory, those whose plan block + leaves
// are at most kSmemStageMax are staged there.  The caps keep two CTAs per SM
// (the register budget allows two), larger instances run from global memory.
constexpr uint64_t kSmemWorkspaceMax = 32ull << 10;
// workspace cap when instances outnumber two CTAs per SM (four CTAs per SM)
constexpr uint64_t kSmemWorkspaceMaxMany = 16ull << 10;
constexpr uint64_t kSmemStageMax = 64ull << 10;
// staging cap when the CTA also holds the tile buffers of CTA-tiled steps
constexpr uint64_t kSmemStageMaxTiled = 52ull << 10;
// staging cap of the wide interpreter (one CTA per SM): room for a plan block
// with its per-item descriptors
constexpr uint64_t kSmemStageMaxWide = 144ull << 10;
constexpr uint64_t kSmemStageMaxWideTiled = 128ull << 10;
inline uint64_t round16(uint64_t x) { return (x + 15) / 16 * 16; }
// offset tables are built when they take at most this many bytes
constexpr uint64_t kMaxTableBytes = 64ull << 10;
// One CTA runs a grouped instance at a few percent of the GPU: a plan above
// this many complex MACs that runs alone (qt_plan_execute) or in a server wave
// goes step by step through the whole-GPU kernels instead.
constexpr int64_t kLoneInstanceMaxMacs = 1ll << 24;
// the same for the FP64 form, whose pipe is ~1/64 of FP32's on this part: one
// CTA takes milliseconds for a 6-qubit depth-10 circuit (1e6 MACs)
constexpr int64_t kLoneInstanceMaxMacsF64 = 1ll << 18;
inline int64_t lone_instance_max_macs(int prec) {
    return prec == 0 ? kLoneInstanceMaxMacsF64 : kLoneInstanceMaxMacs;   // 0: QT_PREC_FP64
}
// plans with at most this many work items carry an item -> step map
constexpr uint64_t kMaxItemMap = 8192;
// plans with at most this many work items carry per-item descriptors (16 B each)
constexpr uint64_t kMaxItemDescs = 8192;

}  // namespace qtg

struct qt_plan {
    explicit qt_plan(qt_ctx *c) : ctx(c) { qtg::ctx_retain(ctx); }
    ~qt_plan() { qtg::ctx_release(ctx); }
    qt_plan(const qt_plan &) = delete;
    qt_plan &operator=(const qt_plan &) = delete;
    qt_ctx *ctx = nullptr;
    std::string qasm, measure, gate_dir;
    std::vector<int> leaf_rank;
    std::vector<std::complex<double>> leaf_values;   // the plan's own circuit, complex128
    std::vector<int32_t> sequence;                    // recorded (idA, idB) pairs
    // rotation leaves in leaf order: kind ("Rx", "Ry", "Rz", "PHASE", "CPHASE"), angle, first element
    std::vector<std::string> rot_kind;
    std::vector<double> rot_angle;
    std::vector<uint64_t> rot_elem;
    std::vector<int> rot_leaf;                        // leaf index of each rotation
    std::vector<uint2> rot_table[2];                  // per precision: (leaf byte offset, RotationKind)
    std::vector<qtg::StepDesc> steps[2];              // per precision, sorted by level
    std::vector<int> a_leaf, b_leaf;                  // leaf index of each operand or -1
    std::vector<int32_t> level_start;
    std::vector<int32_t> level_cta;                   // first CTA-tiled step of each level
    int n_tiled = 0;                                  // CTA-tiled steps
    std::vector<int32_t> rank0_steps;
    std::vector<uint32_t> level_items[2];             // interpreter work items per level, per precision
    std::vector<uint8_t> item_step[2];                // step of each work item (empty: none)
    std::vector<qtg::HotStep> hot[2];                 // packed per-step fields of the interpreter
    std::vector<qtg::ItemDesc> items[2];              // per-item descriptors (mixed form; empty: none)
    std::vector<uint32_t> level_meta[2];              // per level: max lane-group log2, compensated groups
    std::vector<ushort2> tables;                      // interpreter offset tables (empty: none)
    std::vector<uint64_t> leaf_off[2];
    uint64_t leaf_bytes[2] = {0, 0};
    uint64_t ws_bytes[2] = {0, 0};
    int n_steps = 0, n_levels = 0;
    int peak_rank = 0, max_step_out = 0, max_step_k = 0;
    int64_t flops = 0;
    bool grouped = false;
    void *dev[2] = {nullptr, nullptr};
    size_t dev_bytes[2] = {0, 0};
    // dev[prec] is published: readers on other contexts skip the owner's lock
    std::atomic<bool> dev_ready[2]{};
    // slicings made for a workspace budget (per precision: budget, slicing), freed with the plan
    std::vector<std::pair<uint64_t, qt_sliced *>> slicings[2];
};

struct qt_batch {
    explicit qt_batch(qt_ctx *c) : ctx(c) { qtg::ctx_retain(ctx); }
    ~qt_batch() { qtg::ctx_release(ctx); }
    qt_batch(const qt_batch &) = delete;
    qt_batch &operator=(const qt_batch &) = delete;
    qt_ctx *ctx = nullptr;
    std::vector<qt_plan *> plans;                     // per instance
    std::vector<std::vector<std::complex<double>>> leaves;   // per instance, complex128
    int prepared_prec = -1;
    bool dirty = true;
    // device state
    void *d_leaves = nullptr;
    uint64_t leaf_bytes = 0;
    std::vector<uint64_t> inst_leaf_off;
    void *d_inst = nullptr;
    void *d_values = nullptr;
    void *d_ws = nullptr;
    void *d_next = nullptr;                           // dynamic-schedule counter (null: round robin)
    uint32_t tile_bytes = 0;
    uint32_t header_steps = 1;                        // scale header entries per CTA (largest plan)
    uint64_t ws_stride = 0;
    bool ws_in_smem = false;                          // every instance's workspace fits shared memory
    uint32_t ws_smem_bytes = 0;                       // shared-memory workspace region per CTA
    uint32_t stage_bytes = 0;                         // shared memory for staged plan block + leaves
    qt_launch_policy policy{-1, -1, 0, 0, 0};          // defaults (qt_batch_set_launch_policy)
    int variant = 2;                                  // register budget of the interpreter (CTAs per SM)
    int grid = 0;
    void *h_leaves = nullptr;                         // pinned staging of the leaf image
    void *h_values = nullptr;                         // pinned values
    bool use_graph = false;
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t eval_graph = nullptr;             // qt_batch_evaluate: the grouped launch on zero-copy descriptors
    void *d_inst_eval = nullptr;                      // descriptors with host-mapped angles and values
    bool all_grouped = true;
    std::vector<int> stepwise;                        // instances run step by step
    std::vector<char> in_group;                       // instance runs in the grouped launch
    int64_t stepwise_macs = INT64_MAX;                // grouped plans above this run step by step
    // rotation angles applied on the device (mixed precision): pinned + device copies
    bool dev_rot = false;
    int64_t n_angles = 0;
    double *h_angles = nullptr;
    void *d_angles = nullptr;
    std::vector<int64_t> inst_angle_off;              // first angle of each instance
    std::vector<qtg::InstanceDesc> inst_desc;         // host copy of the descriptors
    std::vector<int> inst_index;                      // batch index of each descriptor
    cudaEvent_t angles_done = nullptr;                // the last angle upload has left h_angles
    // resident evaluation (qt_batch_use_resident)
    double res_idle = 0;                              // idle seconds before the engine leaves; 0: off
    cudaStream_t res_stream = nullptr;
    uint32_t *h_mail = nullptr;                       // pinned: [0] request number, [32 + j] done of descriptor j
    void *d_inst_res = nullptr;                       // descriptors on the mapped host angles and values
    uint32_t res_seq = 0;                             // the last request posted
    bool res_running = false;
    bool res_tagged = false;                          // requests post tagged angle words (h_tagged)
    uint64_t *h_tagged = nullptr;                     // pinned: (request << 32) | float bits, one per angle
    uint64_t res_starts = 0;                          // engine launches so far
};

namespace qtg {
qt_status lower_plan(qt_plan *p, const qtorch::Network &net);
void plan_collect_leaves(qt_plan *p, const qtorch::Network &net);
qt_status plan_finish(qt_plan *p, const qtorch::Network &net);
qt_status upload_plan(qt_plan *p, int prec);
void pack_leaves(const qt_plan *p, int prec, const std::complex<double> *src, char *dst);
// runs on `ctx` (its stream, allocator and lock), which may differ from the
// plan's own context: a server lane executes shared plans on its own stream
// Largest intermediate a plan run step by step may have: rank 15, 4^15 =
// 2^30 elements (8.6 GB in complex64).  The step kernels count tiles, runs
// and outputs in 32 bits and pack_tiles' grid caps a GEMM operand at 65,535
// row tiles, so a rank-16 tensor (2^32 elements) is beyond them; such a plan
// is rejected before any launch (the server refuses it at submission).
constexpr int kMaxStepwiseRank = 15;
qt_status execute_stepwise(qt_plan *p, qt_ctx *ctx, int prec, const std::complex<double> *leaves, double *value);
}  // namespace qtg
