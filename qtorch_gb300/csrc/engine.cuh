// Device-side data structures shared by the host planner and the kernels.
//
// A contraction step computes C[c] = sum_k A[a(c,k)] * B[b(c,k)] (the
// reference's ContractIndices, src/Network.h:876-971).  Digit i of C's flat
// index c is wire cA[i] of A or wire cB[i] of B (the other entry is kNoWire),
// as toNotSumOn says; ContractNodes lists A's free wires first
// (src/Network.h:738-769).  So
//   a(c,k) = sum_{i: cA[i] set} digit_i(c) 4^cA[i] + scatter(k, posAs)
//   b(c,k) = sum_{i: cB[i] set} digit_i(c) 4^cB[i] + scatter(k, posBs)
// where scatter(x, pos) places base-4 digit i of x at wire pos[i].  posAs/posBs
// are stored in the reference's inner-loop digit order (digit i of k <-> pair
// nSum-1-i, Network.h:912-916) so that k itself walks the reference's order.
#pragma once
#include <vector_types.h>

#include <cstdint>

#include "scale.cuh"

namespace qtg {

constexpr int kMaxWires = 24;      // rank limit of one operand (4^24 elements is far beyond HBM)
constexpr uint8_t kNoWire = 0xff;
constexpr int kPlanThreads = 256;              // threads of one interpreter CTA
// threads of the wide interpreter variant: one CTA of 512 threads per SM (the
// whole register file at 128 registers a thread) for launches with at most one
// instance per SM, where a level's work items then take half the rounds
constexpr int kPlanThreadsWide = 512;
__host__ __device__ constexpr int plan_threads(int min_ctas) { return min_ctas == 1 ? kPlanThreadsWide : kPlanThreads; }
constexpr int kPlanMaxSteps = 1024;            // steps of a plan the interpreter takes
// per-step scale bookkeeping in shared memory: 8 bytes a step, for as many
// steps as the largest plan of a launch has (rounded up to 128 bytes)
inline __host__ __device__ uint32_t plan_header_bytes(uint32_t steps) { return (8u * steps + 127u) / 128u * 128u; }

enum StepFlags : uint32_t {
    kALeaf = 1u << 0,        // A is read from the leaf buffer (else workspace)
    kBLeaf = 1u << 1,
    kAF64 = 1u << 2,         // A stored as complex128 (FP64 plans; mixed plans read complex64 copies)
    kBF64 = 1u << 3,
    kCF64 = 1u << 4,         // C stored as complex128; mixed plans accumulate it with compensated FP32 (Dot2)
    kOutRank0 = 1u << 5,     // C has rank 0: it takes part in the final-value rule
    kBothRank0 = 1u << 6,    // A and B both rank 0 (Network.h:963)
    kCtaTiled = 1u << 7,     // interpreter: the whole CTA runs this step as a tiled product
};

// CTA-wide tiled steps: C (M x N, flat c = m + M n, M = 4^fA, N = 4^fB) =
// sum_k A~(m, k) B~(k, n).  Tiles of at most kCtaTileDim x kCtaTileDim outputs, the
// summed range in chunks of kCtaTileChunk (mixed) or kCtaTileChunk / 2 (FP64) staged
// in shared memory, 16 x 16 threads with up to 4 x 4 outputs each.
constexpr int kCtaTileDim = 64;
constexpr int kCtaTileChunk = 16;
constexpr uint32_t kCtaTileBytes = 2u * kCtaTileChunk * kCtaTileDim * 8u + 2u * kCtaTileDim * 4u;

struct StepDesc {
    int64_t a_off;           // byte offset into the leaf buffer or the workspace
    int64_t b_off;
    int64_t c_off;           // byte offset into the workspace
    int32_t a_step;          // step that produced A (-1 for a leaf): its scale exponent applies
    int32_t b_step;
    uint32_t flags;
    uint8_t rA, rB, nFree, nSum, fA, fB;
    uint8_t group;               // interpreter: lanes that share one output's k loop (power of two)
    uint8_t pad1;
    uint8_t cA[kMaxWires];       // C digit -> A wire (kNoWire if the digit belongs to B)
    uint8_t cB[kMaxWires];       // C digit -> B wire (kNoWire if the digit belongs to A)
    uint8_t posAs[kMaxWires];
    uint8_t posBs[kMaxWires];
    uint32_t item_start;         // interpreter: first work item of this step inside its level
    uint32_t tab_off;            // interpreter: first entry of this step's offset tables (kNoTable: none)
    uint32_t pad2;
};

constexpr uint32_t kNoTable = 0xffffffffu;

// A dependency level's small contractions, launched together when a plan runs
// step by step (a kernel parameter: no copy).
constexpr int kPairBatchMax = 32;
constexpr int kPairBatchMaxLog2Macs = 22;   // steps of at most 2^22 complex MACs
struct PairJob {
    StepDesc d;
    const void *A;
    const void *B;
    void *C;
    StepScaleRef sc;             // complex64 jobs: the step's scale words (scale.cuh)
    uint64_t n_out, K;
    uint32_t block_begin, pad;
};
struct PairBatch {
    PairJob job[kPairBatchMax];
    uint32_t n_jobs, pad;
};
// passed by value as a kernel parameter (limit 32764 bytes)
static_assert(sizeof(PairBatch) <= 32000, "PairBatch exceeds the kernel-parameter limit");
static_assert(sizeof(StepDesc) % 8 == 0, "StepDesc alignment");

// The fields a work item reads, packed into 32 bytes (two 16-byte loads):
// the interpreter's per-item path reads these instead of the 152-byte StepDesc.
struct HotStep {
    uint32_t a_off, b_off, c_off;   // byte offsets (leaf buffer or workspace)
    uint32_t tab_off;               // offset tables (kNoTable: none)
    uint32_t item_start;            // first work item inside the level
    int16_t a_step, b_step;         // producers (-1: a leaf)
    uint8_t group_log2, nFree, nSum, flags;   // flags: the low 8 bits of StepFlags
    uint32_t pad;
};
static_assert(sizeof(HotStep) == 32, "HotStep layout");

// One work item of the mixed form, prepared on the host (plans whose work-item
// steps all have offset tables): the item's operand and output addresses are
// final, so the interpreter reads one 16-byte descriptor instead of looking up
// its step, unpacking the step's fields and reading the output's offsets.
//   a, b  byte offsets of the item's first operand elements (leaf image or workspace)
//   c     byte offset of its output element in the workspace
//   meta  bits 0-15 first k-offset table entry, 16-18 lane-group log2, 19-22
//         summed wires, 23/24 A/B in the leaf image, 25 compensated output
//         (complex128 + complex64 copy), 26 a real output (0: alignment gap),
//         27-30 the complex64 copy's distance from c in 8-byte units
struct ItemDesc {
    uint32_t a, b, c, meta;
};
static_assert(sizeof(ItemDesc) == 16, "ItemDesc layout");
constexpr uint32_t kItemLeafA = 1u << 23, kItemLeafB = 1u << 24, kItemF64 = 1u << 25, kItemValid = 1u << 26;

// One executable plan in device memory.
struct PlanDesc {
    const StepDesc *steps;       // sorted by level
    const int32_t *level_start;  // n_levels + 1 entries
    const int32_t *rank0_steps;  // steps with a rank-0 output, in contraction (sequence) order
    const uint32_t *level_items; // work items of each level (n_levels entries)
    // Offset tables of steps whose operands have at most 4^8 elements: for step s,
    // tab[tab_off + c] = (A offset, B offset) of output c (n_out entries), then
    // tab[tab_off + n_out + k] = (A offset, B offset) of summed index k (K entries).
    const ushort2 *tables;
    const int32_t *level_cta;    // first CTA-tiled step of each level (tiled steps close their level)
    const uint2 *rotations;      // rotation leaves: (byte offset in the leaf image, RotationKind)
    // step of every work item (relative to its level's first step), levels
    // concatenated; null when the plan has too many items (binary search then)
    const uint8_t *item_step;
    const HotStep *hot;          // per-step packed fields, same order as steps
    // per level: bits 0-7 the largest lane-group log2 of its work items, bit 8
    // set when a compensated (FP64-class) step of it uses lane groups
    const uint32_t *level_meta;
    // per work item, levels concatenated (mixed form; null: look items up)
    const ItemDesc *items;
    int32_t n_steps;
    int32_t n_levels;
    int32_t n_rank0;
    int32_t n_rot;
};

// Parametrised leaves the interpreter can rebuild from an angle on the device
// (complex64 leaves of mixed plans only).
enum RotationKind : uint32_t { kRotRx = 0, kRotRy = 1, kRotRz = 2, kRotCPhase = 3 };

// One instance of a batch: a plan with its own leaves.  Intermediates live in
// the workspace of the CTA that runs the instance.
struct InstanceDesc {
    const PlanDesc *plan;        // device pointer to the plan block (PlanDesc and its arrays)
    const char *leaves;          // leaf buffer of this instance (complex128, or complex64 in mixed mode)
    double *value;               // 2 doubles out
    uint32_t plan_bytes;         // bytes of the plan block (multiple of 16) when it may be staged, else 0
    uint32_t leaf_bytes;         // bytes of the leaf image (multiple of 16)
    uint32_t ws_bytes;           // workspace this instance needs
    uint32_t n_steps;            // steps of the plan (the scale header is cleared before the plan arrives)
    const double *angles;        // rotation angles to build on the device (null: leaves as uploaded)
};

// Parameters of one interpreter launch.  Shared memory of a CTA: the scale
// header, a workspace region of ws_smem_bytes, a staging region of stage_bytes.
// An instance whose workspace or plan block + leaves do not fit there uses the
// CTA's global workspace slab or reads in place.
// The value an instance reports when its staging copies did not arrive in
// time (a NaN with this payload; the host turns it into an error status).
constexpr uint64_t kStagingTimeoutBits = 0x7ff8dead5ca1ab1eull;

struct PlanLaunch {
    const InstanceDesc *instances;
    int n_instances;
    uint32_t ws_smem_bytes;      // shared-memory workspace region (0: none)
    char *ws_base;               // global workspace: ws_base + blockIdx.x * ws_stride
    uint64_t ws_stride;
    uint32_t stage_bytes;        // shared memory for a staged plan block + leaf image (0: none)
    uint32_t tile_bytes;         // shared memory for CTA-tiled steps (0: no instance has one)
    uint32_t *next;              // dynamic schedule: instance counter, zero at launch (null: round robin)
    uint32_t header_steps;       // steps of the largest plan of the launch (scale header size)
    uint32_t pad2;
};

// Resident evaluation: one CTA per instance stays on the GPU between
// evaluations and serves requests posted in pinned host memory (read and
// written over the coherent CPU-GPU link): the host writes the angles, then
// the request number to *seq; each CTA rebuilds its rotation leaves, contracts,
// writes the value and then its done[] slot.  Plan blocks and leaf images stay
// staged in shared memory across requests.
constexpr uint32_t kResidentStop = 0xffffffffu;   // *seq value that makes the engine leave
constexpr uint32_t kResidentLeft = 0xfffffffeu;   // done[] value of a CTA that left (idle, or staging failed)
struct ResidentLaunch {
    PlanLaunch lp;               // instance i on CTA i; angles and values point to mapped host memory
    const uint32_t *seq;         // mapped host: number of the latest request
    uint32_t *done;              // mapped host, one per instance: the last request it finished
    uint32_t first_seq;          // requests up to this number are served already
    uint32_t idle_polls;         // polls (about a microsecond apart) without a request before leaving
    uint32_t tagged;             // 1: each instance's angles are 64-bit words, (request << 32) | the
                                 // angle narrowed to float, so the poll that sees the request also
                                 // brings its angles (instances with at most a CTA's threads of angles)
    uint32_t pad;
};

// The request after `last` (the host's numbering skips 0 and the two reserved
// values kResidentLeft, kResidentStop).
__host__ __device__ inline uint32_t resident_next_request(uint32_t last) {
    const uint32_t n = last + 1u;
    return (n == 0u || n >= kResidentLeft) ? 1u : n;
}

__host__ __device__ inline uint64_t scatter_digits(uint64_t x, const uint8_t *pos, int n) {
    uint64_t off = 0;
    for (int i = 0; i < n; i++) off += ((x >> (2 * i)) & 3ull) << (2 * pos[i]);
    return off;
}

// Offsets of output element c inside A and B.
__host__ __device__ inline void scatter_c(uint64_t c, const StepDesc &d, uint64_t &oa, uint64_t &ob) {
    oa = 0;
    ob = 0;
    for (int i = 0; i < d.nFree; i++) {
        const uint64_t dig = (c >> (2 * i)) & 3ull;
        if (d.cA[i] != kNoWire) oa += dig << (2 * d.cA[i]);
        else ob += dig << (2 * d.cB[i]);
    }
}

}  // namespace qtg
