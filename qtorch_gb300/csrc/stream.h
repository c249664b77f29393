// Streaming kernel for complex64 contraction steps with one small operand
// (stream.cu).  These are the large steps of the QAOA light-cone networks
// under stochastic orderings and of the serving heavy tail: a rank 12-14
// tensor met by a gate-sized one.  They are bound by HBM bandwidth, so the
// kernel reads the large operand L once in contiguous runs (TMA bulk copies)
// and writes the output once in contiguous runs; the small operand S lives in
// shared memory.
#pragma once
#include <cuda_runtime.h>

#include "engine.cuh"
#include "scale.cuh"

namespace qtg {

// Work decomposition over L's wires (base-4 digits):
//   wires 0-3            the thread's own digits: thread t of the CTA reads
//                        element t of every 256-element run (conflict-free)
//   "outer" free wires   (free wires >= 4) the lowest `go` of them are looped
//                        over inside a tile (g); the rest number the work items
//   summed wires >= 4    the lowest `ho` of them are looped over inside a tile
//                        (h); the rest number the chunks of a work item
// A tile is (wires 0-3) x g x h: 4^(4 + go + ho) <= kStreamMaxTile elements,
// copied as runs along L's lowest in-tile wires.  A thread keeps one sum per
// (g, S-free index) in registers across the chunks of a work item; the summed
// digits among wires 0-3 are then reduced by warp shuffles (wires 0 and 1
// lie within a warp) or through shared memory (wires 2 and 3), and the sums
// are written straight to C.
constexpr int kStreamMaxSmallRank = 6;       // S holds at most 4^6 elements (32 KB)
constexpr uint32_t kStreamMaxTile = 4096;    // elements of one L tile (32 KB)
constexpr uint32_t kStreamMaxStage = 16;     // g x S-free sums a thread keeps in registers
constexpr uint32_t kStreamMaxOut = 4096;     // staged outputs of one pass (32 KB)
constexpr int kStreamThreads = 256;          // = 4^4 consumer threads: one per combination of L's wires 0-3
constexpr int kStreamConsumerWarps = kStreamThreads / 32;
constexpr int kStreamBlock = kStreamThreads + 32;   // the consumers and one producer warp
constexpr int kStreamStages = 3;             // tiles in flight per CTA
constexpr int kStreamMaxLoop = 6;            // digits looped over in a tile or chunk

struct StreamStep {
    const float2 *L;
    const float2 *S;
    float2 *C;
    StepScaleRef sc;
    int *error_flag;               // set when a TMA wait timed out (zero on entry)
    uint32_t n_items;              // work items: combinations of the outer wires not looped in a tile
    uint32_t n_chunks;             // tiles per work item: combinations of the summed wires >= 4 not in a tile
    uint32_t run_elems;            // elements of one bulk copy (4^(lowest in-tile wires in a row))
    uint32_t n_runs;               // bulk copies per tile
    uint32_t s_elems;              // 4^rank(S)
    uint32_t s_store;              // elements of S's shared-memory image (blocks with padding)
    // S's image: the in-pass free indices of S are each block's elements, in
    // order (so a thread's NSF values for one element lie side by side and load
    // as 16-byte pairs), blocks NSF + 2 elements apart (NSF > 1; the pad turns
    // the lanes' different blocks onto different banks), S's other wires number
    // the blocks.  s_unit[w]: image offset of one step of S wire w
    uint32_t s_unit[kStreamMaxSmallRank];
    uint32_t nsf;                  // free wires of S
    uint32_t nsfp;                 // of which one pass covers (NSFP = 4^nsfp sums per thread and g)
    uint32_t n_pass;               // passes over a tile: combinations of S's free wires beyond nsfp
    uint32_t go, ho;               // outer / summed digits looped in a tile
    uint32_t n_item_d, n_chunk_d;  // digits of the work-item and chunk indices
    uint32_t n_run_d;              // in-tile digits above the run (bulk-copy index digits)
    uint32_t n_dout, n_klo;        // output digits of a pass; summed wires among 0-3
    uint32_t klo_mode;             // 0: no summed wire among 0-3, 1: only wires 0/1 (shuffles), 2: wires 2/3 too
    uint32_t staged;               // 1: outputs go through shared memory (summed wires 2/3), 0: stored
                                   // by the owning lanes
    uint32_t out_run;              // low staged digits that are C's digits 0, 1, ... in order
    uint32_t smem_bytes;
    uint32_t l_is_b;               // the large operand is B (else A)
    // work item digit j: L wire and C digit
    uint8_t item_lw[kMaxWires], item_cd[kMaxWires];
    // chunk digit j: L wire and S wire of the summed pair
    uint8_t chunk_lw[kMaxWires], chunk_sw[kMaxWires];
    // g digit j: tile-local digit and C digit; h digit j: tile-local digit and S wire
    uint8_t g_pos[kStreamMaxLoop], g_cd[kStreamMaxLoop];
    uint8_t h_pos[kStreamMaxLoop], h_sw[kStreamMaxLoop];
    // bulk copy index digit j: L wire
    uint8_t run_lw[kStreamMaxLoop];
    // wires 0-3 of L: 1 when summed, then the S wire it is summed with (else its C digit)
    uint8_t lo_summed[4], lo_other[4];
    // S-free digit j: S wire and C digit
    uint8_t sf_w[kStreamMaxSmallRank], sf_cd[kStreamMaxSmallRank];
    // staged outputs of a pass, digits in ascending C order: C digit of staged digit r,
    // and the staged digit of each free wire among 0-3, g digit and in-pass S-free digit
    uint8_t dout_cd[kMaxWires];
    uint8_t lo_rank[4], g_rank[kStreamMaxLoop], sf_rank[kStreamMaxSmallRank];
};

// Test hook of the failure path: mode 1 makes every CTA's first tile never
// arrive, so the pipeline's waits run out after `polls` polls (0: the normal
// limit) and the launch reports a timeout; mode 0 restores normal operation.
cudaError_t stream_set_fault(int mode, uint32_t polls);

// Plans the step (false: not a shape this kernel takes).
bool stream_plan(const StepDesc &d, StreamStep &p);
// Launches it on L = A or B as stream_plan chose (p.L, p.S, p.C filled here).
cudaError_t launch_stream(StreamStep &p, const StepDesc &d, const float2 *A, const float2 *B, float2 *C,
                          const StepScaleRef &sc, int *error_flag, cudaStream_t stream);

}  // namespace qtg
