/*
 * qtorch_gb300 — C ABI of the GB300 (sm_103a) contraction engine for
 * qTorch-style density-matrix tensor networks.
 *
 * Tensors follow qTorch's layout: every wire has dimension 4 (s = 2r + c of a
 * one-qubit density matrix), a rank-r tensor holds 4^r complex values and the
 * flat index is sum_i idx_i * 4^i (src/Node.h:112-113, 168-186).
 *
 * All entry points return a qt_status; none throws.  Errors map one to one onto
 * the reference's exception types (src/Exceptions.h:24-59).  A context owns one
 * CUDA stream and a caching device allocator; calls on one context are
 * serialised by an internal lock and may come from any thread.
 */
#ifndef QTORCH_GB300_H
#define QTORCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum qt_status {
    QT_OK = 0,
    QT_ERR_INVALID_ARGUMENT = 1,        /* a bad pointer, size or index map */
    QT_ERR_INVALID_FILE = 2,            /* InvalidFile (Exceptions.h:24) */
    QT_ERR_INVALID_FILE_FORMAT = 3,     /* InvalidFileFormat (Exceptions.h:28) */
    QT_ERR_CONTRACTION_FAILURE = 4,     /* ContractionFailure (Exceptions.h:36) */
    QT_ERR_INVALID_USER_SEQUENCE = 5,   /* InvalidUserContractionSequence (Exceptions.h:40) */
    QT_ERR_INVALID_FUNCTION_INPUT = 6,  /* InvalidFunctionInput (Exceptions.h:44) */
    QT_ERR_INVALID_CONTRACTION_METHOD = 7, /* InvalidContractionMethod (Exceptions.h:52) */
    QT_ERR_REFUSED = 8,                 /* ContractNodes returned nullptr (Network.h:719-723, 772-777) */
    QT_ERR_OUT_OF_MEMORY = 9,           /* device allocation or memory budget exceeded */
    QT_ERR_CUDA = 10,                   /* a CUDA runtime error; see qt_last_error */
    QT_ERR_DEADLINE = 11,               /* the context deadline expired (the reference's maxTime, Network.h:51) */
    QT_ERR_NO_DEVICE = 12,              /* no usable sm_103 device */
    QT_ERR_BUSY = 13                    /* admission refused: not enough free budget right now */
} qt_status;

typedef enum qt_dtype {
    QT_C128 = 0,   /* complex128: interleaved double (re, im) */
    QT_C64 = 1     /* complex64:  interleaved float (re, im) */
} qt_dtype;

typedef enum qt_precision {
    QT_PREC_FP64 = 0,   /* complex128 throughout, each product rounded as the reference's loop */
    QT_PREC_MIXED = 1   /* complex64 storage, FP32 accumulation, power-of-two scaling, compensated (twice-FP32) final reductions */
} qt_precision;

typedef struct qt_ctx qt_ctx;
typedef struct qt_tensor qt_tensor;
typedef struct qt_network qt_network;
typedef struct qt_plan qt_plan;
typedef struct qt_batch qt_batch;
typedef struct qt_server qt_server;

/* ---- context ---------------------------------------------------------- */

/* stream: a cudaStream_t to launch on, or NULL for a context-owned stream. */
qt_status qt_ctx_create(int device, void *stream, qt_ctx **out);
qt_status qt_ctx_destroy(qt_ctx *ctx);
qt_status qt_ctx_synchronize(qt_ctx *ctx);
const char *qt_status_string(qt_status s);
/* last error text of this context (thread-safe copy into buf). */
size_t qt_last_error(qt_ctx *ctx, char *buf, size_t cap);
/* Device memory budget for plans and requests (bytes, 0 = no limit). */
qt_status qt_ctx_set_memory_budget(qt_ctx *ctx, uint64_t bytes);
/* Cooperative deadline in seconds from now (<= 0 clears it).  Mirrors the
 * reference's totTimer/maxTime polling (Network.h:50-51, 899-910): long
 * contractions stop at the deadline and report QT_ERR_DEADLINE. */
qt_status qt_ctx_set_deadline(qt_ctx *ctx, double seconds_from_now);
/* Number of kernels this library launched on the context (for accounting). */
uint64_t qt_ctx_kernel_launches(const qt_ctx *ctx);
/* Contraction steps of this context that ran on the tcgen05 tensor-core GEMM. */
uint64_t qt_ctx_tensor_core_steps(const qt_ctx *ctx);
/* Contraction steps of this context that ran on the streaming kernel (a small
 * operand in shared memory, the large one read once by TMA bulk copies). */
uint64_t qt_ctx_stream_steps(const qt_ctx *ctx);
/* Test hook of the failure path (no reference counterpart): with mode 1 the
 * streaming kernel leaves the first tile of every CTA unissued, so its
 * pipeline waits -- bounded by `polls` polls (0: the normal limit) -- run out;
 * the kernel then waits for the copies it did issue, raises its error flag and
 * returns, and the call reports QT_ERR_CUDA ("TMA pipeline wait timed out")
 * with the context still usable.  mode 0 restores normal operation.  The
 * setting is per device and process. */
qt_status qt_debug_stream_fault(qt_ctx *ctx, int mode, uint32_t polls);
/* The same for the tcgen05 GEMM's pipeline (mode 1: the first k tile of every
 * CTA is never loaded; the step reports QT_ERR_CUDA "TMA pipeline wait timed
 * out") and for the grouped interpreter's staging of plan blocks and leaves
 * (mode 1: no staging copy is issued; batch calls report QT_ERR_CUDA "TMA
 * staging wait timed out").  Test use only; mode 0 restores normal operation. */
qt_status qt_debug_gemm_fault(qt_ctx *ctx, int mode, uint32_t polls);
qt_status qt_debug_staging_fault(qt_ctx *ctx, int mode, uint32_t polls);
/* The context's caching device allocator: bytes handed out, bytes cached for
 * reuse, and how many cudaMalloc calls it has made since the context was
 * created (any pointer may be NULL). */
qt_status qt_ctx_memory_stats(qt_ctx *ctx, uint64_t *bytes_in_use, uint64_t *bytes_cached,
                              uint64_t *device_allocations);

/* ---- tensors ---------------------------------------------------------- */

qt_status qt_tensor_create(qt_ctx *ctx, int rank, qt_dtype dtype, qt_tensor **out);  /* zero-filled */
qt_status qt_tensor_free(qt_ctx *ctx, qt_tensor *t);
qt_status qt_tensor_upload(qt_ctx *ctx, qt_tensor *t, const void *host, size_t bytes);
qt_status qt_tensor_download(qt_ctx *ctx, const qt_tensor *t, void *host, size_t bytes);
int qt_tensor_rank(const qt_tensor *t);
qt_dtype qt_tensor_dtype(const qt_tensor *t);
void *qt_tensor_device_ptr(const qt_tensor *t);

/* ---- the pairwise contraction (the drop-in for ContractIndices) --------
 *
 * Replaces Network::ContractIndices (src/Network.h:112-118, 876-971), called
 * from Network::ContractNodes (src/Network.h:837):
 *   C[c] = sum_k A[a(c,k)] * B[b(c,k)]
 * free_from_a[i], free_idx[i]  = toNotSumOn[i]: digit i of C is wire free_idx[i]
 *                                of A (free_from_a[i] != 0) or of B;
 * sum_a[j], sum_b[j]           = toSumOn[j]: wire sum_a[j] of A is summed
 *                                against wire sum_b[j] of B.
 * Summation runs over k in the reference's order (digit i of k <-> pair
 * n_sum-1-i), one output element per accumulator, so the QT_C128 result equals
 * the reference's bit for bit.  *c_out receives a new tensor of rank n_free.
 */
qt_status qt_contract_pair(qt_ctx *ctx, const qt_tensor *a, const qt_tensor *b,
                           int n_free, const uint8_t *free_from_a, const int32_t *free_idx,
                           int n_sum, const int32_t *sum_a, const int32_t *sum_b,
                           qt_tensor **c_out);

/* The same on caller-owned device buffers (complex128, flat base-4 layout).
 * c must hold 4^n_free elements; it is overwritten.  Asynchronous on the
 * context stream. */
qt_status qt_contract_pair_device(qt_ctx *ctx, const void *a, int rank_a, const void *b, int rank_b,
                                  int n_free, const uint8_t *free_from_a, const int32_t *free_idx,
                                  int n_sum, const int32_t *sum_a, const int32_t *sum_b, void *c);

/* Index permutation of a tensor (the reference forms the index map of
 * src/Network.h:912-916 per element inside ContractIndices; here a copy is a
 * kernel of its own): digit i of the output's flat index is digit perm[i] of
 * the input's, for a permutation perm of 0..rank-1.  The copy moves through
 * shared memory in tiles read along the input's contiguous runs and written
 * along the output's, so both sides are coalesced.  *out receives a new tensor
 * of the same rank and dtype.  QT_ERR_INVALID_ARGUMENT when perm is not a
 * permutation. */
qt_status qt_tensor_permute(qt_ctx *ctx, const qt_tensor *in, const int32_t *perm, qt_tensor **out);
/* The same on caller-owned device buffers of 4^rank elements of `dtype`,
 * 16-byte aligned (QT_ERR_INVALID_ARGUMENT otherwise); asynchronous on the
 * context stream.  in and out must not overlap. */
qt_status qt_permute_device(qt_ctx *ctx, const void *in, int rank, qt_dtype dtype, const int32_t *perm, void *out);

/* The same on host buffers: copies A and B in, contracts, copies C out (synchronous). */
qt_status qt_contract_pair_host(qt_ctx *ctx, const double *a, int rank_a, const double *b, int rank_b,
                                int n_free, const uint8_t *free_from_a, const int32_t *free_idx,
                                int n_sum, const int32_t *sum_a, const int32_t *sum_b, double *c);

/* ---- networks (Network / ContractionTools / LineGraph) ------------------ */

typedef enum qt_ordering {
    QT_ORDER_STOCHASTIC = 0,   /* ContractionTools::ParallelContract (ContractionTools.h:219-388), seeded */
    QT_ORDER_LINEGRAPH = 1,    /* LineGraph + min-fill elimination order (LineGraph.h:92-171, 357-376) */
    QT_ORDER_SEQUENCE = 2,     /* ContractGivenSequence (ContractionTools.h:392-411) */
    QT_ORDER_GREEDY = 3,       /* size-greedy pairwise merges, best of 4096 seeded tries (no reference
                                  counterpart: networks too large for min-fill) */
    QT_ORDER_AUTO = 4          /* QT_ORDER_GREEDY, or the line graph's min-fill walk where the line
                                  graph has <= 1500 wires and that walk is better */
} qt_ordering;

/* Network(qasm, measure) from text (Network.h:148-151, 246-304).  gate_dir
 * resolves relative def1/def2 paths (NULL = current directory).  With ctx ==
 * NULL the network is symbolic: it tracks ranks and wires only (for planning). */
qt_status qt_network_create(qt_ctx *ctx, const char *qasm_text, const char *measure_text,
                            const char *gate_dir, qt_network **out);
qt_status qt_network_create_from_files(qt_ctx *ctx, const char *qasm_path, const char *measure_path,
                                       qt_network **out);
qt_status qt_network_free(qt_network *net);
qt_status qt_network_reset(qt_network *net);                       /* Network::Reset (Network.h:154-171) */
int qt_network_num_qubits(const qt_network *net);
int qt_network_num_nodes(const qt_network *net);                   /* size of GetAllNodes() */
int qt_network_num_uncontracted(const qt_network *net);
int qt_network_node_rank(const qt_network *net, int node_id);
int qt_network_is_done(const qt_network *net);
/* ContractNodes(allNodes[a], allNodes[b], threshold) (Network.h:715-864).
 * *new_id = id of the new node, or -1 when the call returned nullptr. */
qt_status qt_network_contract_nodes(qt_network *net, int node_a, int node_b, int threshold, int *new_id);
/* ContractGivenSequence: pairs[2*i], pairs[2*i+1] index GetAllNodes(). */
qt_status qt_network_contract_sequence(qt_network *net, const int32_t *pairs, int n_pairs);
/* ContractUserDefinedSequenceOfWires (ContractionTools.h:155-214) from text "a b\n..." */
qt_status qt_network_contract_user_sequence(qt_network *net, const char *sequence_text);
/* Stochastic ordering with a fixed seed (the reference seeds from random_device). */
qt_status qt_network_contract_stochastic(qt_network *net, uint64_t seed);
/* Line-graph ordering: min-fill elimination over the line graph, then the LGContract walk. */
qt_status qt_network_contract_linegraph(qt_network *net);
/* LGContract over a caller-given 1-based wire order (the content of a qbb.out). */
qt_status qt_network_contract_wire_order(qt_network *net, const int32_t *order_1based, int n);
/* ReduceCircuit (Network.h:1015-1118). */
qt_status qt_network_reduce(qt_network *net);
qt_status qt_network_final_value(const qt_network *net, double *re_im);
int64_t qt_network_flops(const qt_network *net);                   /* getNumFloatOps (Network.h:91) */
/* The recorded mCreatedFrom pairs (the walk of preprocess.h:41-46); returns the count. */
int qt_network_created_from(const qt_network *net, int32_t *pairs, int cap_pairs);
/* Values of node `node_id` (complex128) if it still holds data; returns count or -1. */
int64_t qt_network_node_values(qt_network *net, int node_id, double *out, int64_t cap_complex);
/* Line-graph wire order chosen by the min-fill heuristic (1-based, qbb.out order). */
int qt_network_linegraph_order(qt_network *net, int32_t *order_1based, int cap);

/* Run an .inp script (src/leviParser.hpp:41-104, the flow of src/main.cpp:42-309):
 * parse the QASM and measurement files it names, ReduceCircuit, contract with
 * its contractmethod (linegraph-qbb | simple-stoch | user-defined; qbbonly /
 * readqbbresonly use output/qbb.out in QuickBB's format) and write its output
 * file.  ctx == NULL runs the bookkeeping only (value 0).  value: 2 doubles. */
qt_status qt_run_inp(qt_ctx *ctx, const char *inp_path, double *value, int64_t *flops);

/* ---- plans: an ordering lowered once, executed many times ---------------
 *
 * A plan is built by running the ordering over a symbolic copy of the network
 * (same bookkeeping as ContractNodes, no data) and recording every step.  The
 * leaves (gate / state / measurement tensors) are bound separately, so one
 * plan serves every parameter point of the same circuit structure.
 */
qt_status qt_plan_build(qt_ctx *ctx, const char *qasm_text, const char *measure_text, const char *gate_dir,
                        qt_ordering ordering, uint64_t seed, const int32_t *sequence_pairs, int n_pairs,
                        qt_plan **out);
/* preProcess (src/preprocess.h:28-52): the reference retries its stochastic
 * ordering up to 100 times and keeps the first sequence that finishes under a
 * time limit.  Here `tries` seeded stochastic orderings (seeds seed, seed + 1,
 * ...) run over a symbolic copy of the network and are scored by the rank of
 * their largest intermediate, then by complex MACs; the best becomes the plan
 * (recorded as a sequence).  max_macs > 0 stops at the first try of at most
 * that many MACs.  *chosen_seed (may be NULL) receives the winning seed, which
 * QT_ORDER_STOCHASTIC reproduces. */
qt_status qt_plan_build_search(qt_ctx *ctx, const char *qasm_text, const char *measure_text, const char *gate_dir,
                               uint64_t seed, int tries, int64_t max_macs, qt_plan **out, uint64_t *chosen_seed);
qt_status qt_plan_free(qt_plan *plan);
int qt_plan_num_steps(const qt_plan *plan);
/* Work items of the mixed form that carry a host-prepared descriptor (0: the
 * interpreter looks each item's step up instead; plans whose work-item steps
 * all have offset tables and at most 8192 items carry them). */
int64_t qt_plan_item_descriptors(const qt_plan *plan);
int qt_plan_num_leaves(const qt_plan *plan);
int qt_plan_peak_rank(const qt_plan *plan);
uint64_t qt_plan_workspace_bytes(const qt_plan *plan, qt_precision prec);
int64_t qt_plan_flops(const qt_plan *plan);                         /* sum of 4^(free+summed) */
/* Algorithmic bytes of one execution: sum over steps of the element size times
 * (4^rank_a + 4^rank_b + 4^rank_c) in the given precision's storage types. */
uint64_t qt_plan_algorithmic_bytes(const qt_plan *plan, qt_precision prec);
/* recorded node-id pairs (replayable through QT_ORDER_SEQUENCE / the oracle) */
int qt_plan_sequence(const qt_plan *plan, int32_t *pairs, int cap_pairs);
/* Leaf tensors of the plan's own circuit, complex128, concatenated in leaf order. */
uint64_t qt_plan_leaf_elems(const qt_plan *plan);
qt_status qt_plan_leaf_values(const qt_plan *plan, double *out, uint64_t cap_complex);
/* One network value (synchronous, host in / host out). */
qt_status qt_plan_execute(qt_ctx *ctx, qt_plan *plan, qt_precision prec, double *re_im);
/* Size of the device array that qt_plan_execute_static works in.  It is
 * reserved statically: every GPU that loads this library holds it until the
 * process exits. */
#define QT_STATIC_SCRATCH_BYTES (8u << 20)

/* One plan instance evaluated without allocating device memory (no reference
 * counterpart: qTorch has no device code).  It is meant for callers that cannot
 * call cudaMalloc -- code running under a framework that owns all device memory
 * (a custom call or operator whose allocator belongs to the host framework) and
 * latency-bound loops that must never pay cudaMalloc's implicit device
 * synchronisation.
 *   leaves_device: the plan's leaf tensors in device memory owned by the caller,
 *                  concatenated in leaf order (the order of qt_plan_leaf_values):
 *                  complex128 for QT_PREC_FP64, complex64 for QT_PREC_MIXED;
 *   value_device:  two doubles (re, im) in device memory owned by the caller.
 * The descriptors of the plan and its intermediates live in a static device
 * array of QT_STATIC_SCRATCH_BYTES; a plan that needs more (descriptors plus
 * workspace) is rejected with QT_ERR_OUT_OF_MEMORY, and a plan beyond the
 * grouped interpreter's limits with QT_ERR_INVALID_ARGUMENT.  The first call on
 * a device looks the array's device address up, so make it before any stream
 * capture.  Every call shares the one array and overwrites what the previous
 * call left there: calls that overlap on the GPU (other streams, other
 * contexts of the same device) race.
 * Stream order: the descriptors are copied from host memory and the kernel is
 * launched on the context's stream, without waiting for earlier work.  The
 * leaves must therefore be complete in that stream's order -- create the
 * context on the stream that writes them (qt_ctx_create's stream argument) or
 * synchronise that stream first -- and value_device may be read once the
 * context's stream has passed the launch. */
qt_status qt_plan_execute_static(qt_ctx *ctx, const qt_plan *plan, qt_precision prec, const void *leaves_device,
                                 double *value_device);
/* Parametrised rotation leaves (Rx, Ry, Rz, PHASE, CPHASE) of the plan, in leaf
 * order: their count, and the angles the plan's own circuit gives them. */
int qt_plan_num_rotations(const qt_plan *plan);
qt_status qt_plan_rotation_angles(const qt_plan *plan, double *angles, int cap);
/* The plan's schedule as the grouped interpreter runs it (no reference
 * counterpart), QT_STEP_INFO_FIELDS int32 per step in execution order:
 * dependency level, rank of A, rank of B, output rank, summed wires, lane-group
 * size, flags (bit 0/1: A/B is a leaf, bit 4: complex128 output), and 1 when the
 * step has offset tables.  Returns the number of steps, -1 on a bad argument. */
#define QT_STEP_INFO_FIELDS 8
int qt_plan_step_info(const qt_plan *plan, qt_precision prec, int32_t *out, int cap_steps);

/* ---- index slicing (no reference counterpart) ---------------------------
 *
 * A plan whose intermediates do not fit a workspace budget is split over the
 * values of up to max_cuts wires: each cut wire is removed from its two leaves
 * (the leaves keep the slice at one index), the plan's recorded sequence is
 * replayed on the cut network (a pair that shared only cut wires becomes an
 * outer product), and the value is the sum over all 4^cuts assignments -- the
 * network value is linear in every leaf.  Wires are cut greedily, the one
 * carried by the largest intermediates first, keeping every leaf and every
 * intermediate but the final one at rank >= 1, until the sliced plan's
 * workspace in `prec` is at most max_workspace_bytes (QT_ERR_OUT_OF_MEMORY
 * when max_cuts do not get there).  ctx may be NULL to inspect the slicing
 * only.  qt_sliced_execute sums the slices' values in assignment order
 * (complex128); instances above 2^24 complex MACs run step by step one at a
 * time, so the device holds one sliced workspace; more than 4096 slices run
 * in chunks of 4096 (one batch each, built per call). */
typedef struct qt_sliced qt_sliced;
qt_status qt_plan_slice(qt_ctx *ctx, const qt_plan *plan, qt_precision prec, uint64_t max_workspace_bytes,
                        int max_cuts, qt_sliced **out);
int qt_sliced_num_cuts(const qt_sliced *s);
qt_plan *qt_sliced_plan(const qt_sliced *s);   /* the plan of one slice (owned by s) */
qt_status qt_sliced_execute(qt_sliced *s, qt_precision prec, double *re_im);
/* The same for other values of the uncut plan's leaves (complex128, its leaf
 * order; NULL: its own), on ctx, every slice step by step one at a time. */
qt_status qt_sliced_execute_leaves(qt_ctx *ctx, const qt_sliced *s, qt_precision prec, const double *leaves,
                                   double *re_im);
qt_status qt_sliced_free(qt_sliced *s);

/* ---- batches: many plan instances in one persistent grouped launch ------ */

/* A batch holds instances (plan, leaf values).  Leaves are complex128 on the
 * host; the batch converts them to the execution precision on upload. */
qt_status qt_batch_create(qt_ctx *ctx, qt_batch **out);
qt_status qt_batch_free(qt_batch *b);
/* leaves = NULL uses the plan's own leaf values. Returns the instance index. */
qt_status qt_batch_add(qt_batch *b, qt_plan *plan, const double *leaves, int *index);
int qt_batch_size(const qt_batch *b);
/* Upload leaves, launch, download values (synchronous). values: 2 doubles per instance. */
qt_status qt_batch_execute(qt_batch *b, qt_precision prec, double *values);
/* Device-resident variants for timing: prepare uploads everything once, run
 * launches only (async on the context stream), fetch copies values back. */
qt_status qt_batch_prepare(qt_batch *b, qt_precision prec);
qt_status qt_batch_run(qt_batch *b);
qt_status qt_batch_fetch(qt_batch *b, double *values);
/* Replace the leaf values of instance i (host complex128) for the next run. */
qt_status qt_batch_set_leaves(qt_batch *b, int index, const double *leaves);
/* New angles for the rotation leaves of every instance, concatenated in
 * instance order (qt_plan_num_rotations angles per instance).  The leaf tensors
 * are rebuilt on the host with the reference's expressions (angles narrowed to
 * float as its parser does) and go to the device with the next upload.  This is
 * how an optimiser moves a batch of QAOA terms to a new (gamma, beta) point
 * without re-planning. */
qt_status qt_batch_set_rotations(qt_batch *b, const double *angles, int64_t n_angles);
/* The same, with the gate tensors built on the device (no reference
 * counterpart): only the angles travel (8 bytes each, one asynchronous copy
 * from pinned memory on the context stream), and every following qt_batch_run
 * rebuilds the rotation leaves inside the interpreter before contracting --
 * Rx/Ry/Rz narrowed to float like the reference's parser, the trigonometry in
 * FP32 (entries within a few ulp of the host-built complex64 leaves).  Batches prepared for QT_PREC_MIXED
 * only; instances run step by step get their leaves on the host.  A later
 * qt_batch_set_rotations or qt_batch_set_leaves switches back to host leaves. */
qt_status qt_batch_set_rotations_device(qt_batch *b, const double *angles, int64_t n_angles);
/* One evaluation of a prepared batch at new angles in a single call (the inner
 * loop of a QAOA optimiser): qt_batch_set_rotations_device (angles may be NULL
 * to keep the current leaves), qt_batch_run, qt_batch_fetch.  From the second
 * call on a mixed batch with graphs enabled, the interpreter reads the angles
 * from and writes the values to pinned host memory directly, and one captured
 * graph launch plus a stream synchronisation make the whole evaluation. */
qt_status qt_batch_evaluate(qt_batch *b, const double *angles, int64_t n_angles, double *values);
/* Upload all leaf values again from the host copies (async; part of an end-to-end step). */
qt_status qt_batch_upload(qt_batch *b);
/* Capture qt_batch_run into a CUDA graph and replay it (0 disables). */
qt_status qt_batch_use_graph(qt_batch *b, int enable);
/* Resident evaluation (no reference counterpart; GB300's coherent CPU-GPU
 * link): with idle_seconds > 0, qt_batch_evaluate with angles keeps one CTA per
 * instance on the GPU between calls, on a stream of the batch's own.  The plan
 * blocks and leaf images stay staged in shared memory; a call writes the angles
 * and a request number into pinned host memory, every CTA rebuilds its
 * rotation leaves, contracts and writes its value and a done flag there, and
 * the call returns when all flags are set -- no launch, copy or stream
 * synchronisation per call.  The engine leaves after idle_seconds without a
 * request and starts again on the next one.  Any other use of the batch
 * (run, upload, new leaves or rotations, a policy change, prepare, free) stops
 * it first.  While it runs the GPU is not idle, so device-wide synchronisation
 * (cudaDeviceSynchronize, cudaFree) waits up to idle_seconds.  Needs a mixed
 * batch whose instances all run in the grouped launch with one CTA each
 * (QT_ERR_INVALID_ARGUMENT otherwise).  idle_seconds <= 0 turns it off.
 * Values are bit-identical with qt_batch_evaluate's other paths. */
qt_status qt_batch_use_resident(qt_batch *b, double idle_seconds);
/* How many times the resident engine was launched (starts after idle exits included). */
uint64_t qt_batch_resident_starts(const qt_batch *b);
uint64_t qt_batch_h2d_bytes(const qt_batch *b);
uint64_t qt_batch_d2h_bytes(const qt_batch *b);
/* kernels launched by one qt_batch_run */
int qt_batch_launches_per_run(const qt_batch *b);

/* Launch policy of a batch's grouped launch (no reference counterpart).  Each
 * interpreter CTA holds, in shared memory, the workspace of instances whose
 * workspace is at most ws_smem_cap bytes (larger ones use a global slab) and a
 * staged copy of the plan block + leaf image of instances whose copy is at most
 * stage_cap bytes (larger ones are read in place).  Larger regions mean fewer
 * CTAs per SM.  Negative caps take the defaults (32 KiB; 64 KiB, 52 KiB when an
 * instance has CTA-tiled steps -- 144 KiB / 128 KiB for the wide variant; 16
 * KiB and no staging when the instances outnumber two CTAs per SM), 0 turns a
 * region off.  ctas_per_sm = 0 runs as
 * many CTAs as fit; static_schedule = 1 replaces the longest-first dynamic
 * schedule (used when there are more instances than CTAs) by a round robin in
 * batch order.  kernel_ctas picks the interpreter's register budget: the
 * variant compiled for 2 (128 registers a thread), 3 (80), 4 (64) or 5 (48)
 * resident CTAs per SM -- fewer registers, more warps to hide latency, some
 * spills -- or 1, the wide variant: 512 threads with 128 registers, one CTA
 * per SM, for a few instances whose levels then take half the rounds; 0 takes
 * 1 when there are no more instances than SMs, 4 when they outnumber two CTAs
 * per SM, else 2.
 * The policy changes where data sits, which CTA runs an instance and how
 * registers are allocated, never the arithmetic: values are bit-identical
 * under every policy. */
typedef struct qt_launch_policy {
    int32_t ws_smem_cap;
    int32_t stage_cap;
    int32_t ctas_per_sm;
    int32_t static_schedule;
    int32_t kernel_ctas;
} qt_launch_policy;
/* Set the policy; a prepared batch is reconfigured in place (leaves and plan
 * blocks stay on the device). */
qt_status qt_batch_set_launch_policy(qt_batch *b, const qt_launch_policy *policy);
qt_status qt_batch_get_launch_policy(const qt_batch *b, qt_launch_policy *policy);
/* What the policy resolved to for the prepared batch. */
typedef struct qt_launch_info {
    int32_t grid;              /* CTAs of the grouped launch (0: none) */
    int32_t n_grouped;         /* instances in the grouped launch */
    int32_t n_stepwise;        /* instances run step by step on the whole GPU */
    int32_t dynamic_schedule;  /* 1: longest-first dynamic schedule */
    int32_t n_ws_smem;         /* instances whose workspace is in shared memory */
    int32_t n_staged;          /* instances staged in shared memory */
    uint32_t smem_bytes;       /* dynamic shared memory of a CTA */
    uint32_t ws_smem_bytes;    /*   of which workspace region */
    uint32_t stage_bytes;      /*   of which staging region */
    uint32_t tile_bytes;       /*   of which CTA-tile buffers */
    uint64_t ws_slab_bytes;    /* global workspace slab, all CTAs */
    int32_t kernel_ctas;       /* register-budget variant of the interpreter */
    int32_t pad;
} qt_launch_info;
qt_status qt_batch_launch_info(const qt_batch *b, qt_launch_info *info);
/* Autotuner: times the prepared batch's grouped launch (CUDA events on the
 * context stream, one untimed launch then the median of `reps`, more for
 * launches shorter than a few hundred microseconds) under candidate
 * policies -- register budget x workspace cap x staging cap as a grid (they
 * trade against each other for CTAs per SM), then CTAs per SM and the
 * schedule one at a time -- and keeps the fastest.  Candidates that resolve to
 * a configuration already timed, or whose shared memory leaves fewer CTAs per
 * SM than their register budget when instances outnumber CTAs, are skipped;
 * the search takes no new candidate after about three seconds.  The chosen policy and its time per launch (microseconds) are returned when the
 * pointers are non-null.  Runs the batch several times; the values it leaves
 * are those of the current leaves. */
qt_status qt_batch_autotune(qt_batch *b, int reps, qt_launch_policy *chosen, double *best_us);

/* ---- QAOA MaxCut term generator (src/maxcut.h:31-233, maxcut.cpp:166-190) --- */

/* Light-cone QASM + measurement text of edge `edge` of a .dgf graph, as the
 * reference writes it (angles with 6 significant digits).  Returns the number
 * of bytes needed (including the NUL); text is truncated to cap. */
int64_t qt_qaoa_term_text(const char *dgf_text, int p, const double *betas_gammas, int edge,
                          char *qasm_out, int64_t qasm_cap, char *measure_out, int64_t measure_cap);
int qt_qaoa_num_edges(const char *dgf_text);
/* The whole MaxCut QAOA circuit of a graph (every qubit and edge), as
 * maxcutGetFinalString writes it (src/maxcut.cpp:52-56). */
int64_t qt_qaoa_circuit_text(const char *dgf_text, int p, const double *betas_gammas, char *qasm_out, int64_t cap);
/* Final-cut decoding (maxcutGetFinalString, src/maxcut.cpp:29-140): qubit by
 * qubit, the probability that it reads 0 given the bits chosen so far
 * (measurement leaves |0><0| / |1><1| / trace on one plan of the whole
 * circuit), the likelier bit chosen; an exact tie takes a coin from
 * std::mt19937(seed) (the reference: rand() seeded by the clock).  bits: one
 * 0/1 per vertex; cut_edges: edges whose ends differ; prob: the probability
 * of the chosen string; marginals (may be NULL, cap_bits entries): the
 * contracted value of each query, P(chosen bits before i, bit i = 0).
 * ordering: QT_ORDER_LINEGRAPH or QT_ORDER_STOCHASTIC (seeded). */
qt_status qt_maxcut_final_string(qt_ctx *ctx, const char *dgf_text, int p, const double *betas_gammas,
                                 qt_precision prec, qt_ordering ordering, uint64_t seed, int32_t *bits,
                                 int cap_bits, int *n_bits, int *cut_edges, double *prob, double *marginals);
/* Seeded x-regular random graph in .dgf text (the XregGraphGen algorithm with
 * std::mt19937(seed), retried until every vertex reaches degree x). */
int64_t qt_random_regular_graph(int num_nodes, int degree, uint64_t seed, char *dgf_out, int64_t cap);

/* ---- serving: continuous batching of contraction requests --------------- */

/* A server admits requests while their plan's workspace fits the context's
 * memory budget and a slot is free, and runs every admitted request in grouped
 * launches; requests that arrive while others run join the next launch.  A
 * request whose workspace exceeds the whole budget is sliced at submission
 * (qt_plan_slice, up to 16 cut wires, cached in the plan) so that one slice
 * fits, and runs alone, slice by slice (in chunks of 4096 slices);
 * QT_ERR_OUT_OF_MEMORY when no such slicing exists.  With a work cap
 * (qt_server_set_max_macs) a request whose complex MACs -- over all its slices
 * -- exceed the cap is refused at submission with QT_ERR_REFUSED, and so is one
 * whose plan (or slice) has an intermediate above rank 15 (4^15 elements, the
 * largest the step-by-step kernels take; qt_plan_execute reports such a plan as
 * QT_ERR_INVALID_FUNCTION_INPUT). */
qt_status qt_server_create(qt_ctx *ctx, int max_inflight, qt_precision prec, qt_server **out);
qt_status qt_server_free(qt_server *s);
/* The work cap of one request in complex MACs (0: none, the default). */
qt_status qt_server_set_max_macs(qt_server *s, int64_t max_macs);
/* Submissions refused so far (work cap, rank limit, budget without a fitting slicing). */
int64_t qt_server_refused(qt_server *s);
/* Heavy requests that ran out of device memory beside others and were run
 * again alone (each at most twice; the admission budget counts plans'
 * workspaces, not the blocks the lanes' allocators keep). */
int64_t qt_server_oom_retries(qt_server *s);
/* Submit (non-blocking).  *ticket identifies the request. */
qt_status qt_server_submit(qt_server *s, qt_plan *plan, const double *leaves, int64_t *ticket);
/* Poll: 1 = done (value written), 0 = pending, <0 = error (status negated). */
int qt_server_poll(qt_server *s, int64_t ticket, double *re_im, double *latency_s);
/* The same, and where the latency went: seconds from submission to admission
 * into a wave, and the lane (0: the light lane) that ran it. */
int qt_server_poll_detail(qt_server *s, int64_t ticket, double *re_im, double *latency_s, double *queued_s,
                          int *lane);
/* Block until every submitted request has finished. */
qt_status qt_server_drain(qt_server *s);
/* p50/p99 latency in seconds and completed count since creation. */
qt_status qt_server_stats(qt_server *s, double *p50, double *p99, int64_t *completed, int64_t *launches);
/* Waves run so far, the requests they carried, and the lane time they took
 * (building the batch, launching, reading values back), summed over lanes. */
qt_status qt_server_wave_stats(qt_server *s, int64_t *waves, int64_t *requests, double *lane_seconds);

#ifdef __cplusplus
}
#endif
#endif
