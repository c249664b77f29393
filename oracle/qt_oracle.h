/*
 * qt_oracle — TEST INFRASTRUCTURE, NOT THE PRODUCT.
 *
 * A plain-C CPU restatement of qTorch's contraction path, used only as the
 * checker by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg.
 * The shipped engine never links or calls it.
 *
 * Pinned against the unmodified reference (oracle/_ref/qt_ref_harness built
 * from the reference headers by oracle/Makefile) through the JSON fixtures under tests/golden:
 * gate tensors, single ContractIndices calls and whole-network replays are
 * compared bit for bit.
 *
 * What it restates (reference file:line):
 *   qto_contract_indices     src/Network.h:876-971  (sequential MAC loop, same digit order,
 *                                                    same complex rounding; built with
 *                                                    -ffp-contract=off)
 *   qto_net_parse            src/Network.h:246-304, 326-707, 177-240, 976-992
 *   qto_net_contract         src/Network.h:715-864  (wire matching, free-index order,
 *                                                    refusal rule, rank-0 final value)
 *   qto_net_replay           src/ContractionTools.h:392-411 (ContractGivenSequence, threshold 100)
 *   qto_net_lg_contract      src/LineGraph.h:92-171 wire numbering + 357-376 contraction walk
 *   qto_gate_tensor          src/Node.h:197-898 superoperator tables
 */
#ifndef QT_ORACLE_H
#define QT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qto_net qto_net;

/* error codes mirror src/Exceptions.h */
enum {
    QTO_OK = 0,
    QTO_INVALID_FILE = 1,
    QTO_INVALID_FILE_FORMAT = 2,
    QTO_CONTRACTION_FAILURE = 3,
    QTO_INVALID_FUNCTION_INPUT = 4,
    QTO_REFUSED = 5
};

/* One ContractIndices call.  Tensors are interleaved complex128 (re, im),
 * flat index sum_i idx_i * 4^i.  free_from_a[i]/free_idx[i] is toNotSumOn[i];
 * sum_a[j]/sum_b[j] is toSumOn[j].  C must hold 2*4^n_free doubles and is
 * overwritten (zero-filled first, as Node(rank) does). */
void qto_contract_indices(int rank_a, const double *a, int rank_b, const double *b,
                          int n_free, const int *free_from_a, const int *free_idx,
                          int n_sum, const int *sum_a, const int *sum_b, double *c);

/* Gate tensor by reference name: "Rx" "Ry" "Rz" "PHASE" (param narrowed to float
 * first, as std::stof does), "CPHASE" (param as double), "CRk" (param = control
 * qubit index), "H" "X" "Y" "Z" "CNOT" "CZ" "SWAP" "INIT" "T" "MX" "MY" "MZ" "M0" "M1".
 * Returns the rank (1, 2 or 4) or -1. out holds 2*4^rank doubles. */
int qto_gate_tensor(const char *name, double param, double *out);

/* Arbitrary gates from a .gate file (Node.h ArbitraryOneQubitNode / ArbitraryTwoQubitNode). */
int qto_arbitrary_gate(const char *path, int two_qubit, double *out);

/* Parse QASM text + measurement text.  gate_dir is where relative def1/def2
 * paths are opened from (NULL = current directory).  On error returns NULL and
 * *err holds a QTO_* code. */
qto_net *qto_net_parse(const char *qasm_text, const char *measure_text, const char *gate_dir, int *err);
void qto_net_free(qto_net *net);

int qto_net_num_qubits(const qto_net *net);
int qto_net_num_nodes(const qto_net *net);          /* size of mAllNodes */
int qto_net_node_rank(const qto_net *net, int id);
int qto_net_node_values(const qto_net *net, int id, double *out, int64_t cap_doubles);

/* ContractNodes(allNodes[a], allNodes[b], threshold).  Returns the id of the new
 * node, -1 for a refusal (nullptr), -2 when the network finished (nullptr). */
int qto_net_contract(qto_net *net, int id_a, int id_b, int threshold);

/* ContractGivenSequence: pairs are ids into mAllNodes. Returns QTO_OK or
 * QTO_CONTRACTION_FAILURE when the network is not done afterwards. */
int qto_net_replay(qto_net *net, const int *pairs, int n_pairs);

/* LineGraph numbering + LGContract walk over a 1-based wire elimination order.
 * Returns QTO_OK or QTO_CONTRACTION_FAILURE. */
int qto_net_lg_contract(qto_net *net, const int *order_1based, int n);

/* Line-graph wire numbering as LineGraph.h:92-171 assigns it: for every node of
 * the uncontracted list, its wire ids (in wire order) -> out (node_count entries
 * of `rank` ids each, flattened), returns total number of wires. */
int qto_net_lg_wire_ids(qto_net *net, int *node_ids, int *ranks, int *wire_ids, int cap);

int qto_net_done(const qto_net *net);
void qto_net_final_value(const qto_net *net, double *re_im);
int64_t qto_net_flops(const qto_net *net);
/* recorded (createdFrom) sequence, the walk preprocess.h:41-46 makes */
int qto_net_created_from(const qto_net *net, int *pairs, int cap_pairs);
/* value of the single remaining uncontracted node (what LGContract reads) */
int qto_net_remaining_value(const qto_net *net, double *re_im);

#ifdef __cplusplus
}
#endif
#endif
