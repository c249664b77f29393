// C ABI over the host library: networks (Network / ContractionTools /
// LineGraph), plans and batches.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <new>
#include <set>
#include <sstream>
#include <tuple>

#include "kernels.h"
#include "plan.h"

using namespace qtg;

struct qt_network {
    explicit qt_network(qt_ctx *c) : ctx(c) { ctx_retain(ctx); }
    ~qt_network() {
        net.reset();   // the nodes give their device tensors back first
        ctx_release(ctx);
    }
    qt_network(const qt_network &) = delete;
    qt_network &operator=(const qt_network &) = delete;
    qt_ctx *ctx = nullptr;
    std::string qasm, measure, gate_dir;
    std::shared_ptr<qtorch::Network> net;
};

// exceptions of the host library -> status codes
template <typename F>
static qt_status guard(qt_ctx *ctx, F &&f) {
    try {
        return f();
    } catch (const qtorch::InvalidFile &) {
        return set_error(ctx, QT_ERR_INVALID_FILE, "invalid file");
    } catch (const qtorch::InvalidFileFormat &) {
        return set_error(ctx, QT_ERR_INVALID_FILE_FORMAT, "invalid file format");
    } catch (const qtorch::ContractionFailure &) {
        return set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "contraction failed");
    } catch (const qtorch::InvalidUserContractionSequence &) {
        return set_error(ctx, QT_ERR_INVALID_USER_SEQUENCE, "invalid user contraction sequence");
    } catch (const qtorch::InvalidFunctionInput &) {
        return set_error(ctx, QT_ERR_INVALID_FUNCTION_INPUT, "invalid function input");
    } catch (const qtorch::InvalidContractionMethod &) {
        return set_error(ctx, QT_ERR_INVALID_CONTRACTION_METHOD, "invalid contraction method");
    } catch (const qtorch::QbbFailure &) {
        return set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "line graph ordering failure");
    } catch (const qtorch::EngineFailure &e) {
        return e.status();
    } catch (const std::bad_alloc &) {
        return set_error(ctx, QT_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception &e) {
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, e.what());
    }
}

// Seeded tries of the size-greedy walk (QT_ORDER_GREEDY, QT_ORDER_AUTO).  On
// the serving mix's large circuits 32 tries left 1.7-6x more MACs than 4096
// (a 26-qubit depth-12 random circuit: 4.7e12 -> 1.4e12 complex MACs); 4096
// walks of a 500-node network take about two core-seconds, spread over the
// host's cores.
constexpr int kGreedyTries = 4096;

static bool slurp(const char *path, std::string &out) {
    std::ifstream in(path, std::ios::binary);
    if (!in.is_open()) return false;
    std::stringstream ss;
    ss << in.rdbuf();
    out = ss.str();
    return true;
}

extern "C" {

// ---------------------------------------------------------------------------
// networks

qt_status qt_network_create(qt_ctx *ctx, const char *qasm_text, const char *measure_text, const char *gate_dir,
                            qt_network **out) {
    if (!qasm_text || !out) return QT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&]() {
        auto *n = new qt_network(ctx);
        n->qasm = qasm_text;
        n->measure = measure_text ? measure_text : "";
        n->gate_dir = gate_dir ? gate_dir : "";
        try {
            n->net = qtorch::Network::FromText(n->qasm, n->measure, n->gate_dir, ctx);
        } catch (...) {
            delete n;
            throw;
        }
        *out = n;
        return QT_OK;
    });
}

qt_status qt_network_create_from_files(qt_ctx *ctx, const char *qasm_path, const char *measure_path, qt_network **out) {
    if (!qasm_path || !out) return QT_ERR_INVALID_ARGUMENT;
    std::string q, m;
    if (!slurp(qasm_path, q)) return set_error(ctx, QT_ERR_INVALID_FILE, "cannot open QASM file");
    if (measure_path) slurp(measure_path, m);   // unreadable: every qubit is traced out
    return qt_network_create(ctx, q.c_str(), m.c_str(), nullptr, out);
}

qt_status qt_network_free(qt_network *n) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    delete n;
    return QT_OK;
}

qt_status qt_network_reset(qt_network *n) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        n->net = qtorch::Network::FromText(n->qasm, n->measure, n->gate_dir, n->ctx);
        return QT_OK;
    });
}

int qt_network_num_qubits(const qt_network *n) { return n ? n->net->GetNumQubits() : -1; }
int qt_network_num_nodes(const qt_network *n) { return n ? (int) n->net->GetAllNodes().size() : -1; }
int qt_network_num_uncontracted(const qt_network *n) { return n ? (int) n->net->GetUncontractedNodes().size() : -1; }

int qt_network_node_rank(const qt_network *n, int id) {
    if (!n || id < 0 || id >= (int) n->net->GetAllNodes().size()) return -1;
    return n->net->GetAllNodes()[id]->mRank;
}

int qt_network_is_done(const qt_network *n) { return n && n->net->IsDone() ? 1 : 0; }

qt_status qt_network_contract_nodes(qt_network *n, int a, int b, int threshold, int *new_id) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    const int cnt = (int) n->net->GetAllNodes().size();
    if (a < 0 || b < 0 || a >= cnt || b >= cnt) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        auto r = n->net->ContractNodes(n->net->GetAllNodes()[a], n->net->GetAllNodes()[b], threshold);
        if (new_id) *new_id = r ? r->mID : -1;
        return QT_OK;
    });
}

qt_status qt_network_contract_sequence(qt_network *n, const int32_t *pairs, int n_pairs) {
    if (!n || (n_pairs && !pairs) || n_pairs < 0) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        std::vector<std::pair<int, int>> seq(n_pairs);
        for (int i = 0; i < n_pairs; i++) seq[i] = {pairs[2 * i], pairs[2 * i + 1]};
        qtorch::ContractionTools t(n->net);
        t.ContractGivenSequence(seq);
        return QT_OK;
    });
}

qt_status qt_network_contract_user_sequence(qt_network *n, const char *text) {
    if (!n || !text) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        qtorch::ContractionTools t(n->net);
        t.ContractUserDefinedSequenceText(text);
        return QT_OK;
    });
}

qt_status qt_network_contract_stochastic(qt_network *n, uint64_t seed) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        qtorch::ContractionTools t(n->net);
        t.Seed(seed);
        t.Contract(qtorch::Stochastic);
        return QT_OK;
    });
}

qt_status qt_network_contract_linegraph(qt_network *n) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        qtorch::LineGraph lg(n->net);
        lg.LGContract();
        return QT_OK;
    });
}

qt_status qt_network_contract_wire_order(qt_network *n, const int32_t *order, int cnt) {
    if (!n || (cnt && !order) || cnt < 0) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        qtorch::LineGraph lg(n->net);
        lg.LGContract(std::vector<int>(order, order + cnt));
        return QT_OK;
    });
}

int qt_network_linegraph_order(qt_network *n, int32_t *order, int cap) {
    if (!n) return -1;
    try {
        qtorch::LineGraph lg(n->net);
        const auto &o = lg.MinFillOrdering();
        for (int i = 0; i < (int) o.size() && i < cap; i++) order[i] = o[i];
        return (int) o.size();
    } catch (...) {
        return -1;
    }
}

qt_status qt_network_reduce(qt_network *n) {
    if (!n) return QT_ERR_INVALID_ARGUMENT;
    return guard(n->ctx, [&]() {
        n->net->ReduceCircuit();
        return QT_OK;
    });
}

qt_status qt_network_final_value(const qt_network *n, double *v) {
    if (!n || !v) return QT_ERR_INVALID_ARGUMENT;
    v[0] = n->net->GetFinalValue().real();
    v[1] = n->net->GetFinalValue().imag();
    return QT_OK;
}

int64_t qt_network_flops(const qt_network *n) { return n ? n->net->getNumFloatOps() : -1; }

int qt_network_created_from(const qt_network *n, int32_t *pairs, int cap) {
    if (!n) return -1;
    int k = 0;
    for (const auto &node : n->net->GetAllNodes()) {
        if (node->mCreatedFrom.first == 0 && node->mCreatedFrom.second == 0) continue;
        if (k < cap && pairs) {
            pairs[2 * k] = node->mCreatedFrom.first;
            pairs[2 * k + 1] = node->mCreatedFrom.second;
        }
        k++;
    }
    return k;
}

int64_t qt_network_node_values(qt_network *n, int id, double *out, int64_t cap) {
    if (!n || id < 0 || id >= (int) n->net->GetAllNodes().size()) return -1;
    auto &node = n->net->GetAllNodes()[id];
    if (!node->HasData()) return -1;
    try {
        auto &v = node->GetTensorVals();
        const int64_t cnt = (int64_t) v.size();
        if (out) std::memcpy(out, v.data(), sizeof(double) * 2 * (size_t) std::min(cnt, cap));
        return cnt;
    } catch (...) {
        return -1;
    }
}

// ---------------------------------------------------------------------------
// plans

}  // extern "C"

namespace qtg {
// The leaves (ranks, complex128 values, rotation leaves) of a network, and once
// it is contracted, its recorded sequence and the lowered schedule.
void plan_collect_leaves(qt_plan *p, const qtorch::Network &net) {
    for (const auto &leaf : net.Leaves()) {
        p->leaf_rank.push_back(leaf->mRank);
        const auto &v = leaf->GetTensorVals();
        const char *kind = nullptr;
        switch (leaf->GetTypeOfNode()) {
            case qtorch::GateType::RX: kind = "Rx"; break;
            case qtorch::GateType::RY: kind = "Ry"; break;
            case qtorch::GateType::RZ: kind = "Rz"; break;
            case qtorch::GateType::PHASE: kind = "PHASE"; break;
            case qtorch::GateType::CPHASE: kind = "CPHASE"; break;
            default: break;
        }
        // a rotation leaf whose wires were sliced away is no longer the gate's table
        if (kind && (int) v.size() == (1 << (2 * leaf->mRank)) && (leaf->mRank == 2 || leaf->mRank == 4)) {
            p->rot_kind.push_back(kind);
            p->rot_angle.push_back(qtorch::GateAngle(*leaf));
            p->rot_elem.push_back(p->leaf_values.size());
            p->rot_leaf.push_back((int) p->leaf_rank.size() - 1);
        }
        p->leaf_values.insert(p->leaf_values.end(), v.begin(), v.end());
    }
}

qt_status plan_finish(qt_plan *p, const qtorch::Network &net) {
    for (const auto &node : net.GetAllNodes()) {
        if (node->mCreatedFrom.first == 0 && node->mCreatedFrom.second == 0) continue;
        p->sequence.push_back(node->mCreatedFrom.first);
        p->sequence.push_back(node->mCreatedFrom.second);
    }
    return lower_plan(p, net);
}
}  // namespace qtg

extern "C" {

qt_status qt_plan_build(qt_ctx *ctx, const char *qasm_text, const char *measure_text, const char *gate_dir,
                        qt_ordering ordering, uint64_t seed, const int32_t *pairs, int n_pairs, qt_plan **out) {
    // ctx may be NULL: the plan can then be inspected (sequence, sizes) but not executed
    if (!qasm_text || !out) return QT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&]() {
        auto *p = new qt_plan(ctx);
        p->qasm = qasm_text;
        p->measure = measure_text ? measure_text : "";
        p->gate_dir = gate_dir ? gate_dir : "";
        std::unique_ptr<qt_plan> owner(p);
        auto net = qtorch::Network::FromText(p->qasm, p->measure, p->gate_dir, nullptr);
        plan_collect_leaves(p, *net);
        if (ordering == QT_ORDER_STOCHASTIC) {
            qtorch::ContractionTools t(net);
            t.Seed(seed);
            t.Contract(qtorch::Stochastic);
        } else if (ordering == QT_ORDER_LINEGRAPH) {
            qtorch::LineGraph lg(net);
            lg.LGContract();
        } else if (ordering == QT_ORDER_GREEDY) {
            qtorch::GreedyContract(*net, seed, kGreedyTries);
        } else if (ordering == QT_ORDER_AUTO) {
            qtorch::AutoContract(net, seed, kGreedyTries, 1500);
        } else if (ordering == QT_ORDER_SEQUENCE) {
            if (n_pairs < 0 || (n_pairs && !pairs)) return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "sequence");
            std::vector<std::pair<int, int>> seq(n_pairs);
            for (int i = 0; i < n_pairs; i++) seq[i] = {pairs[2 * i], pairs[2 * i + 1]};
            qtorch::ContractionTools t(net);
            t.ContractGivenSequence(seq);
        } else {
            return set_error(ctx, QT_ERR_INVALID_CONTRACTION_METHOD, "unknown ordering");
        }
        if (!net->IsDone()) return set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "ordering did not finish the network");
        qt_status s = plan_finish(p, *net);
        if (s != QT_OK) return s;
        *out = owner.release();
        return QT_OK;
    });
}

qt_status qt_plan_build_search(qt_ctx *ctx, const char *qasm_text, const char *measure_text, const char *gate_dir,
                               uint64_t seed, int tries, int64_t max_macs, qt_plan **out, uint64_t *chosen_seed) {
    if (!qasm_text || !out || tries < 1) return QT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    qtorch::PreProcessResult best;
    qt_status s = guard(ctx, [&]() {
        if (!qtorch::preProcess(qasm_text, measure_text ? measure_text : "", gate_dir ? gate_dir : "", seed, tries,
                                (long long) max_macs, best))
            return set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "no stochastic try finished the network");
        return QT_OK;
    });
    if (s != QT_OK) return s;
    if (chosen_seed) *chosen_seed = best.seed;
    std::vector<int32_t> pairs;
    for (const auto &pr : best.sequence) {
        pairs.push_back(pr.first);
        pairs.push_back(pr.second);
    }
    return qt_plan_build(ctx, qasm_text, measure_text, gate_dir, QT_ORDER_SEQUENCE, 0, pairs.data(),
                         (int) best.sequence.size(), out);
}

qt_status qt_plan_free(qt_plan *p) {
    if (!p) return QT_ERR_INVALID_ARGUMENT;
    for (auto &v : p->slicings)
        for (auto &e : v) qt_sliced_free(e.second);
    for (int i = 0; i < 2; i++)
        if (p->dev[i] && p->ctx) dev_free(p->ctx, p->dev[i]);
    delete p;
    return QT_OK;
}

int qt_plan_num_steps(const qt_plan *p) { return p ? p->n_steps : -1; }
int64_t qt_plan_item_descriptors(const qt_plan *p) { return p ? (int64_t) p->items[QT_PREC_MIXED].size() : -1; }
int qt_plan_num_leaves(const qt_plan *p) { return p ? (int) p->leaf_rank.size() : -1; }
int qt_plan_peak_rank(const qt_plan *p) { return p ? p->peak_rank : -1; }
uint64_t qt_plan_workspace_bytes(const qt_plan *p, qt_precision prec) {
    return p && (prec == QT_PREC_FP64 || prec == QT_PREC_MIXED) ? p->ws_bytes[prec] : 0;
}
int64_t qt_plan_flops(const qt_plan *p) { return p ? p->flops : -1; }

uint64_t qt_plan_algorithmic_bytes(const qt_plan *p, qt_precision prec) {
    if (!p || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return 0;
    uint64_t total = 0;
    for (const auto &d : p->steps[prec]) {
        const uint64_t ea = (d.flags & kAF64) ? 16 : 8, eb = (d.flags & kBF64) ? 16 : 8, ec = (d.flags & kCF64) ? 16 : 8;
        total += (ea << (2 * d.rA)) + (eb << (2 * d.rB)) + (ec << (2 * d.nFree));
    }
    return total;
}

int qt_plan_sequence(const qt_plan *p, int32_t *pairs, int cap) {
    if (!p) return -1;
    const int n = (int) p->sequence.size() / 2;
    for (int i = 0; i < n && i < cap; i++) {
        pairs[2 * i] = p->sequence[2 * i];
        pairs[2 * i + 1] = p->sequence[2 * i + 1];
    }
    return n;
}

uint64_t qt_plan_leaf_elems(const qt_plan *p) { return p ? p->leaf_values.size() : 0; }

int qt_plan_num_rotations(const qt_plan *p) { return p ? (int) p->rot_kind.size() : -1; }

qt_status qt_plan_rotation_angles(const qt_plan *p, double *angles, int cap) {
    if (!p || (!angles && cap)) return QT_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < (int) p->rot_angle.size() && i < cap; i++) angles[i] = p->rot_angle[i];
    return QT_OK;
}

int qt_plan_step_info(const qt_plan *p, qt_precision prec, int32_t *out, int cap) {
    if (!p || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED) || (!out && cap)) return -1;
    const auto &steps = p->steps[prec];
    for (int L = 0; L < p->n_levels; L++) {
        for (int i = p->level_start[L]; i < p->level_start[L + 1] && i < cap; i++) {
            const qtg::StepDesc &d = steps[i];
            int32_t *o = out + (size_t) i * QT_STEP_INFO_FIELDS;
            o[0] = L;
            o[1] = d.rA;
            o[2] = d.rB;
            o[3] = d.nFree;
            o[4] = d.nSum;
            o[5] = d.group;
            o[6] = (int32_t) d.flags;
            o[7] = d.tab_off != qtg::kNoTable ? 1 : 0;
        }
    }
    return p->n_steps;
}

qt_status qt_plan_leaf_values(const qt_plan *p, double *out, uint64_t cap) {
    if (!p || !out || cap < p->leaf_values.size()) return QT_ERR_INVALID_ARGUMENT;
    std::memcpy(out, p->leaf_values.data(), p->leaf_values.size() * sizeof(std::complex<double>));
    return QT_OK;
}

qt_status qt_plan_execute(qt_ctx *ctx, qt_plan *p, qt_precision prec, double *v) {
    if (!ctx || !p || !p->ctx || !v || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return QT_ERR_INVALID_ARGUMENT;
    if (!p->grouped || p->flops > lone_instance_max_macs(prec))
        return execute_stepwise(p, ctx, prec, p->leaf_values.data(), v);
    qt_batch *b = nullptr;
    qt_status s = qt_batch_create(ctx, &b);
    if (s != QT_OK) return s;
    int idx;
    s = qt_batch_add(b, p, nullptr, &idx);
    if (s == QT_OK) s = qt_batch_execute(b, prec, v);
    qt_batch_free(b);
    return s;
}

// ---------------------------------------------------------------------------
// batches

static qt_status batch_device_rotations(qt_batch *b, bool on);

// Resident evaluation engine (qt_batch_use_resident).
// Stops the engine if it runs and waits for its CTAs to leave (each polls the
// request word about once a microsecond).
static qt_status resident_stop(qt_batch *b) {
    if (!b->res_running) return QT_OK;
    __atomic_store_n(&b->h_mail[0], kResidentStop, __ATOMIC_RELEASE);
    const cudaError_t e = cudaStreamSynchronize(b->res_stream);
    b->res_running = false;
    __atomic_store_n(&b->h_mail[0], b->res_seq, __ATOMIC_RELEASE);
    return cuda_error(b->ctx, e, "resident engine stop");
}

// Launches the engine on the batch's own stream; requests after first_seq are new.
static qt_status resident_start(qt_batch *b, uint32_t first_seq) {
    qt_ctx *ctx = b->ctx;
    const size_t n = b->inst_desc.size();
    qt_status s = QT_OK;
    cudaError_t e = cudaSuccess;
    if (!b->res_stream) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        e = cudaStreamCreateWithPriority(&b->res_stream, cudaStreamNonBlocking, hi);
        if (e != cudaSuccess) return cuda_error(ctx, e, "resident stream");
    }
    if (!b->h_mail) {
        void *hm = nullptr;
        s = host_alloc(ctx, sizeof(uint32_t) * (32 + n), &hm);
        if (s != QT_OK) return s;
        b->h_mail = static_cast<uint32_t *>(hm);
        std::memset(b->h_mail, 0, sizeof(uint32_t) * (32 + n));
    }
    if (!b->h_angles && b->n_angles) {
        void *ha = nullptr;
        s = host_alloc(ctx, sizeof(double) * b->n_angles, &ha);
        if (s != QT_OK) return s;
        b->h_angles = static_cast<double *>(ha);
    }
    // Requests post tagged angle words when every instance's angles fit one per
    // thread of its CTA (they are polled one per thread).
    if (!b->d_inst_res) {
        const int threads = plan_threads(b->variant);
        b->res_tagged = b->n_angles > 0;
        for (const qt_plan *p : b->plans)
            if ((int) p->rot_kind.size() > threads) b->res_tagged = false;
    }
    if (b->res_tagged && !b->h_tagged) {
        void *ht = nullptr;
        s = host_alloc(ctx, sizeof(uint64_t) * b->n_angles, &ht);
        if (s != QT_OK) return s;
        b->h_tagged = static_cast<uint64_t *>(ht);
        std::memset(b->h_tagged, 0, sizeof(uint64_t) * b->n_angles);   // request 0 is never posted
    }
    void *ha = nullptr, *hv = nullptr, *hm = nullptr;
    if (b->res_tagged) e = cudaHostGetDevicePointer(&ha, b->h_tagged, 0);
    else if (b->h_angles) e = cudaHostGetDevicePointer(&ha, b->h_angles, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(&hv, b->h_values, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(&hm, b->h_mail, 0);
    if (e != cudaSuccess) return cuda_error(ctx, e, "mapped host buffers");
    if (!b->d_inst_res) {
        // descriptor j runs on CTA j: angles from, and the value to, pinned host memory
        std::vector<InstanceDesc> zc = b->inst_desc;
        for (size_t j = 0; j < n; j++) {
            const int i = b->inst_index[j];
            // (tagged: the 64-bit words of h_tagged, one per angle, at the same offsets)
            zc[j].angles = b->plans[i]->rot_kind.empty() ? nullptr
                                                         : static_cast<const double *>(ha) + b->inst_angle_off[i];
            zc[j].value = static_cast<double *>(hv) + 2 * i;
        }
        s = dev_alloc(ctx, sizeof(InstanceDesc) * n, &b->d_inst_res);
        if (s != QT_OK) return s;
        e = cudaMemcpyAsync(b->d_inst_res, zc.data(), sizeof(InstanceDesc) * n, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_error(ctx, e, "resident descriptors");
    }
    ResidentLaunch rl{};
    rl.lp.instances = static_cast<const InstanceDesc *>(b->d_inst_res);
    rl.lp.n_instances = (int) n;
    rl.lp.ws_smem_bytes = b->ws_smem_bytes;
    rl.lp.ws_base = (char *) b->d_ws;
    rl.lp.ws_stride = b->ws_stride;
    rl.lp.stage_bytes = b->stage_bytes;
    rl.lp.tile_bytes = b->tile_bytes;
    rl.lp.next = nullptr;
    rl.lp.header_steps = b->header_steps;
    rl.seq = static_cast<const uint32_t *>(hm);
    rl.done = static_cast<uint32_t *>(hm) + 32;
    rl.first_seq = first_seq;
    rl.idle_polls = (uint32_t) std::min(4.0e9, std::max(1.0, b->res_idle * 1.0e6));
    rl.tagged = b->res_tagged ? 1u : 0u;
    for (size_t j = 0; j < n; j++) __atomic_store_n(&b->h_mail[32 + j], 0u, __ATOMIC_RELAXED);   // no flag from a previous run
    __atomic_store_n(&b->h_mail[0], first_seq, __ATOMIC_RELEASE);
    e = launch_resident(rl, b->res_stream, b->variant);
    if (e != cudaSuccess) return cuda_error(ctx, e, "resident engine launch");
    ctx->launches++;
    b->res_starts++;
    b->res_running = true;
    return QT_OK;
}

// A value slot's contents while its answer has not arrived: a signalling NaN
// (quiet bit clear, payload nonzero), which no arithmetic result can be.
constexpr uint64_t kValuePending = 0x7ff4c0de0000d0e5ull;

// One evaluation through the engine: angles into pinned memory, the request
// number after them, then every CTA's value.
static qt_status resident_evaluate(qt_batch *b, const double *angles, int64_t n_angles, double *values) {
    qt_ctx *ctx = b->ctx;
    if (n_angles != b->n_angles) return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "angle count does not match the batch");
    qt_status s = QT_OK;
    const size_t n = b->inst_desc.size();
    // (an engine whose CTAs left while idle shows it in their flags: the wait
    // below restarts it)
    if (!b->res_running) {
        s = resident_start(b, b->res_seq);
        if (s != QT_OK) return s;
    }
    uint32_t seq = resident_next_request(b->res_seq);
    b->res_seq = seq;
    // Every value slot holds a signalling-NaN pattern until its CTA writes the
    // answer (arithmetic never produces a signalling NaN).  The host watches the
    // values themselves: a CTA writes its value and only then, behind a
    // system-scope release, its done flag, so the value is in host memory one
    // CPU-GPU round trip before the flag.  The slots are reset before the
    // request's angles and number are published (release), so no answer can be
    // overwritten.
    uint64_t *const hv = reinterpret_cast<uint64_t *>(b->h_values);
    for (size_t j = 0; j < n; j++) {
        const size_t i = (size_t) b->inst_index[j];
        __atomic_store_n(hv + 2 * i, kValuePending, __ATOMIC_RELAXED);
        __atomic_store_n(hv + 2 * i + 1, kValuePending, __ATOMIC_RELAXED);
    }
    if (b->res_tagged) {
        // (request << 32) | the angle narrowed to float, as the device narrows it
        __atomic_thread_fence(__ATOMIC_RELEASE);
        for (int64_t r = 0; r < n_angles; r++) {
            const float f = (float) angles[r];
            uint32_t bits;
            std::memcpy(&bits, &f, 4);
            __atomic_store_n(b->h_tagged + r, ((uint64_t) seq << 32) | bits, __ATOMIC_RELAXED);
        }
    } else if (n_angles) {
        // the previous request is complete, so the pinned angles are free
        std::memcpy(b->h_angles, angles, sizeof(double) * n_angles);
    }
    __atomic_store_n(&b->h_mail[0], seq, __ATOMIC_RELEASE);
    // Wait for every CTA's value (or flag).  The engine is asked about only
    // after a millisecond without an answer (a stream query costs more than a
    // request).
    const auto t0 = std::chrono::steady_clock::now();
    bool relaunched = false;
    uint64_t spins = 0;
    for (size_t j = 0; j < n;) {
        const size_t i = (size_t) b->inst_index[j];
        if (__atomic_load_n(hv + 2 * i, __ATOMIC_ACQUIRE) != kValuePending &&
            __atomic_load_n(hv + 2 * i + 1, __ATOMIC_ACQUIRE) != kValuePending) {
            j++;
            continue;
        }
        const uint32_t d = __atomic_load_n(&b->h_mail[32 + j], __ATOMIC_ACQUIRE);
        if (d == seq) {
            j++;
            continue;
        }
        bool restart = d == kResidentLeft;   // the CTA left (idle) just before this request
        if (!restart && (++spins & 1023) == 0) {
            const double waited = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (waited > 10.0) return set_error(ctx, QT_ERR_CUDA, "resident engine did not answer within 10 s");
            if (waited > 1e-3) {
                const cudaError_t q = cudaStreamQuery(b->res_stream);
                if (q == cudaSuccess) restart = true;   // gone without a word
                else if (q != cudaErrorNotReady) return cuda_error(ctx, q, "resident engine");
            }
        }
        if (restart) {
            // CTAs leave on their own idle clocks: stop the rest, start all again
            if (relaunched) return set_error(ctx, QT_ERR_CUDA, "resident engine left without answering");
            relaunched = true;
            s = resident_stop(b);
            if (s == QT_OK) s = resident_start(b, seq - 1);
            if (s != QT_OK) return s;
            __atomic_store_n(&b->h_mail[0], seq, __ATOMIC_RELEASE);
            j = 0;
        }
    }
    std::memcpy(values, b->h_values, sizeof(double) * 2 * b->plans.size());
    return QT_OK;
}

static void batch_release(qt_batch *b) {
    qt_ctx *ctx = b->ctx;
    resident_stop(b);
    dev_free(ctx, b->d_inst_res);
    b->d_inst_res = nullptr;
    host_free(ctx, b->h_mail);
    b->h_mail = nullptr;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (b->eval_graph) {
        cudaGraphExecDestroy(b->eval_graph);
        b->eval_graph = nullptr;
    }
    dev_free(ctx, b->d_leaves);
    dev_free(ctx, b->d_inst);
    dev_free(ctx, b->d_values);
    dev_free(ctx, b->d_ws);
    dev_free(ctx, b->d_next);
    dev_free(ctx, b->d_angles);
    dev_free(ctx, b->d_inst_eval);
    b->d_inst_eval = nullptr;
    b->d_leaves = b->d_inst = b->d_values = b->d_ws = b->d_next = b->d_angles = nullptr;
    b->tile_bytes = 0;
    host_free(ctx, b->h_angles);
    b->h_angles = nullptr;
    host_free(ctx, b->h_tagged);
    b->h_tagged = nullptr;
    b->res_tagged = false;
    if (b->angles_done) cudaEventDestroy(b->angles_done);
    b->angles_done = nullptr;
    b->dev_rot = false;
    host_free(ctx, b->h_leaves);
    host_free(ctx, b->h_values);
    b->h_leaves = b->h_values = nullptr;
    b->prepared_prec = -1;
}

qt_status qt_batch_create(qt_ctx *ctx, qt_batch **out) {
    if (!ctx || !out) return QT_ERR_INVALID_ARGUMENT;
    *out = new (std::nothrow) qt_batch(ctx);
    if (!*out) return QT_ERR_OUT_OF_MEMORY;
    return QT_OK;
}

qt_status qt_batch_free(qt_batch *b) {
    if (!b) return QT_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::recursive_mutex> g(b->ctx->lock);
        cudaStreamSynchronize(b->ctx->stream);
        batch_release(b);
        if (b->res_stream) cudaStreamDestroy(b->res_stream);
        b->res_stream = nullptr;
    }
    delete b;   // may drop the context's last reference
    return QT_OK;
}

qt_status qt_batch_add(qt_batch *b, qt_plan *p, const double *leaves, int *index) {
    // plans may come from another context on the same device (the server's lanes)
    if (!b || !p || !p->ctx || p->ctx->device != b->ctx->device) return QT_ERR_INVALID_ARGUMENT;
    b->plans.push_back(p);
    if (leaves) {
        const auto *c = reinterpret_cast<const std::complex<double> *>(leaves);
        b->leaves.emplace_back(c, c + p->leaf_values.size());
    } else {
        b->leaves.push_back(p->leaf_values);
    }
    b->dirty = true;
    if (index) *index = (int) b->plans.size() - 1;
    return QT_OK;
}

int qt_batch_size(const qt_batch *b) { return b ? (int) b->plans.size() : -1; }

qt_status qt_batch_set_leaves(qt_batch *b, int i, const double *leaves) {
    if (!b || !leaves || i < 0 || i >= (int) b->plans.size()) return QT_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::recursive_mutex> g(b->ctx->lock);
        qt_status s = batch_device_rotations(b, false);
        if (s != QT_OK) return s;
    }
    const auto *c = reinterpret_cast<const std::complex<double> *>(leaves);
    std::copy(c, c + b->leaves[i].size(), b->leaves[i].begin());
    return QT_OK;
}

// Device rotations on/off: the descriptors carry the angle pointers or null.
static qt_status batch_device_rotations(qt_batch *b, bool on) {
    if (b->res_running) {
        qt_status s = resident_stop(b);
        if (s != QT_OK) return s;
    }
    if (b->dev_rot == on || b->inst_desc.empty()) {
        b->dev_rot = on;
        return QT_OK;
    }
    qt_ctx *ctx = b->ctx;
    for (size_t j = 0; j < b->inst_desc.size(); j++) {
        const int i = b->inst_index[j];
        b->inst_desc[j].angles = on && !b->plans[i]->rot_kind.empty()
                                     ? static_cast<const double *>(b->d_angles) + b->inst_angle_off[i]
                                     : nullptr;
    }
    cudaError_t e = cudaMemcpyAsync(b->d_inst, b->inst_desc.data(), sizeof(InstanceDesc) * b->inst_desc.size(),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // the host copy may change again
    if (e != cudaSuccess) return cuda_error(ctx, e, "instance descriptor upload");
    b->dev_rot = on;
    return QT_OK;
}

qt_status qt_batch_set_rotations_device(qt_batch *b, const double *angles, int64_t n_angles) {
    if (!b || (n_angles && !angles)) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (b->prepared_prec != QT_PREC_MIXED)
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "device rotations need a batch prepared for QT_PREC_MIXED");
    if (n_angles != b->n_angles) return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "angle count does not match the batch");
    if (!n_angles) return QT_OK;
    qt_status s = resident_stop(b);
    if (s != QT_OK) return s;
    if (!b->h_angles) {
        void *ha = nullptr;
        s = host_alloc(ctx, sizeof(double) * n_angles, &ha);
        if (s != QT_OK) return s;
        b->h_angles = static_cast<double *>(ha);
    }
    if (!b->angles_done) {
        cudaError_t e = cudaEventCreateWithFlags(&b->angles_done, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_error(ctx, e, "angle staging");
    } else {
        // the previous upload must have read the pinned copy before it is overwritten
        cudaError_t e = cudaEventSynchronize(b->angles_done);
        if (e != cudaSuccess) return cuda_error(ctx, e, "angle staging");
    }
    if (!b->d_angles) {
        s = dev_alloc(ctx, sizeof(double) * n_angles, &b->d_angles);
        if (s != QT_OK) return s;
    }
    std::memcpy(b->h_angles, angles, sizeof(double) * n_angles);
    cudaError_t e = cudaMemcpyAsync(b->d_angles, b->h_angles, sizeof(double) * n_angles, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->angles_done, ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "angle upload");
    // instances run step by step take their leaves from the host
    if (!b->stepwise.empty()) {
        s = guard(ctx, [&]() {
            for (int i : b->stepwise) {
                const qt_plan *p = b->plans[i];
                for (size_t r = 0; r < p->rot_kind.size(); r++) {
                    auto gt = qtorch::MakeGateNode(p->rot_kind[r], angles[b->inst_angle_off[i] + (int64_t) r]);
                    const auto &v = gt->GetTensorVals();
                    std::copy(v.begin(), v.end(), b->leaves[i].begin() + p->rot_elem[r]);
                }
            }
            return QT_OK;
        });
        if (s != QT_OK) return s;
    }
    return batch_device_rotations(b, true);
}

qt_status qt_batch_set_rotations(qt_batch *b, const double *angles, int64_t n_angles) {
    if (!b || (n_angles && !angles)) return QT_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::recursive_mutex> g(b->ctx->lock);
        qt_status s = batch_device_rotations(b, false);
        if (s != QT_OK) return s;
    }
    int64_t need = 0;
    for (auto *p : b->plans) need += (int64_t) p->rot_kind.size();
    if (need != n_angles) return set_error(b->ctx, QT_ERR_INVALID_ARGUMENT, "angle count does not match the batch");
    return guard(b->ctx, [&]() {
        int64_t k = 0;
        for (size_t i = 0; i < b->plans.size(); i++) {
            const qt_plan *p = b->plans[i];
            for (size_t r = 0; r < p->rot_kind.size(); r++, k++) {
                auto g = qtorch::MakeGateNode(p->rot_kind[r], angles[k]);
                const auto &v = g->GetTensorVals();
                std::copy(v.begin(), v.end(), b->leaves[i].begin() + p->rot_elem[r]);
            }
        }
        return QT_OK;
    });
}

static qt_status batch_pack(qt_batch *b) {
    const int prec = b->prepared_prec;
    for (size_t i = 0; i < b->plans.size(); i++) {
        if (!b->in_group[i]) continue;
        pack_leaves(b->plans[i], prec, b->leaves[i].data(), (char *) b->h_leaves + b->inst_leaf_off[i]);
    }
    return QT_OK;
}

// Launch parameters of the grouped launch under the batch's policy: the shared-
// memory regions of a CTA, the grid, the schedule, the global workspace slab
// and the instance descriptors.  Leaf images, values and plan blocks stay where
// they are, so a policy change (and each autotuner candidate) only re-runs this.
// The occupancy figures a batch sizes its launch by, computed once per shape:
// the driver queries behind them can wait while other threads allocate.
static std::mutex g_launch_shape_lock;
static std::map<std::tuple<size_t, int, int, int>, int> g_max_grid;
static std::map<int, size_t> g_smem_limit;

static int cached_max_grid(size_t smem, int per_sm_cap, int variant) {
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(smem, per_sm_cap, variant, dev);
    {
        std::lock_guard<std::mutex> g(g_launch_shape_lock);
        auto it = g_max_grid.find(key);
        if (it != g_max_grid.end()) return it->second;
    }
    const int v = plan_max_grid(smem, per_sm_cap, variant);
    std::lock_guard<std::mutex> g(g_launch_shape_lock);
    g_max_grid[key] = v;
    return v;
}

static size_t cached_smem_limit() {
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> g(g_launch_shape_lock);
        auto it = g_smem_limit.find(dev);
        if (it != g_smem_limit.end()) return it->second;
    }
    const size_t v = plan_smem_limit();
    std::lock_guard<std::mutex> g(g_launch_shape_lock);
    if (v) g_smem_limit[dev] = v;
    return v;
}

static qt_status batch_configure(qt_batch *b) {
    qt_ctx *ctx = b->ctx;
    const int prec = b->prepared_prec;
    const int n = (int) b->plans.size();
    qt_status rs = resident_stop(b);
    if (rs != QT_OK) return rs;
    cudaError_t se = cudaStreamSynchronize(ctx->stream);
    if (se != cudaSuccess) return cuda_error(ctx, se, "sync");
    for (cudaGraphExec_t *g : {&b->graph, &b->eval_graph})
        if (*g) {
            cudaGraphExecDestroy(*g);
            *g = nullptr;
        }
    dev_free(ctx, b->d_ws);
    dev_free(ctx, b->d_next);
    dev_free(ctx, b->d_inst);
    dev_free(ctx, b->d_inst_eval);
    dev_free(ctx, b->d_inst_res);
    b->d_ws = b->d_next = b->d_inst = b->d_inst_eval = b->d_inst_res = nullptr;
    b->inst_desc.clear();
    b->inst_index.clear();
    uint64_t ws = 0;
    int n_grouped = 0;
    bool any_tiled = false;
    for (int i = 0; i < n; i++) {
        if (!b->in_group[i]) continue;
        const qt_plan *p = b->plans[i];
        ws = std::max<uint64_t>(ws, (p->ws_bytes[prec] + 255) / 256 * 256);
        any_tiled = any_tiled || p->n_tiled > 0;
        n_grouped++;
    }
    // a workspace region as large as the largest workspace under the cap, a
    // staging region as large as the largest plan block + leaf image under the
    // cap, and the tile buffers when an instance has CTA-tiled steps; instances
    // beyond either region use the global slab / read in place
    // Defaults: a few instances (at most two CTAs per SM) get the 128-register
    // interpreter -- the wide 512-thread form when one CTA per SM holds them
    // all -- and room to keep small workspaces and staged copies in shared
    // memory; many instances are latency-bound and get the 64-register variant
    // with four CTAs per SM, which leaves room for small workspaces only.
    const qt_launch_policy &pol = b->policy;
    const bool many = n_grouped > 2 * plan_num_sms();
    const bool wide = pol.kernel_ctas == 1 || (!pol.kernel_ctas && !many && n_grouped <= plan_num_sms());
    const uint64_t ws_cap = pol.ws_smem_cap >= 0 ? (uint64_t) pol.ws_smem_cap
                            : many                ? kSmemWorkspaceMaxMany
                                                  : kSmemWorkspaceMax;
    const uint64_t stage_cap = pol.stage_cap >= 0 ? (uint64_t) pol.stage_cap
                               : many             ? 0
                               : wide             ? (any_tiled ? kSmemStageMaxWideTiled : kSmemStageMaxWide)
                               : any_tiled        ? kSmemStageMaxTiled
                                                  : kSmemStageMax;
    uint64_t ws_small = 0, stage_small = 0;
    b->header_steps = 1;
    for (int i = 0; i < n; i++) {
        if (!b->in_group[i]) continue;
        const qt_plan *p = b->plans[i];
        const uint64_t w = (p->ws_bytes[prec] + 255) / 256 * 256;
        if (w <= ws_cap) ws_small = std::max(ws_small, w);
        const uint64_t st = round16(p->dev_bytes[prec]) + round16(p->leaf_bytes[prec]);
        if (st <= stage_cap) stage_small = std::max(stage_small, st);
        b->header_steps = std::max<uint32_t>(b->header_steps, (uint32_t) p->n_steps);
    }
    b->ws_stride = ws;
    b->ws_smem_bytes = (uint32_t) ws_small;
    b->stage_bytes = (uint32_t) stage_small;
    b->tile_bytes = any_tiled ? kCtaTileBytes : 0;
    b->ws_in_smem = ws <= b->ws_smem_bytes;   // no global slab needed
    const size_t smem = plan_header_bytes(b->header_steps) + 128 + b->ws_smem_bytes + b->stage_bytes + b->tile_bytes;
    if (n_grouped && smem > cached_smem_limit())
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "launch policy needs more shared memory than a CTA may have");
    b->variant = pol.kernel_ctas ? pol.kernel_ctas : many ? 4 : n_grouped <= plan_num_sms() ? 1 : 2;
    b->grid = n_grouped ? std::min(n_grouped, cached_max_grid(smem, pol.ctas_per_sm, b->variant)) : 0;
    qt_status s = QT_OK;
    if (b->grid > 0 && !b->ws_in_smem) s = dev_alloc(ctx, b->ws_stride * b->grid, &b->d_ws);
    // more instances than CTAs: a dynamic schedule over the instances sorted by
    // estimated cost, longest first (unless the policy asks for a round robin)
    const bool dynamic = n_grouped > b->grid && !pol.static_schedule;
    if (s == QT_OK && dynamic) s = dev_alloc(ctx, 256, &b->d_next);
    if (s != QT_OK) return s;
    std::vector<int> inst_order;
    for (int i = 0; i < n; i++)
        if (b->in_group[i]) inst_order.push_back(i);
    if (dynamic) {
        auto cost = [&](int i) {
            const qt_plan *p = b->plans[i];
            return (double) p->flops + 2048.0 * p->n_levels;   // MACs plus a per-level latency term
        };
        std::stable_sort(inst_order.begin(), inst_order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    }
    std::vector<InstanceDesc> inst;
    for (int i : inst_order) {
        qt_plan *p = b->plans[i];
        InstanceDesc d{};
        d.plan = reinterpret_cast<const PlanDesc *>(p->dev[prec]);
        d.leaves = (const char *) b->d_leaves + b->inst_leaf_off[i];
        d.value = (double *) b->d_values + 2 * i;
        d.plan_bytes = b->stage_bytes ? (uint32_t) round16(p->dev_bytes[prec]) : 0;
        d.leaf_bytes = (uint32_t) round16(p->leaf_bytes[prec]);
        d.ws_bytes = (uint32_t) ((p->ws_bytes[prec] + 255) / 256 * 256);
        d.n_steps = (uint32_t) p->n_steps;
        d.angles = b->dev_rot && b->d_angles && !p->rot_kind.empty()
                       ? static_cast<const double *>(b->d_angles) + b->inst_angle_off[i]
                       : nullptr;
        inst.push_back(d);
    }
    b->inst_desc = inst;
    b->inst_index = inst_order;
    if (inst.empty()) return QT_OK;
    s = dev_alloc(ctx, sizeof(InstanceDesc) * inst.size(), &b->d_inst);
    if (s != QT_OK) return s;
    // through the context's pinned staging buffer: a copy from pageable memory
    // goes through the driver's shared staging and can wait behind other
    // threads' large pageable copies
    const size_t inst_bytes = sizeof(InstanceDesc) * inst.size();
    s = ensure_pinned(ctx, inst_bytes);
    if (s != QT_OK) return s;
    std::memcpy(ctx->pinned, inst.data(), inst_bytes);
    cudaError_t e = cudaMemcpyAsync(b->d_inst, ctx->pinned, inst_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // the staging buffer is reused
    return cuda_error(ctx, e, "instance upload");
}

qt_status qt_batch_prepare(qt_batch *b, qt_precision prec) {
    if (!b || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    cudaStreamSynchronize(ctx->stream);
    batch_release(b);
    b->prepared_prec = prec;
    const int n = (int) b->plans.size();
    b->stepwise.clear();
    b->inst_leaf_off.assign(n, 0);
    b->in_group.assign(n, 0);
    uint64_t off = 0;
    for (int i = 0; i < n; i++) {
        qt_plan *p = b->plans[i];
        if (!p->grouped || p->flops > b->stepwise_macs) {
            b->stepwise.push_back(i);
            continue;
        }
        b->in_group[i] = 1;
        qt_status s = upload_plan(p, prec);
        if (s != QT_OK) return s;
        b->inst_leaf_off[i] = off;
        off += (p->leaf_bytes[prec] + 255) / 256 * 256;
    }
    b->leaf_bytes = off;
    b->inst_angle_off.assign(n, 0);
    b->n_angles = 0;
    for (int i = 0; i < n; i++) {
        b->inst_angle_off[i] = b->n_angles;
        b->n_angles += (int64_t) b->plans[i]->rot_kind.size();
    }
    qt_status s = QT_OK;
    if (off) {
        s = host_alloc(ctx, off, &b->h_leaves);
        if (s == QT_OK) s = dev_alloc(ctx, off, &b->d_leaves);
    }
    if (s == QT_OK && n) {
        s = host_alloc(ctx, sizeof(double) * 2 * n, &b->h_values);
        if (s == QT_OK) s = dev_alloc(ctx, sizeof(double) * 2 * n, &b->d_values);
    }
    if (s == QT_OK) s = batch_configure(b);
    if (s == QT_OK) s = qt_batch_upload(b);   // packs the leaf images and copies them
    if (s == QT_OK) s = cuda_error(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (s != QT_OK) batch_release(b);
    b->dirty = false;
    return s;
}

qt_status qt_batch_upload(qt_batch *b) {
    if (!b || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    qt_status rs = resident_stop(b);   // the engine holds a staged copy of the leaves
    if (rs != QT_OK) return rs;
    batch_pack(b);
    if (!b->leaf_bytes) return QT_OK;
    return cuda_error(ctx, cudaMemcpyAsync(b->d_leaves, b->h_leaves, b->leaf_bytes, cudaMemcpyHostToDevice, ctx->stream),
                      "leaf upload");
}

static qt_status batch_launch(qt_batch *b, const void *instances = nullptr) {
    qt_ctx *ctx = b->ctx;
    const int n_grouped = (int) b->plans.size() - (int) b->stepwise.size();
    if (n_grouped <= 0) return QT_OK;
    PlanLaunch lp{};
    lp.instances = (const InstanceDesc *) (instances ? instances : b->d_inst);
    lp.n_instances = n_grouped;
    lp.ws_smem_bytes = b->ws_smem_bytes;
    lp.ws_base = (char *) b->d_ws;
    lp.ws_stride = b->ws_stride;
    lp.stage_bytes = b->stage_bytes;
    lp.tile_bytes = b->tile_bytes;
    lp.next = (uint32_t *) b->d_next;
    lp.header_steps = b->header_steps;
    cudaError_t e = cudaSuccess;
    if (lp.next) e = cudaMemsetAsync(lp.next, 0, sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = launch_plan(lp, b->prepared_prec == QT_PREC_MIXED, b->grid, ctx->stream, b->variant);
    ctx->launches++;
    return cuda_error(ctx, e, "plan kernel launch");
}

qt_status qt_batch_run(qt_batch *b) {
    if (!b || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    qt_status rs = resident_stop(b);   // the two must not rebuild the same leaves at once
    if (rs != QT_OK) return rs;
    if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
    if (b->use_graph && !b->graph && b->stepwise.empty()) {
        cudaGraph_t graph;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_error(ctx, e, "begin capture");
        qt_status s = batch_launch(b);
        e = cudaStreamEndCapture(ctx->stream, &graph);
        if (s != QT_OK) return s;
        if (e != cudaSuccess) return cuda_error(ctx, e, "end capture");
        e = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_error(ctx, e, "graph instantiate");
    }
    qt_status s;
    if (b->graph) {
        s = cuda_error(ctx, cudaGraphLaunch(b->graph, ctx->stream), "graph launch");
        ctx->launches++;
    } else {
        s = batch_launch(b);
    }
    if (s != QT_OK) return s;
    // plans too large for one CTA run step by step
    for (int i : b->stepwise) {
        double v[2];
        s = execute_stepwise(b->plans[i], ctx, b->prepared_prec, b->leaves[i].data(), v);
        if (s != QT_OK) return s;
        cudaMemcpyAsync((double *) b->d_values + 2 * i, v, 16, cudaMemcpyHostToDevice, ctx->stream);
    }
    return QT_OK;
}

// An instance whose staging copies did not arrive in time reports a NaN with
// the kStagingTimeoutBits payload: the call then fails instead of returning it.
static qt_status staging_status(qt_ctx *ctx, const double *v, size_t n) {
    for (size_t i = 0; i < n; i++) {
        uint64_t bits;
        std::memcpy(&bits, v + i, sizeof bits);
        if (bits == kStagingTimeoutBits) return set_error(ctx, QT_ERR_CUDA, "TMA staging wait timed out");
    }
    return QT_OK;
}

qt_status qt_batch_evaluate(qt_batch *b, const double *angles, int64_t n_angles, double *values) {
    if (!b || !values || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (b->res_idle > 0 && angles && n_angles > 0) {
        if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
        return resident_evaluate(b, angles, n_angles, values);
    }
    const bool one_graph = angles && n_angles > 0 && b->use_graph && b->stepwise.empty() &&
                           b->prepared_prec == QT_PREC_MIXED && !b->plans.empty();
    if (!one_graph) {
        qt_status s = angles ? qt_batch_set_rotations_device(b, angles, n_angles) : QT_OK;
        if (s == QT_OK) s = qt_batch_run(b);
        if (s == QT_OK) s = qt_batch_fetch(b, values);
        return s;
    }
    if (deadline_passed(ctx)) return set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
    if (!b->eval_graph) {
        // first call: the regular path sets up the angle buffers and the
        // descriptors, then the step is captured as one graph
        qt_status s = qt_batch_set_rotations_device(b, angles, n_angles);
        if (s == QT_OK) s = qt_batch_run(b);
        if (s == QT_OK) s = qt_batch_fetch(b, values);
        if (s != QT_OK) return s;
        // Zero-copy descriptors: the kernel reads the angles from, and writes the
        // values to, the pinned host buffers directly (GB300's coherent C2C link),
        // so the graph is the grouped launch alone -- no copy nodes.
        std::vector<InstanceDesc> zc = b->inst_desc;
        void *ha = nullptr, *hv = nullptr;
        cudaError_t e = cudaHostGetDevicePointer(&ha, b->h_angles, 0);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&hv, b->h_values, 0);
        if (e != cudaSuccess) return cuda_error(ctx, e, "mapped host buffers");
        for (size_t j = 0; j < zc.size(); j++) {
            const int i = b->inst_index[j];
            zc[j].angles = b->plans[i]->rot_kind.empty() ? nullptr
                                                         : static_cast<const double *>(ha) + b->inst_angle_off[i];
            zc[j].value = static_cast<double *>(hv) + 2 * i;
        }
        s = dev_alloc(ctx, sizeof(InstanceDesc) * zc.size(), &b->d_inst_eval);
        if (s != QT_OK) return s;
        e = cudaMemcpyAsync(b->d_inst_eval, zc.data(), sizeof(InstanceDesc) * zc.size(), cudaMemcpyHostToDevice,
                            ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_error(ctx, e, "instance descriptor upload");
        cudaGraph_t graph;
        e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_error(ctx, e, "begin capture");
        s = batch_launch(b, b->d_inst_eval);
        e = cudaStreamEndCapture(ctx->stream, &graph);
        if (s != QT_OK) return s;
        if (e != cudaSuccess) return cuda_error(ctx, e, "end capture");
        e = cudaGraphInstantiate(&b->eval_graph, graph, 0);
        cudaGraphDestroy(graph);
        return cuda_error(ctx, e, "graph instantiate");
    }
    if (n_angles != b->n_angles) return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "angle count does not match the batch");
    qt_status s = batch_device_rotations(b, true);
    if (s != QT_OK) return s;
    // the previous evaluation finished (stream synchronised), so the pinned
    // copies are free
    std::memcpy(b->h_angles, angles, sizeof(double) * n_angles);
    cudaError_t e = cudaGraphLaunch(b->eval_graph, ctx->stream);
    ctx->launches++;
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "evaluation graph");
    std::memcpy(values, b->h_values, sizeof(double) * 2 * b->plans.size());
    return staging_status(ctx, values, 2 * b->plans.size());
}

qt_status qt_batch_fetch(qt_batch *b, double *values) {
    if (!b || !values || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    const size_t bytes = sizeof(double) * 2 * b->plans.size();
    if (!bytes) return QT_OK;
    cudaError_t e = cudaMemcpyAsync(b->h_values, b->d_values, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "value download");
    std::memcpy(values, b->h_values, bytes);
    return staging_status(ctx, values, 2 * b->plans.size());
}

qt_status qt_batch_execute(qt_batch *b, qt_precision prec, double *values) {
    if (!b || !values) return QT_ERR_INVALID_ARGUMENT;
    qt_status s = QT_OK;
    if (b->dirty || b->prepared_prec != (int) prec) s = qt_batch_prepare(b, prec);
    else s = qt_batch_upload(b);
    if (s == QT_OK) s = qt_batch_run(b);
    if (s == QT_OK) s = qt_batch_fetch(b, values);
    return s;
}

qt_status qt_batch_use_graph(qt_batch *b, int enable) {
    if (!b) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(b->ctx->lock);
    b->use_graph = enable != 0;
    if (!b->use_graph && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->use_graph && b->eval_graph) {
        cudaGraphExecDestroy(b->eval_graph);
        b->eval_graph = nullptr;
    }
    return QT_OK;
}

qt_status qt_batch_use_resident(qt_batch *b, double idle_seconds) {
    if (!b) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (!(idle_seconds > 0)) {
        b->res_idle = 0;
        return resident_stop(b);
    }
    if (b->prepared_prec != QT_PREC_MIXED)
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "resident evaluation needs a batch prepared for QT_PREC_MIXED");
    if (!b->stepwise.empty() || b->inst_desc.empty())
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "resident evaluation needs every instance in the grouped launch");
    const size_t smem = plan_header_bytes(b->header_steps) + 128 + b->ws_smem_bytes + b->stage_bytes + b->tile_bytes;
    if ((int) b->inst_desc.size() > b->grid || (int) b->inst_desc.size() > resident_capacity(smem, b->variant))
        return set_error(ctx, QT_ERR_INVALID_ARGUMENT, "resident evaluation needs one resident CTA per instance");
    qt_status s = resident_stop(b);   // a new idle limit takes effect at the next start
    b->res_idle = std::min(idle_seconds, 3600.0);
    return s;
}

uint64_t qt_batch_resident_starts(const qt_batch *b) { return b ? b->res_starts : 0; }

uint64_t qt_batch_h2d_bytes(const qt_batch *b) {
    if (!b) return 0;
    return b->dev_rot ? sizeof(double) * (uint64_t) b->n_angles : b->leaf_bytes;
}
uint64_t qt_batch_d2h_bytes(const qt_batch *b) { return b ? sizeof(double) * 2 * b->plans.size() : 0; }

int qt_batch_launches_per_run(const qt_batch *b) {
    if (!b) return 0;
    int n = ((int) b->plans.size() - (int) b->stepwise.size()) > 0 ? 1 : 0;
    for (int i : b->stepwise) n += b->plans[i]->n_steps;
    return n;
}

qt_status qt_batch_set_launch_policy(qt_batch *b, const qt_launch_policy *policy) {
    if (!b || !policy || policy->ctas_per_sm < 0 || (policy->static_schedule != 0 && policy->static_schedule != 1) ||
        (policy->kernel_ctas != 0 && std::find(std::begin(kPlanVariants), std::end(kPlanVariants),
                                               policy->kernel_ctas) == std::end(kPlanVariants)))
        return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::recursive_mutex> g(b->ctx->lock);
    const qt_launch_policy old = b->policy;
    b->policy = *policy;
    if (b->prepared_prec < 0) return QT_OK;
    qt_status s = batch_configure(b);
    if (s != QT_OK) {
        const std::string why = b->ctx->last_error;
        b->policy = old;
        if (batch_configure(b) != QT_OK) batch_release(b);
        set_error(b->ctx, s, why);
    }
    return s;
}

qt_status qt_batch_get_launch_policy(const qt_batch *b, qt_launch_policy *policy) {
    if (!b || !policy) return QT_ERR_INVALID_ARGUMENT;
    *policy = b->policy;
    return QT_OK;
}

qt_status qt_batch_launch_info(const qt_batch *b, qt_launch_info *info) {
    if (!b || !info || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_launch_info r{};
    r.grid = b->inst_desc.empty() ? 0 : b->grid;
    r.n_grouped = (int32_t) b->inst_desc.size();
    r.n_stepwise = (int32_t) b->stepwise.size();
    r.dynamic_schedule = b->d_next != nullptr;
    for (const InstanceDesc &d : b->inst_desc) {
        r.n_ws_smem += d.ws_bytes <= b->ws_smem_bytes;
        r.n_staged += b->stage_bytes && d.plan_bytes && d.plan_bytes + d.leaf_bytes <= b->stage_bytes;
    }
    r.ws_smem_bytes = b->ws_smem_bytes;
    r.stage_bytes = b->stage_bytes;
    r.tile_bytes = b->tile_bytes;
    r.smem_bytes = plan_header_bytes(b->header_steps) + 128 + b->ws_smem_bytes + b->stage_bytes + b->tile_bytes;
    r.ws_slab_bytes = b->d_ws ? b->ws_stride * (uint64_t) b->grid : 0;
    r.kernel_ctas = b->variant;
    *info = r;
    return QT_OK;
}

// Times one grouped launch of the configured batch: one untimed launch, then
// the median of `reps` launches bracketed by events on the context stream.
static qt_status time_grouped_launch(qt_batch *b, int reps, cudaEvent_t e0, cudaEvent_t e1, double *us) {
    qt_ctx *ctx = b->ctx;
    qt_status s = batch_launch(b);
    std::vector<float> t;
    for (int r = 0; r < reps && s == QT_OK; r++) {
        cudaError_t e = cudaEventRecord(e0, ctx->stream);
        if (e == cudaSuccess) s = batch_launch(b);
        if (s != QT_OK) break;
        e = cudaEventRecord(e1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) return cuda_error(ctx, e, "autotune timing");
        t.push_back(ms);
    }
    if (s != QT_OK) return s;
    std::sort(t.begin(), t.end());
    *us = 1e3 * t[t.size() / 2];
    return QT_OK;
}

qt_status qt_batch_autotune(qt_batch *b, int reps, qt_launch_policy *chosen, double *best_us) {
    if (!b || reps < 0 || b->prepared_prec < 0) return QT_ERR_INVALID_ARGUMENT;
    qt_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (reps == 0) reps = 3;
    double best_t = 0;
    if (b->inst_desc.empty()) {   // nothing in the grouped launch
        if (chosen) *chosen = b->policy;
        if (best_us) *best_us = 0;
        return QT_OK;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return cuda_error(ctx, ce, "autotune events");
    }
    // candidates differ in what they resolve to: skip policies that give a
    // configuration already timed
    auto key = [&]() {
        return std::to_string(b->ws_smem_bytes) + "/" + std::to_string(b->stage_bytes) + "/" +
               std::to_string(b->grid) + "/" + std::to_string(b->d_next != nullptr) + "/" + std::to_string(b->variant);
    };
    std::set<std::string> tried;
    qt_launch_policy best = b->policy;
    qt_status s = batch_configure(b);
    if (s == QT_OK) s = time_grouped_launch(b, reps, e0, e1, &best_t);
    // short launches are noisy: enough repetitions for about 2 ms per
    // candidate; launches of several milliseconds need one
    if (s == QT_OK && best_t * reps < 2000.0) {
        reps = std::min(200, (int) std::ceil(2000.0 / std::max(best_t, 1.0)));
        s = time_grouped_launch(b, reps, e0, e1, &best_t);
    } else if (best_t > 5000.0) {
        reps = 1;
    }
    tried.insert(key());
    // the search stops taking new candidates after about three seconds
    const auto t_start = std::chrono::steady_clock::now();
    const int n_grouped = (int) b->inst_desc.size();
    auto try_policy = [&](const qt_launch_policy &cand) -> qt_status {
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() > 3.0) return QT_OK;
        b->policy = cand;
        qt_status cs = batch_configure(b);
        if (cs == QT_ERR_INVALID_ARGUMENT) return QT_OK;   // does not fit a CTA: not a candidate
        if (cs != QT_OK) return cs;
        // with more instances than CTAs, shared memory that leaves fewer CTAs
        // per SM than the register budget allows only loses warps
        if (cand.ctas_per_sm == 0 && n_grouped > b->grid && b->grid < plan_num_sms() * b->variant) return QT_OK;
        if (!tried.insert(key()).second) return QT_OK;
        double t = 0;
        cs = time_grouped_launch(b, reps, e0, e1, &t);
        if (cs == QT_OK && t < 0.99 * best_t) {
            best_t = t;
            best = cand;
        }
        return cs;
    };
    // register budget and shared-memory regions together (they trade against
    // each other for CTAs per SM), then CTAs per SM and the schedule
    const int32_t ws_caps[] = {0, 8 << 10, 16 << 10, 32 << 10, 48 << 10, 64 << 10, 96 << 10};
    const int32_t stage_caps[] = {0, 24 << 10, 52 << 10, 64 << 10, 96 << 10, 144 << 10};
    const qt_launch_policy start = best;
    for (int32_t v : kPlanVariants)
        for (int32_t w : ws_caps)
            for (int32_t st : stage_caps) {
                qt_launch_policy cand = start;
                cand.kernel_ctas = v;
                cand.ws_smem_cap = w;
                cand.stage_cap = st;
                if (s == QT_OK) s = try_policy(cand);
            }
    for (int32_t c : {1, 2, 3}) {
        qt_launch_policy cand = best;
        cand.ctas_per_sm = c;
        if (s == QT_OK) s = try_policy(cand);
    }
    for (int32_t c : {0, 1}) {
        qt_launch_policy cand = best;
        cand.static_schedule = c;
        if (s == QT_OK) s = try_policy(cand);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->policy = best;
    if (s == QT_OK) s = batch_configure(b);
    if (s == QT_OK) s = batch_launch(b);   // leave the values of the current leaves
    if (s == QT_OK) s = cuda_error(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (s == QT_OK && chosen) *chosen = best;
    if (s == QT_OK && best_us) *best_us = best_t;
    return s;
}

}  // extern "C"
