// Index slicing of a plan (no reference counterpart; the heavy tail of a
// request stream under a device-memory budget).
//
// A contraction whose intermediates do not fit a budget is split over the
// values of a few wires.  Fixing wire w to v cuts w from its two leaves (each
// keeps the slice of its tensor at index v), the recorded sequence is replayed
// on the cut network -- a pair that shared only cut wires becomes an outer
// product -- and the network's value is the sum of the 4^s sliced values over
// every assignment of the s cut wires, because the value is linear in each
// leaf.  Every intermediate that carried a cut wire is 4x smaller per cut.
//
// Cut wires are chosen greedily: among wires whose cut leaves every leaf and
// every intermediate but the final one with at least one wire (so the
// final-value rule of src/Network.h:961-965 still sees one rank-0 result per
// slice), the one carried by the largest intermediates (sum of 4^rank), until
// the sliced plan's workspace fits.
#include <algorithm>
#include <complex>
#include <map>
#include <memory>
#include <vector>

#include "../../include/qtorch/qtorch.hpp"
#include "core.h"
#include "plan.h"

struct qt_sliced {
    explicit qt_sliced(qt_ctx *c) : ctx(c) { qtg::ctx_retain(ctx); }
    ~qt_sliced() { qtg::ctx_release(ctx); }
    qt_sliced(const qt_sliced &) = delete;
    qt_sliced &operator=(const qt_sliced &) = delete;
    qt_ctx *ctx = nullptr;
    qt_plan *plan = nullptr;                          // lowered on the cut network
    struct End {
        int leaf, pos;                                // leaf index and wire position in the uncut network
    };
    std::vector<std::pair<End, End>> cuts;
    std::vector<int> orig_rank;                       // uncut leaves
    std::vector<uint64_t> orig_off;
    std::vector<std::complex<double>> orig_vals;
    qt_batch *batch = nullptr;                        // one instance per assignment
    int batch_prec = -1;
};

namespace {

using C = std::complex<double>;
using End = qt_sliced::End;

// the tensor of a leaf with the wires at `pos` (ascending) fixed to `val`
std::vector<C> restrict_leaf(const C *t, int rank, const std::vector<int> &pos, const std::vector<int> &val) {
    std::vector<int> keep;
    for (int j = 0; j < rank; j++)
        if (std::find(pos.begin(), pos.end(), j) == pos.end()) keep.push_back(j);
    uint64_t base = 0;
    for (size_t i = 0; i < pos.size(); i++) base += (uint64_t) val[i] << (2 * pos[i]);
    std::vector<C> out((size_t) 1 << (2 * keep.size()));
    for (uint64_t x = 0; x < out.size(); x++) {
        uint64_t off = base;
        for (size_t i = 0; i < keep.size(); i++) off += ((x >> (2 * i)) & 3ull) << (2 * keep[i]);
        out[x] = t[off];
    }
    return out;
}

// positions (ascending) and values of the cut wires of each leaf for one assignment
void cut_positions(const std::vector<std::pair<End, End>> &cuts, uint64_t assignment, size_t n_leaves,
                   std::vector<std::vector<int>> &pos, std::vector<std::vector<int>> &val) {
    std::vector<std::vector<std::pair<int, int>>> per(n_leaves);
    for (size_t c = 0; c < cuts.size(); c++) {
        const int v = (int) ((assignment >> (2 * c)) & 3u);
        per[cuts[c].first.leaf].push_back({cuts[c].first.pos, v});
        per[cuts[c].second.leaf].push_back({cuts[c].second.pos, v});
    }
    pos.assign(n_leaves, {});
    val.assign(n_leaves, {});
    for (size_t l = 0; l < n_leaves; l++) {
        std::sort(per[l].begin(), per[l].end());
        for (auto &pv : per[l]) {
            pos[l].push_back(pv.first);
            val[l].push_back(pv.second);
        }
    }
}

std::vector<std::pair<int, int>> sequence_pairs(const qt_plan *p) {
    std::vector<std::pair<int, int>> seq(p->sequence.size() / 2);
    for (size_t i = 0; i < seq.size(); i++) seq[i] = {p->sequence[2 * i], p->sequence[2 * i + 1]};
    return seq;
}

// The plan of the network with the given wires cut (assignment 0 for its own leaves).
qt_status build_cut_plan(qt_ctx *ctx, const qt_plan *p, const std::vector<std::pair<End, End>> &cuts, qt_plan **out) {
    auto net = qtorch::Network::FromText(p->qasm, p->measure, p->gate_dir, nullptr);
    const auto &leaves = net->Leaves();
    std::vector<std::vector<int>> pos, val;
    cut_positions(cuts, 0, leaves.size(), pos, val);
    for (size_t l = 0; l < leaves.size(); l++) {
        if (pos[l].empty()) continue;
        auto &node = *leaves[l];
        auto &vals = node.GetTensorVals();
        vals = restrict_leaf(vals.data(), node.mRank, pos[l], val[l]);
        auto &wires = node.GetWires();
        for (auto it = pos[l].rbegin(); it != pos[l].rend(); ++it) wires.erase(wires.begin() + *it);
        node.mRank -= (int) pos[l].size();
    }
    auto q = std::make_unique<qt_plan>(ctx);
    q->qasm = p->qasm;
    q->measure = p->measure;
    q->gate_dir = p->gate_dir;
    qtg::plan_collect_leaves(q.get(), *net);   // before the replay releases the leaves' data
    net->AllowOuterProducts(true);
    qtorch::ContractionTools t(net);
    t.ContractGivenSequence(sequence_pairs(p));
    if (!net->IsDone()) return QT_ERR_CONTRACTION_FAILURE;
    qt_status s = qtg::plan_finish(q.get(), *net);
    if (s != QT_OK) return s;
    *out = q.release();
    return QT_OK;
}

template <class F>
qt_status guarded(qt_ctx *ctx, F &&f) {
    try {
        return f();
    } catch (const qtorch::ContractionFailure &) {
        return qtg::set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "the sliced network's sequence failed");
    } catch (const std::bad_alloc &) {
        return qtg::set_error(ctx, QT_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception &e) {
        return qtg::set_error(ctx, QT_ERR_INVALID_ARGUMENT, e.what());
    }
}

}  // namespace

extern "C" {

qt_status qt_plan_slice(qt_ctx *ctx, const qt_plan *p, qt_precision prec, uint64_t max_workspace_bytes,
                        int max_cuts, qt_sliced **out) {
    if (!p || !out || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED) || max_cuts < 0 || max_cuts > 16)
        return QT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guarded(ctx, [&]() -> qt_status {
        // the uncut network, replayed, to see which wires each intermediate carries
        auto net = qtorch::Network::FromText(p->qasm, p->measure, p->gate_dir, nullptr);
        std::map<const qtorch::Wire *, int> wire_id;
        std::vector<std::pair<End, End>> ends;
        const auto leaves = net->Leaves();
        for (size_t l = 0; l < leaves.size(); l++) {
            auto &ws = leaves[l]->GetWires();
            for (size_t k = 0; k < ws.size(); k++) {
                auto it = wire_id.find(ws[k].get());
                if (it == wire_id.end()) {
                    wire_id[ws[k].get()] = (int) ends.size();
                    ends.push_back({{(int) l, (int) k}, {-1, -1}});
                } else {
                    ends[it->second].second = {(int) l, (int) k};
                }
            }
        }
        qtorch::ContractionTools t(net);
        t.ContractGivenSequence(sequence_pairs(p));
        if (!net->IsDone()) return qtg::set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "the plan's sequence does not finish");
        std::vector<std::vector<int>> inter;   // wires of every intermediate but the final one
        for (const auto &node : net->GetAllNodes()) {
            if (node->mCreatedFrom.first == 0 && node->mCreatedFrom.second == 0) continue;
            if (node->GetWires().empty()) continue;
            std::vector<int> w;
            for (auto &x : node->GetWires()) w.push_back(wire_id.at(x.get()));
            inter.push_back(w);
        }
        std::vector<int> leaf_rank(leaves.size());
        for (size_t l = 0; l < leaves.size(); l++) leaf_rank[l] = (int) leaves[l]->GetWires().size();
        std::vector<char> cut(ends.size(), 0);
        std::vector<std::pair<End, End>> chosen;
        auto sliced = std::make_unique<qt_sliced>(ctx);
        sliced->orig_rank = p->leaf_rank;
        uint64_t off = 0;
        for (int r : sliced->orig_rank) {
            sliced->orig_off.push_back(off);
            off += 1ull << (2 * r);
        }
        sliced->orig_vals = p->leaf_values;
        qt_plan *plan = nullptr;
        qt_status s = build_cut_plan(ctx, p, chosen, &plan);
        while (s == QT_OK && plan->ws_bytes[prec] > max_workspace_bytes) {
            if ((int) chosen.size() >= max_cuts) {
                qt_plan_free(plan);
                return qtg::set_error(ctx, QT_ERR_OUT_OF_MEMORY, "no slicing within the cut limit fits the workspace budget");
            }
            // the wire carried by the largest intermediates whose cut keeps every
            // leaf and every intermediate but the last at rank >= 1
            int best = -1;
            double best_score = 0;
            for (size_t w = 0; w < ends.size(); w++) {
                if (cut[w] || ends[w].second.leaf < 0) continue;
                if (leaf_rank[ends[w].first.leaf] < 2 || leaf_rank[ends[w].second.leaf] < 2) continue;
                double score = 0;
                bool ok = true;
                for (const auto &iw : inter) {
                    if (std::find(iw.begin(), iw.end(), (int) w) == iw.end()) continue;
                    int r = 0;
                    for (int x : iw) r += !cut[x];
                    if (r < 2) ok = false;
                    score += (double) (1ull << (2 * std::min(r, 30)));
                }
                if (ok && score > best_score) {
                    best_score = score;
                    best = (int) w;
                }
            }
            if (best < 0) {
                qt_plan_free(plan);
                return qtg::set_error(ctx, QT_ERR_OUT_OF_MEMORY, "no wire left to slice");
            }
            cut[best] = 1;
            leaf_rank[ends[best].first.leaf]--;
            leaf_rank[ends[best].second.leaf]--;
            chosen.push_back(ends[best]);
            qt_plan_free(plan);
            plan = nullptr;
            s = build_cut_plan(ctx, p, chosen, &plan);
        }
        if (s != QT_OK) return qtg::set_error(ctx, s, "slicing");
        sliced->plan = plan;
        sliced->cuts = chosen;
        *out = sliced.release();
        return QT_OK;
    });
}

int qt_sliced_num_cuts(const qt_sliced *s) { return s ? (int) s->cuts.size() : -1; }
qt_plan *qt_sliced_plan(const qt_sliced *s) { return s ? s->plan : nullptr; }

}  // extern "C"

namespace {

// Slices per batch: a sliced plan with more assignments runs them in chunks of
// this many (each chunk one batch), so the host and device hold the leaves of
// at most this many slices at a time.
constexpr uint64_t kSliceChunk = 4096;

// A batch of slices a0 .. a1-1 of `s` built from the uncut leaves `orig` (the
// plan's leaf order), on ctx.  stepwise_macs: instances above it run step by
// step, one at a time.
qt_status slice_batch(qt_ctx *ctx, const qt_sliced *s, const C *orig, int64_t stepwise_macs, uint64_t a0,
                      uint64_t a1, qt_batch **out) {
    qt_batch *b = nullptr;
    qt_status st = qt_batch_create(ctx, &b);
    if (st != QT_OK) return st;
    b->stepwise_macs = stepwise_macs;
    const size_t n_leaves = s->orig_rank.size();
    for (uint64_t a = a0; a < a1 && st == QT_OK; a++) {
        std::vector<std::vector<int>> pos, val;
        cut_positions(s->cuts, a, n_leaves, pos, val);
        std::vector<C> leaves;
        leaves.reserve(s->plan->leaf_values.size());
        for (size_t l = 0; l < n_leaves; l++) {
            const C *t = orig + s->orig_off[l];
            if (pos[l].empty()) {
                leaves.insert(leaves.end(), t, t + (1ull << (2 * s->orig_rank[l])));
            } else {
                auto r = restrict_leaf(t, s->orig_rank[l], pos[l], val[l]);
                leaves.insert(leaves.end(), r.begin(), r.end());
            }
        }
        if (leaves.size() != s->plan->leaf_values.size())
            st = qtg::set_error(ctx, QT_ERR_INVALID_ARGUMENT, "sliced leaves do not match the slice's plan");
        int idx = 0;
        if (st == QT_OK) st = qt_batch_add(b, s->plan, reinterpret_cast<const double *>(leaves.data()), &idx);
    }
    if (st != QT_OK) {
        qt_batch_free(b);
        return st;
    }
    *out = b;
    return QT_OK;
}

// the values of a batch of n slices added, in assignment order, to re_im
qt_status add_slices(qt_batch *b, uint64_t n, double *re_im) {
    std::vector<double> v(2 * n);
    qt_status st = qt_batch_run(b);
    if (st == QT_OK) st = qt_batch_fetch(b, v.data());
    if (st != QT_OK) return st;
    for (uint64_t a = 0; a < n; a++) {
        re_im[0] += v[2 * a];
        re_im[1] += v[2 * a + 1];
    }
    return QT_OK;
}

// every slice, chunk by chunk, summed in assignment order
qt_status run_chunks(qt_ctx *ctx, const qt_sliced *s, const C *orig, int64_t stepwise_macs, qt_precision prec,
                     double *re_im) {
    const uint64_t n = 1ull << (2 * s->cuts.size());
    double acc[2] = {0.0, 0.0};
    for (uint64_t a0 = 0; a0 < n; a0 += kSliceChunk) {
        const uint64_t a1 = std::min(n, a0 + kSliceChunk);
        qt_batch *b = nullptr;
        qt_status st = slice_batch(ctx, s, orig, stepwise_macs, a0, a1, &b);
        if (st == QT_OK) st = qt_batch_prepare(b, prec);
        if (st == QT_OK) st = add_slices(b, a1 - a0, acc);
        if (b) qt_batch_free(b);
        if (st != QT_OK) return st;
    }
    re_im[0] = acc[0];
    re_im[1] = acc[1];
    return QT_OK;
}

}  // namespace

extern "C" {

qt_status qt_sliced_execute(qt_sliced *s, qt_precision prec, double *re_im) {
    if (!s || !re_im || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return QT_ERR_INVALID_ARGUMENT;
    if (!s->ctx) return QT_ERR_INVALID_ARGUMENT;   // built for inspection only
    const uint64_t n = 1ull << (2 * s->cuts.size());
    // instances that are large for one CTA run step by step, one at a time
    if (n > kSliceChunk) return run_chunks(s->ctx, s, s->orig_vals.data(), qtg::kLoneInstanceMaxMacs, prec, re_im);
    if (!s->batch || s->batch_prec != (int) prec) {
        if (s->batch) qt_batch_free(s->batch);
        s->batch = nullptr;
        qt_status st = slice_batch(s->ctx, s, s->orig_vals.data(), qtg::kLoneInstanceMaxMacs, 0, n, &s->batch);
        if (st == QT_OK) st = qt_batch_prepare(s->batch, prec);
        if (st != QT_OK) return st;
        s->batch_prec = (int) prec;
    }
    re_im[0] = re_im[1] = 0.0;
    return add_slices(s->batch, n, re_im);
}

qt_status qt_sliced_execute_leaves(qt_ctx *ctx, const qt_sliced *s, qt_precision prec, const double *leaves,
                                   double *re_im) {
    if (!ctx || !s || !re_im || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return QT_ERR_INVALID_ARGUMENT;
    // every slice step by step, one at a time: the device holds one slice's workspace
    return run_chunks(ctx, s, leaves ? reinterpret_cast<const C *>(leaves) : s->orig_vals.data(), -1, prec, re_im);
}

qt_status qt_sliced_free(qt_sliced *s) {
    if (!s) return QT_ERR_INVALID_ARGUMENT;
    if (s->batch) qt_batch_free(s->batch);
    if (s->plan) qt_plan_free(s->plan);
    delete s;
    return QT_OK;
}

}  // extern "C"
