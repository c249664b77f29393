// Plans and batches: an ordering is run once over a symbolic copy of the
// network (the same ContractNodes bookkeeping, no data), every contraction is
// recorded, and the record is lowered to device step descriptors:
//   * steps are grouped into dependency levels (all steps of a level are
//     independent and run concurrently inside one CTA);
//   * intermediates get workspace offsets from a first-fit allocator driven by
//     liveness across levels;
//   * leaves (state, gate and measurement tensors) are bound per instance, so
//     one plan serves every parameter point of a circuit structure.
// Small plans run in the grouped interpreter (one CTA per instance, one launch
// for a whole batch); plans with large intermediates run step by step with the
// whole-GPU pairwise kernel.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>

#include "kernels.h"

namespace qtg {

static uint64_t align_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

// first-fit allocator over a linear workspace
class OffsetAllocator {
public:
    uint64_t alloc(uint64_t bytes) {
        bytes = align_up(bytes ? bytes : 1, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const uint64_t off = it->first, sz = it->second;
                free_.erase(it);
                if (sz > bytes) free_[off + bytes] = sz - bytes;
                return off;
            }
        }
        const uint64_t off = top_;
        top_ += bytes;
        return off;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = align_up(bytes ? bytes : 1, 256);
        auto it = free_.emplace(off, bytes).first;
        // coalesce with the next and the previous block
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t high_water() const { return top_; }
private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t top_ = 0;
};

// A step runs CTA-wide as a tiled product when C's digits are A's free wires
// followed by B's (the ContractNodes order) and both sides give at least 16
// rows (an output of at least one element per thread).  Its operand slices are
// gathered once per chunk of the sum and reused across the tile, where work
// items would each load their own operands: with workspaces in global memory
// this took the 16-point batched QAOA step from 2.15 to 1.92 ms (requiring 4
// elements per thread instead).
static bool cta_tiled(const qtorch::StepRecord &r) {
    int fa = 0, fb = 0;
    for (size_t i = 0; i < r.freeIdx.size(); i++) {
        if (r.freeIdx[i].first) {
            if (fb) return false;   // an A wire after a B wire
            fa++;
        } else {
            fb++;
        }
    }
    return fa >= 2 && fb >= 2 && !r.sumIdx.empty();
}

qt_status lower_plan(qt_plan *p, const qtorch::Network &net) {
    const auto &leaves = net.Leaves();
    const auto &rec = net.Steps();
    const int L = (int) leaves.size();
    const int S = (int) rec.size();
    // tensor ids: leaves 0..L-1, then one per step in creation order
    std::map<int64_t, int> producer;   // tensor id -> step (contraction order)
    for (int s = 0; s < S; s++) producer[rec[s].c] = s;
    std::vector<int> level(S, 0);
    int n_levels = 0;
    for (int s = 0; s < S; s++) {
        int la = 0, lb = 0;
        auto ia = producer.find(rec[s].a), ib = producer.find(rec[s].b);
        if (ia != producer.end()) la = level[ia->second];
        if (ib != producer.end()) lb = level[ib->second];
        level[s] = 1 + std::max(la, lb);
        n_levels = std::max(n_levels, level[s]);
    }
    std::vector<int> order(S);
    std::vector<bool> tiled(S);
    for (int s = 0; s < S; s++) {
        order[s] = s;
        tiled[s] = cta_tiled(rec[s]);
    }
    // by level; inside a level the CTA-tiled steps come last
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return level[x] != level[y] ? level[x] < level[y] : (!tiled[x] && tiled[y]);
    });
    std::vector<int> sorted_of(S);
    for (int i = 0; i < S; i++) sorted_of[order[i]] = i;
    // consumer level of every intermediate tensor
    std::map<int64_t, int> consumer_level;
    for (int s = 0; s < S; s++) {
        consumer_level[rec[s].a] = level[s];
        consumer_level[rec[s].b] = level[s];
    }
    p->level_start.assign(n_levels + 1, 0);
    p->level_cta.assign(n_levels, 0);
    p->n_tiled = 0;
    for (int i = 0, L0 = 1; L0 <= n_levels; L0++) {
        p->level_start[L0 - 1] = i;
        while (i < S && level[order[i]] == L0 && !tiled[order[i]]) i++;
        p->level_cta[L0 - 1] = i;
        while (i < S && level[order[i]] == L0) {
            i++;
            p->n_tiled++;
        }
        p->level_start[L0] = i;
    }
    p->rank0_steps.clear();
    for (int s = 0; s < S; s++)
        if (rec[s].freeIdx.empty()) p->rank0_steps.push_back(sorted_of[s]);

    p->peak_rank = 0;
    p->flops = 0;
    p->max_step_out = 0;
    p->max_step_k = 0;
    for (int s = 0; s < S; s++) {
        p->peak_rank = std::max<int>(p->peak_rank, (int) rec[s].freeIdx.size());
        p->flops += (int64_t) 1 << (2 * (rec[s].freeIdx.size() + rec[s].sumIdx.size()));
        p->max_step_out = std::max<int>(p->max_step_out, (int) rec[s].freeIdx.size());
        p->max_step_k = std::max<int>(p->max_step_k, (int) rec[s].sumIdx.size());
    }
    for (int i = 0; i < L; i++) p->peak_rank = std::max(p->peak_rank, leaves[i]->mRank);

    for (int prec = 0; prec < 2; prec++) {
        const bool mixed = prec == QT_PREC_MIXED;
        // leaf layout
        uint64_t loff = 0;
        std::vector<uint64_t> leaf_off(L);
        for (int i = 0; i < L; i++) {
            leaf_off[i] = loff;
            loff = align_up(loff + ((uint64_t) (mixed ? 8 : 16) << (2 * leaves[i]->mRank)), 16);
        }
        p->leaf_bytes[prec] = loff;
        p->leaf_off[prec] = leaf_off;
        p->rot_table[prec].clear();
        for (size_t r = 0; r < p->rot_kind.size(); r++) {
            const std::string &k = p->rot_kind[r];
            const uint32_t kind = k == "Rx" ? kRotRx : k == "Ry" ? kRotRy : k == "CPHASE" ? kRotCPhase : kRotRz;
            p->rot_table[prec].push_back(make_uint2((uint32_t) leaf_off[p->rot_leaf[r]], kind));
        }
        // workspace layout, level by level
        OffsetAllocator alloc;
        std::map<int64_t, std::pair<uint64_t, uint64_t>> live;   // tensor id -> (offset, bytes)
        std::vector<uint64_t> c_off(S), c_bytes(S);
        std::vector<bool> c_f64(S);
        std::vector<uint64_t> shadow(S, 0);   // mixed: offset of the complex64 copy of a complex128 output
        std::map<int64_t, bool> rank0_out;
        for (int s = 0; s < S; s++) rank0_out[rec[s].c] = rec[s].freeIdx.empty();
        for (int L0 = 1; L0 <= n_levels; L0++) {
            for (auto it = live.begin(); it != live.end();) {
                auto cl = consumer_level.find(it->first);
                // rank-0 outputs stay: the final-value rule reads all of them at the end
                const bool keep = rank0_out[it->first];
                if (!keep && cl != consumer_level.end() && cl->second < L0) {
                    alloc.release(it->second.first, it->second.second);
                    it = live.erase(it);
                } else {
                    ++it;
                }
            }
            for (int i = p->level_start[L0 - 1]; i < p->level_start[L0]; i++) {
                const int s = order[i];
                const int nf = (int) rec[s].freeIdx.size();
                // mixed plans keep the expectation-value reductions in twice-FP32 accuracy
                const int ns = (int) rec[s].sumIdx.size();
                const bool f64 = !mixed || nf == 0 || (nf <= kMixedTailRank && ns >= kMixedTailMinSum);
                // a mixed complex128 output carries a complex64 copy for its consumers,
                // which then never convert on the (narrow) FP64 pipe
                const uint64_t bytes = (uint64_t) (f64 ? (mixed ? 24 : 16) : 8) << (2 * nf);
                c_off[s] = alloc.alloc(bytes);
                if (mixed && f64) shadow[s] = c_off[s] + (16ull << (2 * nf));
                c_bytes[s] = bytes;
                c_f64[s] = f64;
                live[rec[s].c] = {c_off[s], bytes};
            }
        }
        p->ws_bytes[prec] = align_up(alloc.high_water(), 256);
        // descriptors in sorted order
        std::vector<StepDesc> &steps = p->steps[prec];
        steps.assign(S, StepDesc());
        p->a_leaf.assign(S, -1);
        p->b_leaf.assign(S, -1);
        for (int i = 0; i < S; i++) {
            const int s = order[i];
            const auto &r = rec[s];
            std::vector<uint8_t> ffa(r.freeIdx.size());
            std::vector<int32_t> fi(r.freeIdx.size()), sa(r.sumIdx.size()), sb(r.sumIdx.size());
            for (size_t k = 0; k < r.freeIdx.size(); k++) {
                ffa[k] = r.freeIdx[k].first;
                fi[k] = r.freeIdx[k].second;
            }
            for (size_t k = 0; k < r.sumIdx.size(); k++) {
                sa[k] = r.sumIdx[k].first;
                sb[k] = r.sumIdx[k].second;
            }
            StepDesc &d = steps[i];
            qt_status st = make_step(r.rankA, r.rankB, (int) ffa.size(), ffa.data(), fi.data(), (int) sa.size(),
                                     sa.data(), sb.data(), &d);
            if (st != QT_OK) return st;
            auto ia = producer.find(r.a), ib = producer.find(r.b);
            d.flags = 0;
            if (ia == producer.end()) {
                d.flags |= kALeaf;
                d.a_off = (int64_t) leaf_off[r.a];
                p->a_leaf[i] = (int) r.a;
                d.a_step = -1;
                if (!mixed) d.flags |= kAF64;
            } else {
                d.a_off = (int64_t) c_off[ia->second];
                d.a_step = sorted_of[ia->second];
                if (c_f64[ia->second]) {
                    if (mixed) d.a_off = (int64_t) shadow[ia->second];
                    else d.flags |= kAF64;
                }
            }
            if (ib == producer.end()) {
                d.flags |= kBLeaf;
                d.b_off = (int64_t) leaf_off[r.b];
                p->b_leaf[i] = (int) r.b;
                d.b_step = -1;
                if (!mixed) d.flags |= kBF64;
            } else {
                d.b_off = (int64_t) c_off[ib->second];
                d.b_step = sorted_of[ib->second];
                if (c_f64[ib->second]) {
                    if (mixed) d.b_off = (int64_t) shadow[ib->second];
                    else d.flags |= kBF64;
                }
            }
            d.c_off = (int64_t) c_off[s];
            if (c_f64[s]) d.flags |= kCF64;
            if (r.freeIdx.empty()) d.flags |= kOutRank0;
            if (r.rankA == 0 && r.rankB == 0) d.flags |= kBothRank0;
            if (tiled[s]) d.flags |= kCtaTiled;
        }
        // interpreter schedule: work items of each level, lane groups for tiny outputs
        // (mixed form only; FP64 keeps one accumulator per output element)
        p->level_items[prec].assign(n_levels, 0);
        for (int L0 = 0; L0 < n_levels; L0++) {
            uint32_t acc = 0;
            for (int i = p->level_cta[L0]; i < p->level_start[L0 + 1]; i++) {
                steps[i].group = 1;
                steps[i].item_start = 0xffffffffu;   // never found by the item search
            }
            // Mixed form: outputs share their k loop among a lane group (a power of
            // two, at most a warp).  The level's group size is the largest that
            // keeps all of its outputs within one round of the CTA's threads, so a
            // level of many small steps is not spread over extra rounds; a step
            // with a long sum gets enough lanes for <= 64 terms per lane anyway.
            // The FP64 form keeps one accumulator per output (the reference's order).
            uint64_t base = 0;
            for (int i = p->level_start[L0]; i < p->level_cta[L0]; i++) base += 1ull << (2 * steps[i].nFree);
            uint64_t gl = 1;
            while (gl < 32 && base * gl * 2 <= (uint64_t) kPlanThreads) gl *= 2;
            for (int i = p->level_start[L0]; i < p->level_cta[L0]; i++) {
                StepDesc &d = steps[i];
                const uint64_t n_out = 1ull << (2 * d.nFree), K = 1ull << (2 * d.nSum);
                uint32_t g = 1;
                if (mixed) g = (uint32_t) std::min<uint64_t>({K, 32, std::max<uint64_t>(gl, K / 64)});
                acc = (acc + g - 1) / g * g;   // a lane group starts on a multiple of its size
                d.group = (uint8_t) g;
                d.item_start = acc;
                const uint64_t next = acc + n_out * g;
                acc = next > 0xffffffffull ? 0xffffffffu : (uint32_t) next;
            }
            p->level_items[prec][L0] = acc;
        }
        // item -> step map for small plans (replaces the per-item binary search)
        p->item_step[prec].clear();
        uint64_t total_items = 0;
        bool fits = true;
        for (int L0 = 0; L0 < n_levels; L0++) {
            total_items += p->level_items[prec][L0];
            fits = fits && p->level_cta[L0] - p->level_start[L0] <= 256;
        }
        if (fits && total_items <= kMaxItemMap) {
            for (int L0 = 0; L0 < n_levels; L0++) {
                int si = p->level_start[L0];
                for (uint32_t item = 0; item < p->level_items[prec][L0]; item++) {
                    while (si + 1 < p->level_cta[L0] && steps[si + 1].item_start <= item) si++;
                    p->item_step[prec].push_back((uint8_t) (si - p->level_start[L0]));
                }
            }
        }
    }
    // offset tables for the interpreter when every operand fits 16-bit offsets
    // (same maps for both precisions; offsets in elements)
    {
        bool small = true;
        uint64_t entries = 0;
        for (const auto &d : p->steps[QT_PREC_FP64]) {
            if (d.rA > 8 || d.rB > 8) small = false;
            entries += (1ull << (2 * d.nFree)) + (1ull << (2 * d.nSum));
        }
        p->tables.clear();
        if (small && entries * sizeof(uint16_t) * 2 <= kMaxTableBytes) {
            for (int i = 0; i < S; i++) {
                const StepDesc &d = p->steps[QT_PREC_FP64][i];
                const uint32_t off = (uint32_t) p->tables.size();
                for (int prec = 0; prec < 2; prec++) p->steps[prec][i].tab_off = off;
                const uint64_t n_out = 1ull << (2 * d.nFree), K = 1ull << (2 * d.nSum);
                for (uint64_t c = 0; c < n_out; c++) {
                    uint64_t oa, ob;
                    scatter_c(c, d, oa, ob);
                    p->tables.push_back({(uint16_t) oa, (uint16_t) ob});
                }
                for (uint64_t k = 0; k < K; k++)
                    p->tables.push_back({(uint16_t) scatter_digits(k, d.posAs, d.nSum),
                                         (uint16_t) scatter_digits(k, d.posBs, d.nSum)});
            }
        } else {
            for (int prec = 0; prec < 2; prec++)
                for (auto &d : p->steps[prec]) d.tab_off = kNoTable;
        }
    }
    // packed per-step fields for the work-item path (after the offset tables)
    for (int prec = 0; prec < 2; prec++) {
        const std::vector<StepDesc> &steps = p->steps[prec];
        p->level_meta[prec].assign(n_levels, 0);
        for (int L0 = 0; L0 < n_levels; L0++) {
            uint32_t lg = 0, comp = 0;
            for (int i = p->level_start[L0]; i < p->level_cta[L0]; i++) {
                const uint32_t g = steps[i].group ? steps[i].group : 1;
                const uint32_t l = (uint32_t) __builtin_ctz(g);
                lg = std::max(lg, l);
                if (l > 0 && (steps[i].flags & kCF64)) comp = 1;
            }
            p->level_meta[prec][L0] = lg | (comp << 8);
        }
        p->hot[prec].assign(S, HotStep());
        for (int i = 0; i < S; i++) {
            const StepDesc &d = steps[i];
            HotStep &hs = p->hot[prec][i];
            hs.a_off = (uint32_t) d.a_off;
            hs.b_off = (uint32_t) d.b_off;
            hs.c_off = (uint32_t) d.c_off;
            hs.tab_off = d.tab_off;
            hs.item_start = d.item_start;
            hs.a_step = (int16_t) d.a_step;
            hs.b_step = (int16_t) d.b_step;
            hs.group_log2 = (uint8_t) __builtin_ctz(d.group ? d.group : 1);
            hs.nFree = d.nFree;
            hs.nSum = d.nSum;
            hs.flags = (uint8_t) d.flags;
            hs.pad = 0;
        }
    }
    // per-item descriptors of the mixed form: every work-item step tabled
    {
        const int prec = QT_PREC_MIXED;
        const std::vector<StepDesc> &steps = p->steps[prec];
        p->items[prec].clear();
        uint64_t total = 0;
        bool ok = !p->tables.empty();
        for (int L0 = 0; L0 < n_levels && ok; L0++) {
            total += p->level_items[prec][L0];
            for (int i = p->level_start[L0]; i < p->level_cta[L0]; i++) ok = ok && steps[i].tab_off != kNoTable;
        }
        ok = ok && total <= kMaxItemDescs;
        for (int L0 = 0; L0 < n_levels && ok; L0++) {
            int si = p->level_start[L0];
            for (uint32_t item = 0; item < p->level_items[prec][L0]; item++) {
                while (si + 1 < p->level_cta[L0] && steps[si + 1].item_start <= item) si++;
                const StepDesc &d = steps[si];
                const uint32_t g = d.group ? d.group : 1, lg = (uint32_t) __builtin_ctz(g);
                const uint32_t local = item - d.item_start, c = local >> lg;
                const uint32_t n_out = 1u << (2 * d.nFree);
                ItemDesc it{0, 0, 0, 0};
                it.meta = (lg << 16) | ((uint32_t) d.nSum << 19);
                if (d.flags & kALeaf) it.meta |= kItemLeafA;
                if (d.flags & kBLeaf) it.meta |= kItemLeafB;
                const bool f64 = (d.flags & kCF64) != 0;
                if (f64) it.meta |= kItemF64;
                if (item >= d.item_start && c < n_out) {
                    const ushort2 o = p->tables[d.tab_off + c];
                    const uint64_t a = (uint64_t) d.a_off + 8ull * o.x, b = (uint64_t) d.b_off + 8ull * o.y;
                    const uint64_t cc = (uint64_t) d.c_off + (f64 ? 16ull : 8ull) * c;
                    const uint64_t kt = (uint64_t) d.tab_off + n_out;
                    // the complex64 copy of a compensated output: 16 n_out + 8 c bytes past its start
                    const uint32_t delta = f64 ? 2 * n_out - c : 0;
                    if (a > 0xffffffffull || b > 0xffffffffull || cc > 0xffffffffull || kt > 0xffffull || delta > 15) {
                        ok = false;
                        break;
                    }
                    it.a = (uint32_t) a;
                    it.b = (uint32_t) b;
                    it.c = (uint32_t) cc;
                    it.meta |= (uint32_t) kt | kItemValid | (delta << 27);
                }
                p->items[prec].push_back(it);
            }
        }
        if (!ok) p->items[prec].clear();
    }
    p->n_steps = S;
    p->n_levels = n_levels;
    p->grouped = p->max_step_out <= kGroupedMaxRank && p->max_step_k <= kGroupedMaxSum &&
                 p->ws_bytes[QT_PREC_FP64] <= kGroupedMaxWorkspace && S <= kPlanMaxSteps;
    for (int i = 0; i < L; i++) p->peak_rank = std::max(p->peak_rank, leaves[i]->mRank);
    return QT_OK;
}

qt_status upload_plan(qt_plan *p, int prec) {
    // uploaded once; later callers (batches on other contexts) do not take the
    // owner's lock, which a long step-by-step run on that context may hold
    if (p->dev_ready[prec].load(std::memory_order_acquire)) return QT_OK;
    qt_ctx *ctx = p->ctx;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    if (p->dev[prec]) return QT_OK;
    const size_t steps_bytes = sizeof(StepDesc) * p->steps[prec].size();
    const size_t lvl_bytes = sizeof(int32_t) * p->level_start.size();
    const size_t r0_bytes = sizeof(int32_t) * (p->rank0_steps.size() + 1);
    const size_t items_bytes = sizeof(uint32_t) * (p->level_items[prec].size() + 1);
    const size_t cta_bytes = sizeof(int32_t) * (p->level_cta.size() + 1);
    const size_t off_steps = align_up(sizeof(PlanDesc), 256);
    const size_t off_lvl = align_up(off_steps + steps_bytes, 256);
    const size_t off_r0 = align_up(off_lvl + lvl_bytes, 256);
    const size_t off_items = align_up(off_r0 + r0_bytes, 256);
    const size_t tab_bytes = sizeof(ushort2) * p->tables.size();
    const size_t off_cta = align_up(off_items + items_bytes, 16);
    const size_t rot_bytes = sizeof(uint2) * p->rot_table[prec].size();
    const size_t off_rot = align_up(off_cta + cta_bytes, 16);
    const size_t map_bytes = p->item_step[prec].size();
    const size_t off_map = align_up(off_rot + rot_bytes, 16);
    const size_t hot_bytes = sizeof(HotStep) * p->hot[prec].size();
    const size_t off_hot = align_up(off_map + map_bytes, 16);
    const size_t meta_bytes = sizeof(uint32_t) * p->level_meta[prec].size();
    const size_t off_meta = align_up(off_hot + hot_bytes, 16);
    const size_t desc_bytes = sizeof(ItemDesc) * p->items[prec].size();
    const size_t off_desc = align_up(off_meta + meta_bytes, 16);
    const size_t off_tab = align_up(off_desc + desc_bytes, 256);
    const size_t total = off_tab + tab_bytes + 16;
    void *d = nullptr;
    qt_status s = dev_alloc(ctx, total, &d);
    if (s != QT_OK) return s;
    std::vector<char> host(total, 0);
    PlanDesc pd;
    std::memset(&pd, 0, sizeof pd);
    pd.steps = reinterpret_cast<const StepDesc *>((char *) d + off_steps);
    pd.level_start = reinterpret_cast<const int32_t *>((char *) d + off_lvl);
    pd.rank0_steps = reinterpret_cast<const int32_t *>((char *) d + off_r0);
    pd.level_items = reinterpret_cast<const uint32_t *>((char *) d + off_items);
    pd.tables = reinterpret_cast<const ushort2 *>((char *) d + off_tab);
    pd.level_cta = reinterpret_cast<const int32_t *>((char *) d + off_cta);
    pd.rotations = reinterpret_cast<const uint2 *>((char *) d + off_rot);
    pd.item_step = map_bytes ? reinterpret_cast<const uint8_t *>((char *) d + off_map) : nullptr;
    pd.hot = reinterpret_cast<const HotStep *>((char *) d + off_hot);
    pd.level_meta = reinterpret_cast<const uint32_t *>((char *) d + off_meta);
    pd.items = desc_bytes ? reinterpret_cast<const ItemDesc *>((char *) d + off_desc) : nullptr;
    if (desc_bytes) std::memcpy(host.data() + off_desc, p->items[prec].data(), desc_bytes);
    if (meta_bytes) std::memcpy(host.data() + off_meta, p->level_meta[prec].data(), meta_bytes);
    if (hot_bytes) std::memcpy(host.data() + off_hot, p->hot[prec].data(), hot_bytes);
    if (map_bytes) std::memcpy(host.data() + off_map, p->item_step[prec].data(), map_bytes);
    if (rot_bytes) std::memcpy(host.data() + off_rot, p->rot_table[prec].data(), rot_bytes);
    if (!p->level_cta.empty())
        std::memcpy(host.data() + off_cta, p->level_cta.data(), cta_bytes - sizeof(int32_t));
    if (tab_bytes) std::memcpy(host.data() + off_tab, p->tables.data(), tab_bytes);
    pd.n_steps = p->n_steps;
    pd.n_levels = p->n_levels;
    pd.n_rank0 = (int32_t) p->rank0_steps.size();
    pd.n_rot = (int32_t) p->rot_table[prec].size();
    std::memcpy(host.data(), &pd, sizeof(pd));
    if (steps_bytes) std::memcpy(host.data() + off_steps, p->steps[prec].data(), steps_bytes);
    if (lvl_bytes) std::memcpy(host.data() + off_lvl, p->level_start.data(), lvl_bytes);
    if (!p->rank0_steps.empty()) std::memcpy(host.data() + off_r0, p->rank0_steps.data(), r0_bytes - sizeof(int32_t));
    if (!p->level_items[prec].empty())
        std::memcpy(host.data() + off_items, p->level_items[prec].data(), items_bytes - sizeof(uint32_t));
    cudaError_t e = cudaMemcpyAsync(d, host.data(), total, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        dev_free(ctx, d);
        return cuda_error(ctx, e, "plan upload");
    }
    p->dev[prec] = d;
    p->dev_bytes[prec] = total;
    p->dev_ready[prec].store(true, std::memory_order_release);
    return QT_OK;
}

// leaves of one instance in the execution precision, written at dst
void pack_leaves(const qt_plan *p, int prec, const std::complex<double> *src, char *dst) {
    const bool mixed = prec == QT_PREC_MIXED;
    uint64_t e = 0;
    for (size_t i = 0; i < p->leaf_rank.size(); i++) {
        const uint64_t n = 1ull << (2 * p->leaf_rank[i]);
        char *o = dst + p->leaf_off[prec][i];
        if (mixed) {
            float *f = reinterpret_cast<float *>(o);
            for (uint64_t j = 0; j < n; j++) {
                f[2 * j] = (float) src[e + j].real();
                f[2 * j + 1] = (float) src[e + j].imag();
            }
        } else {
            std::memcpy(o, src + e, n * sizeof(std::complex<double>));
        }
        e += n;
    }
}

// Step-by-step execution with the whole-GPU pairwise kernel (plans whose
// intermediates are too large for one CTA).  Mixed precision runs every step
// in complex64 with per-tensor power-of-two scaling (a scale word per step,
// scale.cuh) and reads the final value back as FP64, times 2^E of its step.
qt_status execute_stepwise(qt_plan *p, qt_ctx *ctx, int prec, const std::complex<double> *leaves, double *value) {
    if (p->peak_rank > kMaxStepwiseRank)
        return set_error(ctx, QT_ERR_INVALID_FUNCTION_INPUT,
                         "plan has a rank-" + std::to_string(p->peak_rank) +
                             " intermediate: above 4^15 elements, beyond the step kernels (slice it)");
    const bool mixed = prec == QT_PREC_MIXED;
    const size_t es = mixed ? 8 : 16;
    std::lock_guard<std::recursive_mutex> g(ctx->lock);
    // leaf buffer in the uniform precision of this mode
    uint64_t loff = 0;
    std::vector<uint64_t> leaf_off(p->leaf_rank.size());
    for (size_t i = 0; i < p->leaf_rank.size(); i++) {
        leaf_off[i] = loff;
        loff = align_up(loff + (es << (2 * p->leaf_rank[i])), 256);
    }
    std::vector<char> host(loff);
    uint64_t e = 0;
    for (size_t i = 0; i < p->leaf_rank.size(); i++) {
        const uint64_t n = 1ull << (2 * p->leaf_rank[i]);
        if (mixed) {
            float *f = reinterpret_cast<float *>(host.data() + leaf_off[i]);
            for (uint64_t j = 0; j < n; j++) {
                f[2 * j] = (float) leaves[e + j].real();
                f[2 * j + 1] = (float) leaves[e + j].imag();
            }
        } else {
            std::memcpy(host.data() + leaf_off[i], leaves + e, n * 16);
        }
        e += n;
    }
    void *dleaf = nullptr;
    qt_status s = dev_alloc(ctx, loff ? loff : 256, &dleaf);
    if (s != QT_OK) return s;
    cudaError_t ce = cudaMemcpyAsync(dleaf, host.data(), loff, cudaMemcpyHostToDevice, ctx->stream);
    if (ce != cudaSuccess) {
        dev_free(ctx, dleaf);
        return cuda_error(ctx, ce, "leaf upload");
    }
    // intermediates: one device buffer per step output, released when consumed
    const auto &steps = p->steps[QT_PREC_FP64];   // index maps are precision independent
    std::vector<void *> outs(steps.size(), nullptr);
    std::vector<int> uses(steps.size(), 0);
    for (const auto &d : steps) {
        if (d.a_step >= 0) uses[d.a_step]++;
        if (d.b_step >= 0) uses[d.b_step]++;
    }
    s = QT_OK;
    // level by level (the steps are stored in level order and a level's steps
    // are independent): the level's small steps go out as one batched launch,
    // the others one launch each; the inputs a level consumed last are released
    // once the level is on the stream
    auto pb = std::make_unique<PairBatch>();
    pb->n_jobs = 0;
    // one timeout flag for every tensor-core step, read once at the end
    void *gflag = nullptr;
    s = dev_alloc(ctx, 256, &gflag);
    if (s == QT_OK) s = cuda_error(ctx, cudaMemsetAsync(gflag, 0, sizeof(int), ctx->stream), "flag clear");
    // mixed form: the scale word of every step output, zeroed
    ScaleWord *words = nullptr;
    if (s == QT_OK && mixed) {
        const size_t wb = sizeof(ScaleWord) * std::max<size_t>(steps.size(), 1);
        s = dev_alloc(ctx, wb, reinterpret_cast<void **>(&words));
        if (s == QT_OK) s = cuda_error(ctx, cudaMemsetAsync(words, 0, wb, ctx->stream), "scale words clear");
    }
    auto flush = [&]() -> qt_status {
        const cudaError_t fe = launch_pair_batch(*pb, !mixed, ctx->stream);
        if (pb->n_jobs) ctx->launches++;
        pb->n_jobs = 0;
        return cuda_error(ctx, fe, "batched pair launch");
    };
    const int n_levels = (int) p->level_start.size() - 1;
    for (int L = 0; L < n_levels && s == QT_OK; L++) {
        if (deadline_passed(ctx)) {
            s = set_error(ctx, QT_ERR_DEADLINE, "deadline expired");
            break;
        }
        const int i0 = p->level_start[L], i1 = p->level_start[L + 1];
        for (int i = i0; i < i1 && s == QT_OK; i++) {
            const StepDesc &d = steps[i];
            const void *A = (d.flags & kALeaf) ? (const char *) dleaf + leaf_off[p->a_leaf[i]] : outs[d.a_step];
            const void *B = (d.flags & kBLeaf) ? (const char *) dleaf + leaf_off[p->b_leaf[i]] : outs[d.b_step];
            s = dev_alloc(ctx, es << (2 * d.nFree), &outs[i]);
            if (s != QT_OK) break;
            StepScaleRef sc;
            if (mixed) {
                sc.a = d.a_step >= 0 ? words + d.a_step : nullptr;
                sc.b = d.b_step >= 0 ? words + d.b_step : nullptr;
                sc.c = words + i;
            }
            if (pair_batchable(d, !mixed)) {
                PairJob &w = pb->job[pb->n_jobs++];
                w.d = d;
                w.A = A;
                w.B = B;
                w.C = outs[i];
                w.sc = sc;
                if (pb->n_jobs == (uint32_t) kPairBatchMax) s = flush();
            } else {
                s = run_contraction(ctx, d, A, B, outs[i], !mixed, (int *) gflag, sc);
            }
        }
        if (s == QT_OK) s = flush();
        if (s != QT_OK) break;
        for (int i = i0; i < i1; i++) {
            const StepDesc &d = steps[i];
            if (d.a_step >= 0 && --uses[d.a_step] == 0 && !(steps[d.a_step].flags & kOutRank0)) {
                dev_free(ctx, outs[d.a_step]);
                outs[d.a_step] = nullptr;
            }
            if (d.b_step >= 0 && --uses[d.b_step] == 0 && !(steps[d.b_step].flags & kOutRank0)) {
                dev_free(ctx, outs[d.b_step]);
                outs[d.b_step] = nullptr;
            }
        }
    }
    if (s == QT_OK) {
        int h = 0;
        ce = cudaMemcpyAsync(&h, gflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
        s = cuda_error(ctx, ce, "tensor-core contraction");
        if (s == QT_OK && h) s = set_error(ctx, QT_ERR_CUDA, "tensor-core pipeline wait timed out");
    }
    if (s == QT_OK) {
        // final-value rule over the rank-0 outputs in contraction order (Network.h:961-965)
        double fre = 0.0, fim = 0.0;
        for (int r : p->rank0_steps) {
            double v[2];
            if (mixed) {
                float f[2];
                ScaleWord w{};
                ce = cudaMemcpyAsync(f, outs[r], 8, cudaMemcpyDeviceToHost, ctx->stream);
                if (ce == cudaSuccess) ce = cudaMemcpyAsync(&w, words + r, sizeof w, cudaMemcpyDeviceToHost, ctx->stream);
                if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
                v[0] = std::ldexp((double) f[0], w.expo);
                v[1] = std::ldexp((double) f[1], w.expo);
            } else {
                ce = cudaMemcpyAsync(v, outs[r], 16, cudaMemcpyDeviceToHost, ctx->stream);
                if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
            }
            if (ce != cudaSuccess) {
                s = cuda_error(ctx, ce, "value download");
                break;
            }
            if ((std::fabs(fre) <= 1.0e-30 && std::fabs(fim) <= 1.0e-30) || (steps[r].flags & kBothRank0)) {
                fre = v[0];
                fim = v[1];
            }
        }
        value[0] = fre;
        value[1] = fim;
    }
    for (void *o : outs) dev_free(ctx, o);
    dev_free(ctx, dleaf);
    dev_free(ctx, gflag);
    dev_free(ctx, words);
    return s;
}

}  // namespace qtg
