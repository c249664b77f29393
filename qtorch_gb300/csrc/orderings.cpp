// Contraction orderings on top of Network::ContractNodes.
//
//   ContractionTools::ParallelContract   src/ContractionTools.h:219-388, 1261-1279
//   ContractionTools::ContractGivenSequence                  :392-411
//   ContractionTools::ContractUserDefinedSequenceOfWires     :155-214
//   LineGraph (wire numbering, line-graph edges)     src/LineGraph.h:92-171
//   LineGraph::LGContract walk                       src/LineGraph.h:357-376
//   Network::ReduceCircuit                           src/Network.h:1015-1118
//
// Differences from the reference, on purpose:
//  * the stochastic ordering draws from one std::mt19937 with a caller-given
//    seed and runs the two partition loops one after the other, so an ordering
//    is reproducible (the reference seeds from std::random_device and lets two
//    threads share one generator);
//  * the line-graph elimination order comes from a min-fill heuristic computed
//    here instead of the external QuickBB binary (which the reference calls
//    with --min-fill-ordering).
#include <algorithm>
#include <cmath>
#include <exception>
#include <fstream>
#include <functional>
#include <map>
#include <queue>
#include <random>
#include <set>
#include <sstream>
#include <thread>

#include "../../include/qtorch/qtorch.hpp"

namespace qtorch {

// ===========================================================================
// ContractionTools

ContractionTools::ContractionTools(const std::string &inputFile, const std::string &measureFile, int numThreads)
    : mString(inputFile), mMeasureFile(measureFile), mRandGen(std::random_device()()), mCopyCreated(false),
      mNumThreadsInNetwork(numThreads) {}

ContractionTools::ContractionTools(std::shared_ptr<Network> network)
    : mNetwork(network), mRandGen(std::random_device()()), mCopyCreated(true) {}

void ContractionTools::Reset() {
    mNetwork = nullptr;
    mCopyCreated = false;
}

void ContractionTools::Reset(const std::string &inputFile, const std::string &measureFile, int numThreads) {
    mNetwork = nullptr;
    mCopyCreated = false;
    mString = inputFile;
    mMeasureFile = measureFile;
    mNumThreadsInNetwork = numThreads;
}

std::shared_ptr<Network> ContractionTools::Acquire() {
    if (!mCopyCreated) {
        mNetwork = std::make_shared<Network>(mString, mMeasureFile);
        mNetwork->SetNumThreads(mNumThreadsInNetwork);
    }
    return mNetwork;
}

std::shared_ptr<Network> ContractionTools::Contract(ContractionType type, int, int) {
    if (type == Stochastic) return ParallelContract(mRandGen);
    throw InvalidContractionMethod();
}

std::shared_ptr<Network> ContractionTools::ParallelContract(std::mt19937 &gen) {
    std::shared_ptr<Network> net = Acquire();
    if (net->HasFailed()) return nullptr;
    // CreateChunksOfNodes: partitions of size n/2, the remainder last (ContractionTools.h:1261-1279)
    const std::vector<std::shared_ptr<Node>> &all = net->GetUncontractedNodes();
    std::vector<std::vector<std::shared_ptr<Node>>> parts;
    {
        const int size = (int) all.size();
        int skip = size / 2, counter = 0;
        size_t it = 0;
        while (it < all.size() && skip > 0) {
            parts.emplace_back(all.begin() + it, all.begin() + it + skip);
            it += skip;
            counter += skip;
            if (size - counter < skip) skip = size - counter;
        }
        if (it < all.size()) parts.emplace_back(all.begin() + it, all.end());
    }
    auto remove_pair = [](std::vector<std::shared_ptr<Node>> &v, int one, int two) {
        if (two == (int) v.size() - 1) {
            v[two] = v.back();
            v.pop_back();
            v[one] = v.back();
            v.pop_back();
        } else {
            v[one] = v.back();
            v.pop_back();
            v[two] = v.back();
            v.pop_back();
        }
    };
    // contractPieceFunction (ContractionTools.h:248-305), threshold 1
    for (auto &part : parts) {
        int failures = 0;
        while (part.size() != 1 && failures < (int) std::pow(part.size(), 2)) {
            std::uniform_int_distribution<> dist(0, (int) part.size() - 1);
            const int one = dist(gen), two = dist(gen);
            if (one == two) continue;
            auto r = net->ContractNodes(part[one], part[two], 1);
            if (r) {
                remove_pair(part, one, two);
                failures = 0;
                part.push_back(r);
            } else if (!net->IsDone()) {
                failures++;
            } else {
                break;
            }
        }
    }
    // contractNodesLeftFunction (ContractionTools.h:309-356), adaptive threshold from -1
    std::vector<std::shared_ptr<Node>> left;
    for (auto &part : parts) left.insert(left.end(), part.begin(), part.end());
    int threshold = -1, fails = 0;
    while (!net->IsDone()) {
        if (fails > std::pow(left.size(), 2)) {
            threshold++;
            fails = 0;
        }
        std::uniform_int_distribution<> dist(0, (int) left.size() - 1);
        const int one = dist(gen), two = dist(gen);
        if (one == two || left[one]->mContracted || left[two]->mContracted) continue;
        auto r = net->ContractNodes(left[one], left[two], threshold);
        if (r) {
            remove_pair(left, one, two);
            left.push_back(r);
            fails = 0;
            threshold = -1;
        } else {
            fails++;
        }
    }
    mFinalVal = net->GetFinalValue();
    return net;
}

std::shared_ptr<Network> ContractionTools::ContractGivenSequence(const std::vector<std::pair<int, int>> &sequence) {
    std::shared_ptr<Network> net = Acquire();
    if (net->HasFailed()) return nullptr;
    for (const auto &p : sequence) {
        const auto &all = net->GetAllNodes();
        if (p.first < 0 || p.second < 0 || p.first >= (int) all.size() || p.second >= (int) all.size())
            throw ContractionFailure();
        net->ContractNodes(all[p.first], all[p.second], 100);
    }
    if (!net->IsDone()) throw ContractionFailure();
    mFinalVal = net->GetFinalValue();
    return net;
}

std::shared_ptr<Network> ContractionTools::ContractUserDefinedSequenceOfWires(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw InvalidFile();
    std::stringstream ss;
    ss << in.rdbuf();
    return ContractUserDefinedSequenceText(ss.str());
}

std::shared_ptr<Network> ContractionTools::ContractUserDefinedSequenceText(const std::string &text) {
    std::shared_ptr<Network> net = Acquire();
    if (net->HasFailed()) return nullptr;
    // one "a b" pair per line, every line read (ContractionTools.h:168-186)
    std::vector<std::pair<int, int>> order;
    std::istringstream in(text);
    std::string line;
    const int n = (int) net->GetAllNodes().size();
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        int a, b;
        if (!(ls >> a >> b)) continue;
        if (a < 0 || a > n || b < 0 || b > n) throw InvalidFileFormat();
        order.push_back({a, b});
    }
    std::vector<int> map(net->GetAllNodes().size());
    for (size_t i = 0; i < map.size(); i++) map[i] = (int) i;
    for (const auto &p : order) {
        if (p.first >= (int) map.size() || p.second >= (int) map.size()) throw InvalidUserContractionSequence();
        const auto &all = net->GetAllNodes();
        auto a = all[map[p.first]], b = all[map[p.second]];
        if (a->mContracted || b->mContracted) continue;
        net->ContractNodes(a, b, 10000);
        map[p.first] = (int) net->GetAllNodes().size() - 1;
        map[p.second] = (int) net->GetAllNodes().size() - 1;
    }
    if (!net->IsDone()) throw InvalidUserContractionSequence();
    mFinalVal = net->GetFinalValue();
    return net;
}

// ===========================================================================
// LineGraph

LineGraph::LineGraph(std::shared_ptr<Network> network) : mNetwork(network) { Build(); }

void LineGraph::Reset(std::shared_ptr<Network> network) {
    if (!network) {
        mNetwork->Reset();
    } else {
        mNetwork = network;
    }
    Build();
}

void LineGraph::Build() {
    mGraphWires.clear();
    mEdges.clear();
    mOrder.clear();
    // wire ids in first-seen order over the uncontracted nodes; every pair of
    // wires of one node is a line-graph edge (LineGraph.h:92-130)
    for (const auto &n : mNetwork->GetUncontractedNodes()) {
        auto &ws = n->GetWires();
        for (size_t w = 0; w < ws.size(); w++) {
            auto &wire = ws[w];
            if (std::find(mGraphWires.begin(), mGraphWires.end(), wire) == mGraphWires.end()) {
                wire->SetWireID((int) mGraphWires.size());
                mGraphWires.push_back(wire);
            }
            for (size_t w2 = 0; w2 < w; w2++) mEdges.push_back({ws[w2]->GetWireID(), wire->GetWireID()});
        }
    }
}

namespace {

// Greedy min-fill elimination of the line graph (adjacency adj0, n wires).
// ends[v] = the two nodes wire v joins.  The walk LGContract makes from the
// order merges the two nodes on each eliminated wire, so the order fixes the
// contraction tree.  Ties of the fill score go to the smaller degree (classic
// min-fill), or, with shallow_ties, first to the wire whose merge reaches the
// lowest height in the tree (node heights tracked with a union-find).
// salt != 0 breaks the remaining ties (equal fill, height and degree) with a
// seeded hash instead of the smallest id, for restarts.
std::vector<int> min_fill_order(const std::vector<std::set<int>> &adj0, const std::vector<std::array<int, 2>> &ends,
                                int n_nodes, bool shallow_ties, uint64_t salt = 0, long long slack = 0) {
    const int n = (int) adj0.size();
    std::vector<std::set<int>> adj = adj0;
    std::vector<char> gone(n, 0);
    auto fill_of = [&](int v) {
        long long fill = 0;
        for (auto i = adj[v].begin(); i != adj[v].end(); ++i) {
            auto j = i;
            for (++j; j != adj[v].end(); ++j)
                if (!adj[*i].count(*j)) fill++;
        }
        return fill;
    };
    // fill counts are cached; eliminating x changes them only within distance 2 of x
    std::vector<long long> fill(n);
    for (int v = 0; v < n; v++) fill[v] = fill_of(v);
    std::vector<int> mark(n, -1);
    std::vector<int> parent(n_nodes), height(n_nodes, 0);
    for (int i = 0; i < n_nodes; i++) parent[i] = i;
    std::function<int(int)> find = [&](int x) { return parent[x] == x ? x : parent[x] = find(parent[x]); };
    auto merged_height = [&](int v) {
        const int a = find(ends[v][0]), b = find(ends[v][1]);
        return a == b ? 0 : std::max(height[a], height[b]) + 1;
    };
    std::vector<int> order;
    order.reserve(n);
    for (int step = 0; step < n; step++) {
        // with slack, any wire within `slack` of the smallest fill competes on height
        long long min_fill = -1;
        if (slack > 0)
            for (int v = 0; v < n; v++)
                if (!gone[v] && (min_fill < 0 || fill[v] < min_fill)) min_fill = fill[v];
        int best = -1, best_h = 0;
        uint64_t best_key = 0;
        auto key_of = [&](int v) {
            uint64_t x = (uint64_t) v * 0x9e3779b97f4a7c15ull ^ salt;   // splitmix64 finaliser
            x ^= x >> 30;
            x *= 0xbf58476d1ce4e5b9ull;
            x ^= x >> 27;
            x *= 0x94d049bb133111ebull;
            return x ^ (x >> 31);
        };
        for (int v = 0; v < n; v++) {
            if (gone[v]) continue;
            if (slack > 0) {
                if (fill[v] > min_fill + slack) continue;
                const int h = merged_height(v);
                if (best < 0 || h < best_h || (h == best_h && fill[v] < fill[best]) ||
                    (h == best_h && fill[v] == fill[best] && adj[v].size() < adj[best].size())) {
                    best = v;
                    best_h = h;
                }
                continue;
            }
            if (best >= 0 && fill[v] > fill[best]) continue;
            const int h = shallow_ties ? merged_height(v) : 0;
            const uint64_t key = salt ? key_of(v) : 0;
            if (best < 0 || fill[v] < fill[best] || h < best_h ||
                (h == best_h && adj[v].size() < adj[best].size()) ||
                (salt && h == best_h && adj[v].size() == adj[best].size() && key < best_key)) {
                best = v;
                best_h = h;
                best_key = key;
            }
        }
        gone[best] = 1;
        order.push_back(best);
        {
            const int a = find(ends[best][0]), b = find(ends[best][1]);
            if (a != b) {
                parent[a] = b;
                height[b] = std::max(height[a], height[b]) + 1;
            }
        }
        std::vector<int> nb(adj[best].begin(), adj[best].end());
        for (size_t i = 0; i < nb.size(); i++)
            for (size_t j = i + 1; j < nb.size(); j++) {
                adj[nb[i]].insert(nb[j]);
                adj[nb[j]].insert(nb[i]);
            }
        for (int u : nb) adj[u].erase(best);
        adj[best].clear();
        std::vector<int> affected;
        for (int u : nb) {
            if (mark[u] != step) {
                mark[u] = step;
                affected.push_back(u);
            }
            for (int w : adj[u])
                if (mark[w] != step) {
                    mark[w] = step;
                    affected.push_back(w);
                }
        }
        for (int u : affected) fill[u] = fill_of(u);
    }
    return order;
}

struct WalkCost {
    double macs = 0;   // complex MACs of the walk
    int peak = 0;      // largest rank it creates
    int height = 0;    // height of its contraction tree
};

// The walk LGContract makes from an order, without data: every merge sums over
// all wires the two nodes share (ContractNodes), 4^(rank C + shared) MACs.
WalkCost walk_cost(const std::vector<int> &order, const std::vector<std::array<int, 2>> &ends, int n_nodes) {
    std::vector<int> parent(n_nodes), height(n_nodes, 0);
    std::vector<std::set<int>> wires(n_nodes);
    for (int i = 0; i < n_nodes; i++) parent[i] = i;
    for (size_t v = 0; v < ends.size(); v++) {
        wires[ends[v][0]].insert((int) v);
        wires[ends[v][1]].insert((int) v);
    }
    std::function<int(int)> find = [&](int x) { return parent[x] == x ? x : parent[x] = find(parent[x]); };
    WalkCost c;
    for (int v : order) {
        const int a = find(ends[v][0]), b = find(ends[v][1]);
        if (a == b) continue;
        std::set<int> merged;
        int shared = 0;
        for (int w : wires[a]) {
            if (wires[b].count(w)) shared++;
            else merged.insert(w);
        }
        for (int w : wires[b])
            if (!wires[a].count(w)) merged.insert(w);
        c.macs += std::pow(4.0, (double) (merged.size() + shared));
        c.peak = std::max(c.peak, (int) merged.size());
        parent[a] = b;
        height[b] = std::max(height[a], height[b]) + 1;
        c.height = std::max(c.height, height[b]);
        wires[b].swap(merged);
        wires[a].clear();
    }
    return c;
}

// An order that builds the contraction tree in rounds: every round merges a
// maximal set of disjoint pairs of the current nodes joined by a wire,
// smallest merged rank first (then fewest MACs), and never a pair whose merge
// would exceed `cap` wires unless no pair fits.  Each round adds at most one
// level to the tree, so the height is about log2 of the node count when the
// graph allows.
std::vector<int> matching_order(const std::vector<std::array<int, 2>> &ends, int n_nodes, int cap) {
    std::vector<int> parent(n_nodes);
    std::vector<std::set<int>> wires(n_nodes);
    for (int i = 0; i < n_nodes; i++) parent[i] = i;
    for (size_t v = 0; v < ends.size(); v++) {
        wires[ends[v][0]].insert((int) v);
        wires[ends[v][1]].insert((int) v);
    }
    std::function<int(int)> find = [&](int x) { return parent[x] == x ? x : parent[x] = find(parent[x]); };
    std::vector<int> order;
    std::vector<char> placed(ends.size(), 0);
    for (;;) {
        struct Cand {
            int merged, shared, v, a, b;
        };
        std::vector<Cand> cands;
        std::set<std::pair<int, int>> seen;
        for (size_t v = 0; v < ends.size(); v++) {
            const int a = find(ends[v][0]), b = find(ends[v][1]);
            if (a == b || !seen.insert({std::min(a, b), std::max(a, b)}).second) continue;
            int shared = 0;
            for (int w : wires[a]) shared += (int) wires[b].count(w);
            const int merged = (int) (wires[a].size() + wires[b].size()) - 2 * shared;
            cands.push_back({merged, shared, (int) v, a, b});
        }
        if (cands.empty()) break;
        std::sort(cands.begin(), cands.end(), [](const Cand &x, const Cand &y) {
            if (x.merged != y.merged) return x.merged < y.merged;
            if (x.merged + x.shared != y.merged + y.shared) return x.merged + x.shared < y.merged + y.shared;
            return x.v < y.v;
        });
        std::vector<char> used(n_nodes, 0);
        std::vector<Cand> round;
        for (const auto &c : cands) {
            if (used[c.a] || used[c.b] || c.merged > cap) continue;
            used[c.a] = used[c.b] = 1;
            round.push_back(c);
        }
        if (round.empty()) round.push_back(cands.front());
        for (const auto &c : round) {
            order.push_back(c.v);
            placed[c.v] = 1;
            std::set<int> merged;
            for (int w : wires[c.a])
                if (!wires[c.b].count(w)) merged.insert(w);
            for (int w : wires[c.b])
                if (!wires[c.a].count(w)) merged.insert(w);
            parent[c.a] = c.b;
            wires[c.b].swap(merged);
            wires[c.a].clear();
        }
    }
    for (size_t v = 0; v < ends.size(); v++)   // wires already summed inside a node
        if (!placed[v]) order.push_back((int) v);
    return order;
}

}  // namespace

const std::vector<int> &LineGraph::MinFillOrdering() {
    if (!mOrder.empty() || mGraphWires.empty()) return mOrder;
    const int n = (int) mGraphWires.size();
    std::vector<std::set<int>> adj(n);
    for (auto &e : mEdges) {
        if (e[0] == e[1]) continue;
        adj[e[0]].insert(e[1]);
        adj[e[1]].insert(e[0]);
    }
    std::map<const Node *, int> node_index;
    std::vector<std::array<int, 2>> ends(n);
    for (int v = 0; v < n; v++) {
        for (int s = 0; s < 2; s++) {
            auto nd = s == 0 ? mGraphWires[v]->GetNodeA().lock() : mGraphWires[v]->GetNodeB().lock();
            auto it = node_index.find(nd.get());
            if (it == node_index.end()) it = node_index.emplace(nd.get(), (int) node_index.size()).first;
            ends[v][s] = it->second;
        }
    }
    const int n_nodes = (int) node_index.size();
    // On the GPU a small network's latency is the height of its contraction
    // tree, a large one's is its MACs: the shallow-tie order is taken when it
    // costs no larger intermediate and at most 1.5x the MACs of classic min-fill.
    // Candidates: classic min-fill, the shallow-tie order, and for small line
    // graphs seeded restarts of it (remaining ties at random) and orders that let
    // wires within 1-3 of the smallest fill compete on height.  The walk with
    // the lowest estimated GPU time wins among those that create no larger
    // intermediate than classic min-fill: ~1.5 us per dependent level of the
    // interpreter plus the MACs at one CTA's ~2e9 complex MAC/s -- height decides
    // for tiny networks, MACs for large ones.  (Weighting MACs 5-25x lower, so
    // that shallower trees with more MACs win, was measured slower everywhere:
    // batched QAOA 1.90 -> 2.88 ms, config-3 terms 189 -> 195 us.)
    auto est = [](const WalkCost &c) { return 1.5e-6 * c.height + c.macs / 2e9; };
    std::vector<int> classic = min_fill_order(adj, ends, n_nodes, false);
    const WalkCost cc = walk_cost(classic, ends, n_nodes);
    std::vector<int> pick = classic;
    WalkCost pc = cc;
    const int restarts = n <= 400 ? 8 : 0;
    for (int r = 0; r <= restarts + (n <= 400 ? 3 : 0); r++) {
        // r <= restarts: seeded ties; beyond: fill slack 1..3 traded for height
        const long long slack = r > restarts ? r - restarts : 0;
        std::vector<int> o = min_fill_order(adj, ends, n_nodes, true,
                                            (r == 0 || slack) ? 0 : 0x5eed0000ull + (uint64_t) r, slack);
        const WalkCost c = walk_cost(o, ends, n_nodes);
        if (c.peak > cc.peak) continue;
        if (est(c) < est(pc)) {
            pick = std::move(o);
            pc = c;
        }
    }
    // trees built in rounds of disjoint merges (lowest height), for small
    // graphs; where intermediates are tiny anyway (rank <= 6, 32 KB in
    // complex64) they may grow by up to two wires over classic min-fill
    if (n <= 400) {
        const int allowed = std::max(cc.peak, std::min(cc.peak + 2, 6));
        for (int cap = cc.peak; cap <= allowed; cap++) {
            std::vector<int> o = matching_order(ends, n_nodes, cap);
            const WalkCost c = walk_cost(o, ends, n_nodes);
            if (c.peak <= allowed && est(c) < est(pc)) {
                pick = std::move(o);
                pc = c;
            }
        }
    }
    for (int v : pick) mOrder.push_back(v + 1);
    return mOrder;
}

bool LineGraph::LGContract() { return LGContract(MinFillOrdering()); }

bool LineGraph::LGContract(const std::vector<int> &order) {
    // contract both endpoints of each not yet contracted wire, threshold 100 (LineGraph.h:357-376)
    for (int id1 : order) {
        if (id1 < 1 || id1 > (int) mGraphWires.size()) throw QbbFailure();
        auto &w = mGraphWires[id1 - 1];
        if (w->IsContracted()) continue;
        auto a = w->GetNodeA().lock(), b = w->GetNodeB().lock();
        if (!a || !b) continue;
        mNetwork->ContractNodes(a, b, 100);
    }
    // A circuit whose qubits form several unconnected groups leaves one rank-0
    // node per group; the reference stops with ContractionFailure there
    // (LineGraph.h:384-388).  They are multiplied together here instead, in
    // list order, as the stochastic ordering's leftover phase does.
    while (mNetwork->GetUncontractedNodes().size() > 1) {
        const auto &r = mNetwork->GetUncontractedNodes();
        bool all_scalar = true;
        for (const auto &x : r) all_scalar = all_scalar && x->mRank == 0;
        if (!all_scalar) break;
        mNetwork->ContractNodes(r[0], r[1], 100);
    }
    const auto &rem = mNetwork->GetUncontractedNodes();
    if (rem.size() != 1) throw ContractionFailure();
    if (rem[0]->mRank != 0) throw ContractionFailure();
    return true;
}

// ===========================================================================
// ReduceCircuit (src/Network.h:1015-1118): fold rank-2 gates into their
// predecessor on the wire, then merge consecutive two-qubit gates on the same
// pair of wires.

void Network::ReduceCircuit() {
    std::vector<std::vector<std::shared_ptr<Node>>> holder(mNumberOfQubits);
    for (int i = 0; i < mNumberOfQubits; i++) {
        for (auto &node : mNodesByWire[i]) {
            if (node->mRank == 2) {
                std::shared_ptr<Node> prev = holder[i].back();
                std::shared_ptr<Node> t = ContractNodes(prev, node, 0);
                if (!t) throw ContractionFailure();
                auto in0 = node->GetWires()[0]->GetNodeA().lock();
                t->AddWireNumber(in0->GetWireNumber()[0]);
                if (in0->mRank > 2) t->AddWireNumber(in0->GetWireNumber()[1]);
                if (prev->GetTypeOfNode() == GateType::INITSTATE) {
                    t->SetTypeOfNode(GateType::INITSTATE);
                    t->SetTypeOfNodeString("INITSTATE(Manipulated)");
                }
                FindAndReplace(mNodesByWire, prev, t);
                FindAndReplace(holder, prev, t);
            } else {
                holder[i].push_back(node);
            }
        }
    }
    mNodesByWire = std::move(holder);

    std::vector<std::vector<std::shared_ptr<Node>>> next(mNumberOfQubits);
    std::vector<std::shared_ptr<Node>> current(mNumberOfQubits);
    std::vector<int> idx(mNumberOfQubits, 0);
    std::vector<bool> updated(mNumberOfQubits, false);
    bool finished = false, found = false;
    while (!finished) {
        for (int j = 0; j < mNumberOfQubits; j++) {
            if (idx[j] >= (int) mNodesByWire[j].size() || updated[j]) continue;
            std::shared_ptr<Node> t = mNodesByWire[j][idx[j]];
            if (t->mRank == 1) {
                current[j] = t;
                updated[j] = true;
                idx[j]++;
                continue;
            }
            const int w0 = t->GetWireNumber()[0], w1 = t->GetWireNumber()[1];
            if (!updated[w1] && !updated[w0]) {
                if (idx[w0] < (int) mNodesByWire[w0].size() && idx[w1] < (int) mNodesByWire[w1].size() &&
                    mNodesByWire[w0][idx[w0]] == mNodesByWire[w1][idx[w1]]) {
                    if (current[w0] == current[w1] && current[w0]) {
                        current[w0] = ContractNodes(t, current[w0], 0);
                        if (!current[w0]) throw ContractionFailure();
                        current[w1] = current[w0];
                        current[w0]->AddWireNumber(w0);
                        current[w0]->AddWireNumber(w1);
                        found = true;
                    } else {
                        current[w0] = t;
                        current[w1] = t;
                    }
                    idx[w0]++;
                    idx[w1]++;
                    updated[w0] = true;
                    updated[w1] = true;
                }
            }
        }
        for (int j = 0; j < mNumberOfQubits; j++) {
            if (updated[j]) {
                if (found && !next[j].empty()) next[j].back() = current[j];
                else next[j].push_back(current[j]);
            } else if (idx[j] < (int) mNodesByWire[j].size() && !found) {
                next[j].push_back(nullptr);
            }
        }
        if (std::all_of(updated.begin(), updated.end(), [](bool b) { return !b; })) finished = true;
        std::fill(updated.begin(), updated.end(), false);
        found = false;
    }
    mNodesByWire = std::move(next);
}

// ---- preProcess (src/preprocess.h:28-52) ----------------------------------

bool preProcess(const std::string &qasmText, const std::string &measureText, const std::string &gateDir,
                uint64_t seed, int tries, long long maxMacs, PreProcessResult &best) {
    best = PreProcessResult{};
    bool found = false;
    for (int i = 0; i < tries; i++) {
        auto net = Network::FromText(qasmText, measureText, gateDir, nullptr);   // symbolic
        ContractionTools t(net);
        t.Seed(seed + (uint64_t) i);
        t.Contract(Stochastic);
        if (!net->IsDone()) continue;
        int peak = 0;
        for (const auto &n : net->GetAllNodes()) peak = std::max(peak, n->mRank);
        const long long macs = net->getNumFloatOps();
        best.tries = i + 1;
        if (!found || peak < best.peakRank || (peak == best.peakRank && macs < best.flops)) {
            found = true;
            best.seed = seed + (uint64_t) i;
            best.peakRank = peak;
            best.flops = macs;
            best.sequence.clear();
            // the walk of preprocess.h:41-46
            for (const auto &n : net->GetAllNodes())
                if (!(n->mCreatedFrom.first == 0 && n->mCreatedFrom.second == 0))
                    best.sequence.push_back(n->mCreatedFrom);
        }
        if (maxMacs > 0 && macs <= maxMacs) break;
    }
    return found;
}

// ---- size-greedy ordering --------------------------------------------------

namespace {

struct GreedyWalk {
    std::vector<std::pair<int, int>> merges;   // node indices: 0..n-1 the leaves, n+k the k-th merge
    int peak = 0;
    double macs = 0;
    int height = 0;
};

// One greedy walk over the abstract network: wires of each node (sorted),
// ends of each wire.  temperature 0: the plain size-change order; > 0: each
// score gets seeded Gumbel noise scaled by the larger operand's size.
GreedyWalk greedy_walk(std::vector<std::vector<int>> nw, std::vector<std::array<int, 2>> we, double temperature,
                       uint64_t seed) {
    const int n0 = (int) nw.size();
    std::vector<int> height(n0, 0);
    std::vector<char> alive(n0, 1);
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> uni(1e-12, 1.0);
    auto p4 = [](int r) { return std::ldexp(1.0, 2 * r); };
    struct Cand {
        double key;
        int a, b;
        bool operator<(const Cand &o) const {   // min-heap on key, then indices
            if (key != o.key) return key > o.key;
            if (a != o.a) return a > o.a;
            return b > o.b;
        }
    };
    std::priority_queue<Cand> heap;
    std::vector<int> scratch;
    // rank of the merge of a and b: wires in exactly one of them
    auto merged_rank = [&](int a, int b, int &shared) {
        const auto &x = nw[a], &y = nw[b];
        size_t i = 0, j = 0;
        int common = 0;
        while (i < x.size() && j < y.size()) {
            if (x[i] == y[j]) {
                common++;
                i++;
                j++;
            } else if (x[i] < y[j]) {
                i++;
            } else {
                j++;
            }
        }
        shared = common;
        return (int) (x.size() + y.size()) - 2 * common;
    };
    auto push = [&](int a, int b) {
        if (a == b || !alive[a] || !alive[b]) return;
        int shared = 0;
        const int rc = merged_rank(a, b, shared);
        const int ra = (int) nw[a].size(), rb = (int) nw[b].size();
        double key = p4(rc) - p4(ra) - p4(rb);
        if (temperature > 0) key -= temperature * p4(std::max(ra, rb)) * -std::log(-std::log(uni(gen)));
        heap.push({key, std::min(a, b), std::max(a, b)});
    };
    for (size_t w = 0; w < we.size(); w++) push(we[w][0], we[w][1]);
    GreedyWalk out;
    while (!heap.empty()) {
        const Cand c = heap.top();
        heap.pop();
        if (!alive[c.a] || !alive[c.b]) continue;
        const int k = (int) nw.size();
        scratch.clear();
        int shared = 0;
        {
            const auto &x = nw[c.a], &y = nw[c.b];
            size_t i = 0, j = 0;
            while (i < x.size() || j < y.size()) {
                if (j == y.size() || (i < x.size() && x[i] < y[j])) {
                    scratch.push_back(x[i++]);
                } else if (i == x.size() || y[j] < x[i]) {
                    scratch.push_back(y[j++]);
                } else {
                    shared++;
                    i++;
                    j++;
                }
            }
        }
        nw.push_back(scratch);
        alive.push_back(1);
        alive[c.a] = alive[c.b] = 0;
        height.push_back(std::max(height[c.a], height[c.b]) + 1);
        for (int w : nw[k])
            for (int s = 0; s < 2; s++)
                if (we[w][s] == c.a || we[w][s] == c.b) we[w][s] = k;
        out.merges.push_back({c.a, c.b});
        out.peak = std::max(out.peak, (int) nw[k].size());
        out.macs += p4((int) nw[k].size() + shared);
        out.height = std::max(out.height, height[k]);
        nw[c.a].clear();
        nw[c.b].clear();
        nw[c.a].shrink_to_fit();
        nw[c.b].shrink_to_fit();
        for (int w : nw[k]) {
            const int other = we[w][0] == k ? we[w][1] : we[w][0];
            push(k, other);
        }
    }
    return out;
}

// The uncontracted nodes as an abstract graph: wires of each node (sorted
// ids), the two nodes of each wire.  Wire ids are given in first-seen order
// over the nodes and their wires, as LineGraph::Build numbers them.
void abstract_network(const Network &net, std::vector<std::vector<int>> &nw, std::vector<std::array<int, 2>> &we) {
    const auto &nodes = net.GetUncontractedNodes();
    std::map<const Node *, int> index;
    for (size_t i = 0; i < nodes.size(); i++) index[nodes[i].get()] = (int) i;
    std::map<const Wire *, int> wire_id;
    nw.assign(nodes.size(), {});
    we.clear();
    for (size_t i = 0; i < nodes.size(); i++) {
        for (auto &w : nodes[i]->GetWires()) {
            auto it = wire_id.find(w.get());
            if (it == wire_id.end()) {
                auto a = w->GetNodeA().lock(), b = w->GetNodeB().lock();
                if (!a || !b || !index.count(a.get()) || !index.count(b.get())) throw ContractionFailure();
                it = wire_id.emplace(w.get(), (int) we.size()).first;
                we.push_back({index[a.get()], index[b.get()]});
            }
            nw[i].push_back(it->second);
        }
        std::sort(nw[i].begin(), nw[i].end());
        nw[i].erase(std::unique(nw[i].begin(), nw[i].end()), nw[i].end());
    }
}

// A walk may go one rank above the smallest largest intermediate found when
// that cuts its MACs by a third or more, up to this rank (the largest intermediate the
// step-by-step kernels take: 4^15 elements).
constexpr int kGreedyRankStretchMax = 15;

// The walks of `tries` seeded tries, spread over up to 16 host threads.  The
// kept one: the fewest MACs (then the lowest try number) among the walks with
// the smallest largest intermediate P -- or, when a walk with a largest
// intermediate of P + 1 <= 15 needs at most two thirds of those MACs, the
// fewest MACs among those.  A 4^(P+1) intermediate costs 4x the memory of a
// 4^P one; on the serving mix's large circuits it can halve the work (18
// qubits at depth 16: 5.0e12 -> 2.6e12 complex MACs).  The choice does not depend on how
// many threads ran the tries; the winner's merges come from running its try
// once more.  A walk of a 400-500 node network takes about half a millisecond.
GreedyWalk best_greedy_walk(const std::vector<std::vector<int>> &nw, const std::vector<std::array<int, 2>> &we,
                            uint64_t seed, int tries) {
    auto run = [&](int t) {
        // temperatures cycle over a few scales so that both small and large
        // perturbations of the plain order are tried
        static const double kTemps[4] = {0.02, 0.1, 0.3, 1.0};
        const double temp = t == 0 ? 0.0 : kTemps[(t - 1) % 4];
        return greedy_walk(nw, we, temp, seed * 0x9e3779b97f4a7c15ull + (uint64_t) t);
    };
    std::vector<int> peak(tries);
    std::vector<double> macs(tries);
    const unsigned hw = std::thread::hardware_concurrency();
    const int n_threads = std::max(1, std::min({tries / 64, 16, (int) (hw ? hw : 1)}));
    // an exception of a worker thread (a failed allocation) reaches the caller
    // after every thread has joined, as it would from a single thread
    std::vector<std::exception_ptr> failed(n_threads);
    auto worker = [&](int w) {
        try {
            for (int t = w; t < tries; t += n_threads) {
                const GreedyWalk g = run(t);
                peak[t] = g.peak;
                macs[t] = g.macs;
            }
        } catch (...) {
            failed[w] = std::current_exception();
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < n_threads; w++) pool.emplace_back(worker, w);
    worker(0);
    for (auto &th : pool) th.join();
    for (auto &f : failed)
        if (f) std::rethrow_exception(f);
    const int p_min = *std::min_element(peak.begin(), peak.end());
    auto fewest = [&](int max_peak, int exact) {
        int k = -1;
        for (int t = 0; t < tries; t++) {
            if (exact ? peak[t] != max_peak : peak[t] > max_peak) continue;
            if (k < 0 || macs[t] < macs[k]) k = t;
        }
        return k;
    };
    int k = fewest(p_min, 1);
    if (p_min + 1 <= kGreedyRankStretchMax) {
        const int k1 = fewest(p_min + 1, 0);
        if (k1 >= 0 && 3 * macs[k1] <= 2 * macs[k]) k = k1;
    }
    return run(k);
}

// Replays merges (indices as in GreedyWalk) on the network, then multiplies
// leftover rank-0 nodes of unconnected groups in list order.
void replay_merges(Network &net, const std::vector<std::pair<int, int>> &merges) {
    std::vector<std::shared_ptr<Node>> nodes = net.GetUncontractedNodes();
    for (const auto &m : merges) {
        auto c = net.ContractNodes(nodes[m.first], nodes[m.second], 100);
        if (!c) {
            if (net.IsDone()) return;   // the merge that finished the network
            throw ContractionFailure();
        }
        nodes.push_back(c);
    }
    while (net.GetUncontractedNodes().size() > 1) {
        const auto &rem = net.GetUncontractedNodes();
        bool all_scalar = true;
        for (const auto &x : rem) all_scalar = all_scalar && x->mRank == 0;
        if (!all_scalar) throw ContractionFailure();
        net.ContractNodes(rem[0], rem[1], 100);
    }
}

// The LGContract walk of a 1-based wire order over the abstract graph.
GreedyWalk order_walk(const std::vector<int> &order1, const std::vector<std::vector<int>> &nw,
                      const std::vector<std::array<int, 2>> &we) {
    std::vector<std::array<int, 2>> ends(we.size());
    for (size_t v = 0; v < we.size(); v++) ends[v] = we[v];
    std::vector<int> order0;
    for (int v : order1) order0.push_back(v - 1);
    const WalkCost c = walk_cost(order0, ends, (int) nw.size());
    GreedyWalk g;
    g.peak = c.peak;
    g.macs = c.macs;
    g.height = c.height;
    return g;
}

}  // namespace

GreedyResult GreedyContract(Network &net, uint64_t seed, int tries) {
    if (tries < 1) throw InvalidFunctionInput();
    std::vector<std::vector<int>> nw;
    std::vector<std::array<int, 2>> we;
    abstract_network(net, nw, we);
    GreedyWalk best = best_greedy_walk(nw, we, seed, tries);
    GreedyResult r;
    r.tries = tries;
    r.peakRank = best.peak;
    r.macs = best.macs;
    r.height = best.height;
    replay_merges(net, best.merges);
    return r;
}

GreedyResult AutoContract(std::shared_ptr<Network> net, uint64_t seed, int tries, int maxMinFillWires) {
    std::vector<std::vector<int>> nw;
    std::vector<std::array<int, 2>> we;
    abstract_network(*net, nw, we);
    GreedyWalk g = best_greedy_walk(nw, we, seed, tries);
    GreedyResult r;
    r.tries = tries;
    if ((int) we.size() <= maxMinFillWires) {
        LineGraph lg(net);
        const std::vector<int> order = lg.MinFillOrdering();
        const GreedyWalk m = order_walk(order, nw, we);
        // the GPU time estimate of the min-fill walk (1.5 us per dependent
        // level, MACs at ~2e9 a second per CTA) decides unless the greedy walk
        // keeps a smaller largest intermediate
        auto est = [](const GreedyWalk &w) { return 1.5e-6 * w.height + w.macs / 2e9; };
        const bool take_minfill = m.peak < g.peak || (m.peak == g.peak && est(m) <= est(g)) ||
                                  (m.peak == g.peak + 1 && est(m) * 2 <= est(g));
        if (take_minfill) {
            r.peakRank = m.peak;
            r.macs = m.macs;
            r.height = m.height;
            lg.LGContract(order);
            return r;
        }
    }
    r.peakRank = g.peak;
    r.macs = g.macs;
    r.height = g.height;
    replay_merges(*net, g.merges);
    return r;
}

}  // namespace qtorch
