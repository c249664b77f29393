// MaxCut QAOA workload generation: the per-edge light-cone circuits of
// src/maxcut.h:31-233 / src/maxcut.cpp:166-190 and the seeded x-regular graph
// generator of XregGraphGen/main.cpp:47-126.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/qtorch_gb300.h"

namespace {

struct Graph {
    std::vector<std::pair<int, int>> pairs;
    int num_qubits = 0;
};

// ExtraData::ReadInData (src/maxcut.h:56-103): 'c' lines are comments, 'e a b' edges
Graph read_dgf(const char *text) {
    Graph g;
    std::istringstream in(text);
    char ch;
    int mx = 0;
    while (in >> ch) {
        if (ch != 'e') {
            std::string rest;
            std::getline(in, rest);
            continue;
        }
        int a, b;
        if (!(in >> a >> b)) break;
        mx = std::max(mx, std::max(a, b));
        g.pairs.push_back({a, b});
    }
    g.num_qubits = mx + 1;
    return g;
}

// PopulateIterations / PopulateIterationsHelper (src/maxcut.h:105-186): the
// light cone of one edge, p BFS levels deep, with qubits renumbered in
// discovery order (the first endpoint is qubit 0).
void light_cone(const Graph &g, const std::vector<std::vector<int>> &adj, int edge, int p,
                std::vector<std::pair<int, int>> &real, int &needed) {
    const int n = g.num_qubits;
    const int first = g.pairs[edge].first, second = g.pairs[edge].second;
    std::vector<int> mp(n, -1);
    std::vector<int> working = {first, second};
    mp[first] = 0;
    int qn = 1;
    std::vector<char> new_working(n, 0), checked(n, 0), in_working(n, 0);
    in_working[first] = in_working[second] = 1;
    std::vector<std::pair<int, int>> iters;
    for (int level = 0; level < p; level++) {
        for (int v : working) {
            for (int t : adj[v]) {
                if (checked[t]) continue;
                if (mp[t] == -1) mp[t] = qn++;
                iters.push_back({v, t});
                if (!in_working[t]) new_working[t] = 1;
            }
            checked[v] = 1;
        }
        working.clear();
        std::fill(in_working.begin(), in_working.end(), 0);
        for (int i = 0; i < n; i++)
            if (new_working[i]) {
                working.push_back(i);
                in_working[i] = 1;
            }
        std::fill(new_working.begin(), new_working.end(), 0);
    }
    real.clear();
    for (auto &e : iters) real.push_back({mp[e.first], mp[e.second]});
    needed = qn;
}

std::string fmt_g(double x) {
    // operator<< of a double with default flags: 6 significant digits
    char buf[64];
    std::snprintf(buf, sizeof buf, "%g", x);
    return buf;
}

// outputInitialPlusStateToFile + applyU_CsThenU_Bs (src/maxcut.h:194-233):
// H on every qubit, then per layer i the U_C of every pair (CNOT, Rz(-gamma_i),
// CNOT) and the U_B of every qubit (Rx(2 beta_i)); betas first, then gammas
std::string circuit_text(const std::vector<std::pair<int, int>> &pairs, int nq, int p, const double *bg) {
    std::string q = std::to_string(nq) + "\n";
    for (int i = 0; i < nq; i++) q += "H " + std::to_string(i) + "\n";
    for (int i = 0; i < p; i++) {
        const double gamma = bg[i + p], beta = bg[i];
        for (auto &e : pairs) {
            const std::string a = std::to_string(e.first), b = std::to_string(e.second);
            q += "CNOT " + a + " " + b + "\n";
            q += "Rz " + fmt_g(-gamma) + " " + b + "\n";
            q += "CNOT " + a + " " + b + "\n";
        }
        for (int j = 0; j < nq; j++) q += "Rx " + fmt_g(beta * 2.0) + " " + std::to_string(j) + "\n";
    }
    return q;
}

int64_t copy_out(const std::string &s, char *out, int64_t cap) {
    if (out && cap > 0) {
        const int64_t n = std::min<int64_t>((int64_t) s.size(), cap - 1);
        std::memcpy(out, s.data(), (size_t) n);
        out[n] = 0;
    }
    return (int64_t) s.size() + 1;
}

}  // namespace

extern "C" {

int qt_qaoa_num_edges(const char *dgf_text) {
    if (!dgf_text) return -1;
    return (int) read_dgf(dgf_text).pairs.size();
}

int64_t qt_qaoa_term_text(const char *dgf_text, int p, const double *bg, int edge, char *qasm_out, int64_t qasm_cap,
                          char *measure_out, int64_t measure_cap) {
    if (!dgf_text || !bg || p < 1) return -1;
    Graph g = read_dgf(dgf_text);
    if (edge < 0 || edge >= (int) g.pairs.size()) return -1;
    std::vector<std::vector<int>> adj(g.num_qubits);
    for (auto &e : g.pairs) {
        adj[e.first].push_back(e.second);
        adj[e.second].push_back(e.first);
    }
    std::vector<std::pair<int, int>> real;
    int nq;
    light_cone(g, adj, edge, p, real, nq);
    // F_p (src/maxcut.cpp:171-188) through outputInitialPlusStateToFile / applyU_CsThenU_Bs
    const std::string q = circuit_text(real, nq, p, bg);
    std::string m;
    for (int i = 0; i < nq; i++) m += (i == 0 || i == 1) ? "Z " : "T ";
    copy_out(m, measure_out, measure_cap);
    return copy_out(q, qasm_out, qasm_cap);
}

int64_t qt_qaoa_circuit_text(const char *dgf_text, int p, const double *bg, char *qasm_out, int64_t qasm_cap) {
    if (!dgf_text || !bg || p < 1) return -1;
    const Graph g = read_dgf(dgf_text);
    if (g.pairs.empty()) return -1;
    return copy_out(circuit_text(g.pairs, g.num_qubits, p, bg), qasm_out, qasm_cap);
}

qt_status qt_maxcut_final_string(qt_ctx *ctx, const char *dgf_text, int p, const double *bg, qt_precision prec,
                                 qt_ordering ordering, uint64_t seed, int32_t *bits, int cap_bits, int *n_bits,
                                 int *cut_edges, double *prob, double *marginals) {
    if (!ctx || !dgf_text || !bg || p < 1 || !bits || !n_bits || !cut_edges || !prob) return QT_ERR_INVALID_ARGUMENT;
    if (ordering == QT_ORDER_SEQUENCE) return QT_ERR_INVALID_CONTRACTION_METHOD;
    const Graph g = read_dgf(dgf_text);
    const int n = g.num_qubits;
    if (g.pairs.empty() || cap_bits < n) return QT_ERR_INVALID_ARGUMENT;
    const std::string q = circuit_text(g.pairs, n, p, bg);
    std::string trace;
    for (int i = 0; i < n; i++) trace += "T ";
    // one plan for every query: only the measurement leaves change (|0><0|,
    // |1><1| or the trace on each qubit, all rank 1 and last in leaf order)
    qt_plan *plan = nullptr;
    qt_status s = qt_plan_build(ctx, q.c_str(), trace.c_str(), nullptr, ordering, seed, nullptr, 0, &plan);
    if (s != QT_OK) return s;
    std::vector<double> leaves(2 * qt_plan_leaf_elems(plan));
    s = qt_plan_leaf_values(plan, leaves.data(), leaves.size() / 2);
    qt_batch *batch = nullptr;
    if (s == QT_OK) s = qt_batch_create(ctx, &batch);
    int idx = -1;
    if (s == QT_OK) s = qt_batch_add(batch, plan, nullptr, &idx);
    // maxcutGetFinalString (src/maxcut.cpp:40-122): qubit by qubit, the
    // probability of 0 given the bits chosen so far; ties by a seeded coin
    std::mt19937 coin((uint32_t) seed);
    std::vector<char> answer;
    double current = 1.0;
    const size_t meas0 = leaves.size() - 8 * (size_t) n;   // first measurement leaf (doubles)
    for (int i = 0; i < n && s == QT_OK; i++) {
        for (int j = 0; j < n; j++) {
            double *v = leaves.data() + meas0 + 8 * (size_t) j;
            std::fill(v, v + 8, 0.0);
            if (j < i) v[answer[j] ? 6 : 0] = 1.0;   // |1><1| or |0><0|
            else if (j == i) v[0] = 1.0;             // |0><0|
            else v[0] = v[6] = 1.0;                  // trace
        }
        s = qt_batch_set_leaves(batch, idx, leaves.data());
        double val[2];
        if (s == QT_OK) s = qt_batch_execute(batch, prec, val);
        if (s != QT_OK) break;
        if (marginals) marginals[i] = val[0];
        const double next = val[0] / current;
        if (next > 0.5) {
            current *= next;
            answer.push_back(0);
        } else if (next < 0.5) {
            current *= 1.0 - next;
            answer.push_back(1);
        } else {
            answer.push_back((char) (coin() & 1u));
            current *= 0.5;
        }
    }
    if (batch) qt_batch_free(batch);
    qt_plan_free(plan);
    if (s != QT_OK) return s;
    int cut = 0;
    for (auto &e : g.pairs) cut += answer[e.first] != answer[e.second];
    for (int i = 0; i < n; i++) bits[i] = answer[i];
    *n_bits = n;
    *cut_edges = cut;
    *prob = current;
    return QT_OK;
}

int64_t qt_random_regular_graph(int num_nodes, int degree, uint64_t seed, char *out, int64_t cap) {
    if (num_nodes < 2 || degree < 1 || degree >= num_nodes || (num_nodes * degree) % 2) return -1;
    std::mt19937 gen((std::mt19937::result_type) seed);
    for (int attempt = 0; attempt < 10000; attempt++) {
        // one run of XregGraphGen/main.cpp:47-126: x*n/2 rounds, each trying one
        // pick and then up to 100 more until an edge between two vertices of
        // degree < x that are not yet connected is added
        std::vector<int> deg(num_nodes, 0);
        std::vector<std::vector<char>> conn(num_nodes, std::vector<char>(num_nodes, 0));
        std::uniform_int_distribution<> dist(0, num_nodes - 1);
        std::string text = "c Randomly generated " + std::to_string(num_nodes) + " vertex " + std::to_string(degree) +
                           "regular graph\n";
        auto try_add = [&](int one, int two) {
            if (one == two || deg[one] >= degree || deg[two] >= degree || conn[one][two]) return false;
            conn[one][two] = conn[two][one] = 1;
            deg[one]++;
            deg[two]++;
            text += "e " + std::to_string(one) + " " + std::to_string(two) + "\n";
            return true;
        };
        for (int i = 0; i < degree * num_nodes / 2; i++) {
            const int a0 = dist(gen), b0 = dist(gen);
            bool ok = try_add(a0, b0);
            // the retry loop always makes one more pick before it checks for success
            for (int k = 0; k < 100; k++) {
                const int a = dist(gen), b = dist(gen);
                if (try_add(a, b)) ok = true;
                if (ok) break;
            }
        }
        if (std::all_of(deg.begin(), deg.end(), [&](int d) { return d == degree; })) {
            if (out && cap > 0) {
                const int64_t n = std::min<int64_t>((int64_t) text.size(), cap - 1);
                std::memcpy(out, text.data(), (size_t) n);
                out[n] = 0;
            }
            return (int64_t) text.size() + 1;
        }
    }
    return -1;
}

}  // extern "C"
