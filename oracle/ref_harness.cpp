// Test-infrastructure only: a small driver around the UNMODIFIED qTorch
// headers (compiled from the reference source tree by oracle/Makefile, never
// copied into this repository).  It is used to generate golden vectors that
// pin the CPU oracle port and the CUDA path.  Nothing in the product links or
// runs it.
//
// Sub-commands (all results go to stdout; the reference's own chatter on
// std::cout is discarded):
//   stoch  <qasm> <measure> <threads>       stochastic contraction (ContractionTools.h:219-388)
//                                           -> value, flop counter, recorded mCreatedFrom sequence
//   seq    <qasm> <measure> <seqfile>       ContractGivenSequence replay (ContractionTools.h:392-411)
//   seqtime <qasm> <measure> <seqfile> <seconds>
//                                           the same replay repeated (parse + contraction each time, one
//                                           thread) for at least `seconds`; prints the value, the
//                                           repetitions and the seconds per repetition
//   lg     <qasm> <measure> <qbbfile>       LineGraph::LGContract replay of a qbb.out ordering (LineGraph.h:357-376)
//   lgwires <qasm> <measure>                wire ids assigned by the LineGraph constructor (LineGraph.h:92-171)
//   gates                                   every gate tensor of Node.h for a fixed set of parameters
//   pair   <in.bin> <out.bin>               one ContractIndices call (Network.h:876-971) on raw tensors
//   qaoa   <dgf> <p> <b_1..b_p g_1..g_p>    per-edge light-cone QASM text exactly as maxcut.cpp:166-190 writes it
//   bench  <dgf> <p> <seqfile> <anglesfile> <workers> <workdir>
//                                           the reference's own QAOA objective per step (the F_p body,
//                                           maxcut.cpp:166-196): for every edge term write the QASM and
//                                           measurement files, parse them, contract them with
//                                           ContractGivenSequence (ContractionTools.h:392-411) under a
//                                           recorded ordering.  Terms go to `workers` forked processes
//                                           (dynamic, one term at a time); one step per line of
//                                           anglesfile ("b_1..b_p g_1..g_p"); prints "step <s> <f_p>"
//                                           per step, "value <term> <re> <im>" for the first step, and
//                                           "split <prep> <contract>": worker seconds spent writing and
//                                           parsing the terms' files and contracting them
#include <atomic>
#include <chrono>
#include <cstdio>
#include <new>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>
#include <string>

#include <sys/mman.h>
#include <sys/wait.h>
#include <unistd.h>

#include "maxcut.h"   // pulls in ContractionTools.h, Network.h, Node.h, LineGraph.h, preprocess.h

using namespace qtorch;

static std::ofstream g_null;

static void print_value(const std::complex<double> &v) {
    std::printf("value %.17g %.17g\n", v.real(), v.imag());
}

static void print_sequence(const std::shared_ptr<Network> &net) {
    // the same walk preprocess.h:41-46 makes over mAllNodes
    std::printf("sequence");
    for (const auto &n : net->GetAllNodes()) {
        if (!(n->mCreatedFrom.first == 0 && n->mCreatedFrom.second == 0)) {
            std::printf(" %d %d", n->mCreatedFrom.first, n->mCreatedFrom.second);
        }
    }
    std::printf("\n");
}

// Exposes the protected ContractIndices of the reference Network.
class PairHarness : public Network {
public:
    void run(std::shared_ptr<Node> a, std::shared_ptr<Node> b, std::shared_ptr<Node> c,
             const std::vector<std::pair<bool, int>> &freeIdx, const std::vector<std::pair<int, int>> &sumIdx) {
        std::vector<int> ia(a->mRank), ib(b->mRank);
        ContractIndices(freeIdx, sumIdx, ia, ib, a, b, c);
    }
};

static int cmd_pair(const char *inPath, const char *outPath) {
    // binary layout (int32 little endian then float64):
    // rankA rankB nFree [fromA idx]*nFree nSum [ia ib]*nSum  A(2*4^rA doubles) B(2*4^rB doubles)
    FILE *f = std::fopen(inPath, "rb");
    if (!f) return 2;
    int32_t rA, rB, nF, nS;
    if (std::fread(&rA, 4, 1, f) != 1 || std::fread(&rB, 4, 1, f) != 1 || std::fread(&nF, 4, 1, f) != 1) return 3;
    std::vector<std::pair<bool, int>> freeIdx;
    for (int i = 0; i < nF; i++) {
        int32_t fa, idx;
        if (std::fread(&fa, 4, 1, f) != 1 || std::fread(&idx, 4, 1, f) != 1) return 3;
        freeIdx.push_back({fa != 0, idx});
    }
    if (std::fread(&nS, 4, 1, f) != 1) return 3;
    std::vector<std::pair<int, int>> sumIdx;
    for (int i = 0; i < nS; i++) {
        int32_t ia, ib;
        if (std::fread(&ia, 4, 1, f) != 1 || std::fread(&ib, 4, 1, f) != 1) return 3;
        sumIdx.push_back({ia, ib});
    }
    auto a = std::make_shared<Node>(rA);
    auto b = std::make_shared<Node>(rB);
    auto c = std::make_shared<Node>(nF);
    if (std::fread(a->GetTensorVals().data(), 16, a->GetTensorVals().size(), f) != a->GetTensorVals().size()) return 3;
    if (std::fread(b->GetTensorVals().data(), 16, b->GetTensorVals().size(), f) != b->GetTensorVals().size()) return 3;
    std::fclose(f);
    PairHarness h;
    h.SetNumThreads(1);
    h.run(a, b, c, freeIdx, sumIdx);
    FILE *o = std::fopen(outPath, "wb");
    if (!o) return 2;
    std::fwrite(c->GetTensorVals().data(), 16, c->GetTensorVals().size(), o);
    std::fclose(o);
    return 0;
}

static void dump_node(const char *name, Node &n) {
    std::printf("gate %s %d", name, n.mRank);
    for (const auto &v : n.GetTensorVals()) std::printf(" %.17g %.17g", v.real(), v.imag());
    std::printf("\n");
}

static int cmd_gates(const char *gateDir) {
    const double angles[] = {0.1, -0.1, 0.785399, 2.5, -3.0, 1e-3};
    for (double th : angles) {
        char nm[64];
        float thf = (float) th;  // the parser narrows angles through std::stof (Network.h:342)
        std::snprintf(nm, sizeof nm, "Rx:%.17g", (double) thf); { RxNode n(thf); dump_node(nm, n); }
        std::snprintf(nm, sizeof nm, "Ry:%.17g", (double) thf); { RyNode n(thf); dump_node(nm, n); }
        std::snprintf(nm, sizeof nm, "Rz:%.17g", (double) thf); { RzNode n(thf); dump_node(nm, n); }
        std::snprintf(nm, sizeof nm, "PHASE:%.17g", (double) thf); { PhaseNode n(thf); dump_node(nm, n); }
        std::snprintf(nm, sizeof nm, "CPHASE:%.17g", th); { CPhaseNode n(th); dump_node(nm, n); }
    }
    for (int k = 0; k < 6; k++) {
        char nm[32];
        std::snprintf(nm, sizeof nm, "CRk:%d", k);
        CRkNode n(k);
        dump_node(nm, n);
    }
    { HNode n; dump_node("H", n); }
    { XNode n; dump_node("X", n); }
    { YNode n; dump_node("Y", n); }
    { ZNode n; dump_node("Z", n); }
    { CNOTNode n; dump_node("CNOT", n); }
    { CZNode n; dump_node("CZ", n); }
    { SwapNode n; dump_node("SWAP", n); }
    { ZeroStateNode n; dump_node("INIT", n); }
    { TraceNode n; dump_node("T", n); }
    { XMeasure n; dump_node("MX", n); }
    { YMeasure n; dump_node("MY", n); }
    { ZMeasure n; dump_node("MZ", n); }
    { ProjectZero n; dump_node("M0", n); }
    { ProjectOne n; dump_node("M1", n); }
    if (gateDir) {
        std::string d(gateDir);
        { ArbitraryOneQubitNode n(d + "/../s.gate", "s"); dump_node("ARB1:s.gate", n); }
        { ArbitraryOneQubitNode n(d + "/../t.gate", "t"); dump_node("ARB1:t.gate", n); }
        { ArbitraryOneQubitNode n(d + "/../tdagger.gate", "td"); dump_node("ARB1:tdagger.gate", n); }
        { ArbitraryOneQubitNode n(d + "/../zee.gate", "z"); dump_node("ARB1:zee.gate", n); }
        for (int i = 0; i < 3; i++) {
            char nm[64];
            std::snprintf(nm, sizeof nm, "ARB2:matrix%d.gate", i);
            ArbitraryTwoQubitNode n(d + "/matrix" + std::to_string(i) + ".gate", "m");
            dump_node(nm, n);
        }
    }
    return 0;
}

static int cmd_qaoa(int argc, char **argv) {
    // argv: dgf p betas.. gammas..
    int p = std::atoi(argv[1]);
    std::vector<double> bg;
    for (int i = 0; i < 2 * p; i++) bg.push_back(std::atof(argv[2 + i]));
    ExtraData e(p, argv[0]);
    for (size_t counter = 0; counter < e.pairs.size(); counter++) {
        // the body of F_p (maxcut.cpp:166-190), writing to a string instead of input/tempMaxCut.qasm
        std::string path = "/tmp/qt_ref_harness_term.qasm";
        std::ofstream q(path);
        int numQubits = e.qubitsNeeded[counter];
        q << numQubits << std::endl;
        outputInitialPlusStateToFile(q, numQubits);
        applyU_CsThenU_Bs(e.realIterations[counter], e.p, bg, numQubits, q);
        q.close();
        std::ifstream r(path);
        std::stringstream ss;
        ss << r.rdbuf();
        std::string text = ss.str();
        std::printf("term %zu %d %d %d\n", counter, e.pairs[counter].first, e.pairs[counter].second, numQubits);
        std::printf("%s", text.c_str());
        std::printf("endterm\n");
        std::remove(path.c_str());
    }
    return 0;
}


// ---- bench: the reference's objective evaluation on all host cores -------------

namespace {

// shared between the forked workers: the next term index of the current step
// at offset 0, the values (re, im per term) from offset 64
constexpr size_t kValuesOffset = 64;

bool read_full(int fd, void *buf, size_t n) {
    char *p = static_cast<char *>(buf);
    while (n) {
        ssize_t r = ::read(fd, p, n);
        if (r <= 0) return false;
        p += r;
        n -= (size_t) r;
    }
    return true;
}

bool write_full(int fd, const void *buf, size_t n) {
    const char *p = static_cast<const char *>(buf);
    while (n) {
        ssize_t r = ::write(fd, p, n);
        if (r <= 0) return false;
        p += r;
        n -= (size_t) r;
    }
    return true;
}

// One term exactly as F_p handles it (maxcut.cpp:171-196), with the stochastic
// contraction replaced by the replay of a recorded ordering.
std::complex<double> bench_term(ExtraData &e, size_t k, const std::vector<double> &bg,
                                const std::vector<std::pair<int, int>> &seq, const std::string &qasmPath,
                                const std::string &measPath, double *split) {
    const auto t0 = std::chrono::steady_clock::now();
    std::ofstream q(qasmPath);
    std::ofstream meas(measPath);
    int numQubits = e.qubitsNeeded[k];
    q << numQubits << std::endl;
    outputInitialPlusStateToFile(q, numQubits);
    applyU_CsThenU_Bs(e.realIterations[k], e.p, bg, numQubits, q);
    for (int i = 0; i < numQubits; i++) meas << ((i == 0 || i == 1) ? "Z " : "T ");
    meas.close();
    q.close();
    ContractionTools t(qasmPath, measPath, 1);
    const auto t1 = std::chrono::steady_clock::now();
    t.ContractGivenSequence(seq);
    const std::complex<double> v = t.GetFinalVal();
    const auto t2 = std::chrono::steady_clock::now();
    // [0]: writing and parsing the term's files, [1]: the contraction
    split[0] += std::chrono::duration<double>(t1 - t0).count();
    split[1] += std::chrono::duration<double>(t2 - t1).count();
    return v;
}

}  // namespace

static int cmd_bench(char **argv) {
    const char *dgf = argv[0];
    int p = std::atoi(argv[1]);
    const char *seqPath = argv[2], *anglesPath = argv[3];
    int workers = std::max(1, std::atoi(argv[4]));
    std::string workdir = argv[5];

    ExtraData e(p, dgf);
    size_t nTerms = e.pairs.size();
    // seqfile: one line per term, "a b a b ..." (node-id pairs of GetAllNodes())
    std::vector<std::vector<std::pair<int, int>>> seqs;
    {
        std::ifstream f(seqPath);
        std::string line;
        while (std::getline(f, line)) {
            std::istringstream ls(line);
            std::vector<std::pair<int, int>> s;
            int a, b;
            while (ls >> a >> b) s.push_back({a, b});
            seqs.push_back(s);
        }
    }
    if (seqs.size() != nTerms) {
        std::fprintf(stderr, "bench: %zu sequences for %zu terms\n", seqs.size(), nTerms);
        return 3;
    }
    std::vector<std::vector<double>> steps;
    {
        std::ifstream f(anglesPath);
        std::string line;
        while (std::getline(f, line)) {
            std::istringstream ls(line);
            std::vector<double> bg;
            double x;
            while (ls >> x) bg.push_back(x);
            if ((int) bg.size() == 2 * p) steps.push_back(bg);
        }
    }

    size_t shBytes = kValuesOffset + sizeof(double) * 2 * nTerms + sizeof(double) * 2 * (size_t) workers;
    void *mem = mmap(nullptr, shBytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    if (mem == MAP_FAILED) return 5;
    std::atomic<long> *next = new (mem) std::atomic<long>(0);
    double *values = reinterpret_cast<double *>(static_cast<char *>(mem) + kValuesOffset);
    double *splits = values + 2 * nTerms;   // per worker: file write + parse seconds, contraction seconds

    std::vector<int> toChild(workers), fromChild(workers);
    std::vector<pid_t> pids(workers);
    for (int w = 0; w < workers; w++) {
        int a[2], b[2];
        if (pipe(a) || pipe(b)) return 5;
        pid_t pid = fork();
        if (pid < 0) return 5;
        if (pid == 0) {
            ::close(a[1]);
            ::close(b[0]);
            std::string qp = workdir + "/tempMaxCut" + std::to_string(w) + ".qasm";
            std::string mp = workdir + "/measureTest" + std::to_string(w) + ".txt";
            int32_t s;
            while (read_full(a[0], &s, sizeof s) && s >= 0) {
                const std::vector<double> &bg = steps[(size_t) s];
                int32_t ok = 1;
                try {
                    for (long k; (k = next->fetch_add(1)) < (long) nTerms;) {
                        std::complex<double> v = bench_term(e, (size_t) k, bg, seqs[(size_t) k], qp, mp, splits + 2 * w);
                        values[2 * k] = v.real();
                        values[2 * k + 1] = v.imag();
                    }
                } catch (std::exception &) {
                    ok = 0;
                }
                if (!write_full(b[1], &ok, sizeof ok)) break;
            }
            std::remove(qp.c_str());
            std::remove(mp.c_str());
            _exit(0);
        }
        ::close(a[0]);
        ::close(b[1]);
        toChild[w] = a[1];
        fromChild[w] = b[0];
        pids[w] = pid;
    }

    int rc = 0;
    for (size_t s = 0; s < steps.size() && rc == 0; s++) {
        next->store(0);
        auto t0 = std::chrono::steady_clock::now();
        int32_t cmd = (int32_t) s;
        for (int w = 0; w < workers; w++) write_full(toChild[w], &cmd, sizeof cmd);
        for (int w = 0; w < workers; w++) {
            int32_t ok = 0;
            if (!read_full(fromChild[w], &ok, sizeof ok) || !ok) rc = 4;
        }
        double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        double fp = 0.0;   // F_p (maxcut.cpp:196)
        for (size_t k = 0; k < nTerms; k++) fp += 0.5 * (1.0 - values[2 * k]);
        std::printf("step %zu %.9f %.17g\n", s, sec, fp);
        if (s == 0) {
            for (size_t k = 0; k < nTerms; k++)
                std::printf("value %zu %.17g %.17g\n", k, values[2 * k], values[2 * k + 1]);
        }
        std::fflush(stdout);
    }
    double prep = 0, contract = 0;
    for (int w = 0; w < workers; w++) {
        prep += splits[2 * w];
        contract += splits[2 * w + 1];
    }
    std::printf("split %.9f %.9f\n", prep, contract);   // summed over the workers and steps
    int32_t stop = -1;
    for (int w = 0; w < workers; w++) {
        write_full(toChild[w], &stop, sizeof stop);
        ::close(toChild[w]);
        ::close(fromChild[w]);
    }
    for (int w = 0; w < workers; w++) waitpid(pids[w], nullptr, 0);
    munmap(mem, shBytes);
    return rc;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s stoch|seq|lg|lgwires|gates|pair|qaoa|bench ...\n", argv[0]);
        return 1;
    }
    g_null.open("/dev/null");
    std::streambuf *orig = std::cout.rdbuf(g_null.rdbuf());
    std::string cmd(argv[1]);
    int rc = 0;
    try {
        if (cmd == "stoch" && argc >= 5) {
            ContractionTools t(argv[2], argv[3], std::atoi(argv[4]));
            auto net = t.Contract(Stochastic);
            print_value(t.GetFinalVal());
            std::printf("flops %lld\n", net->getNumFloatOps());
            print_sequence(net);
        } else if (cmd == "seq" && argc >= 5) {
            std::vector<std::pair<int, int>> seq;
            std::ifstream s(argv[4]);
            int a, b;
            while (s >> a >> b) seq.push_back({a, b});
            ContractionTools t(argv[2], argv[3], 1);
            auto net = t.ContractGivenSequence(seq);
            print_value(t.GetFinalVal());
            std::printf("flops %lld\n", net->getNumFloatOps());
        } else if (cmd == "seqtime" && argc >= 6) {
            std::vector<std::pair<int, int>> seq;
            std::ifstream s(argv[4]);
            int a, b;
            while (s >> a >> b) seq.push_back({a, b});
            const double budget = std::atof(argv[5]);
            std::complex<double> v;
            long reps = 0;
            const auto t0 = std::chrono::steady_clock::now();
            double el = 0;
            do {
                ContractionTools t(argv[2], argv[3], 1);
                t.ContractGivenSequence(seq);
                v = t.GetFinalVal();
                reps++;
                el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            } while (el < budget);
            print_value(v);
            std::printf("reps %ld\nseconds_per_rep %.9g\n", reps, el / (double) reps);
        } else if (cmd == "lg" && argc >= 5) {
            auto net = std::make_shared<Network>(argv[2], argv[3]);
            net->SetNumThreads(1);
            LineGraph lg(net);
            lg.SetQBBOutFiles("/dev/null", argv[4], "/dev/null");
            lg.LGContract();
            print_value(net->GetFinalValue());
            auto rem = net->GetUncontractedNodes();
            print_value(rem[0]->GetTensorVals()[0]);
            std::printf("flops %lld\n", net->getNumFloatOps());
            print_sequence(net);
        } else if (cmd == "reduce" && argc >= 4) {
            // ReduceCircuit (Network.h:1015-1118), then a stochastic contraction
            auto net = std::make_shared<Network>(argv[2], argv[3]);
            net->SetNumThreads(1);
            net->ReduceCircuit();
            std::printf("reduced_nodes %zu %zu\n", net->GetAllNodes().size(), net->GetUncontractedNodes().size());
            print_sequence(net);
            ContractionTools t(net);
            t.Contract(Stochastic);
            print_value(t.GetFinalVal());
            print_sequence(net);
        } else if (cmd == "lgwires" && argc >= 4) {
            auto net = std::make_shared<Network>(argv[2], argv[3]);
            LineGraph lg(net);
            for (const auto &n : net->GetUncontractedNodes()) {
                std::printf("node %d", n->mID);
                for (const auto &w : n->GetWires()) {
                    std::printf(" %d:%d:%d", w->GetWireID(), w->GetNodeA().lock()->mID, w->GetNodeB().lock()->mID);
                }
                std::printf("\n");
            }
        } else if (cmd == "gates") {
            rc = cmd_gates(argc >= 3 ? argv[2] : nullptr);
        } else if (cmd == "pair" && argc >= 4) {
            rc = cmd_pair(argv[2], argv[3]);
        } else if (cmd == "bench" && argc >= 8) {
            rc = cmd_bench(argv + 2);
        } else if (cmd == "qaoa" && argc >= 4) {
            rc = cmd_qaoa(argc - 2, argv + 2);
        } else {
            std::fprintf(stderr, "bad command\n");
            rc = 1;
        }
    } catch (std::exception &e) {
        std::printf("exception %s\n", e.what());
        rc = 4;
    }
    std::cout.rdbuf(orig);
    return rc;
}
