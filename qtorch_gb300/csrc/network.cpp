// Node / Wire / Network on the GB300 engine.
//
// Bookkeeping follows the reference one to one, because node ids, wire order
// and the free-index order of every contraction decide both the values and the
// replayability of orderings:
//   parse          src/Network.h:246-304 (ParseNetwork), 326-707 (ParseNode),
//                  177-194 (initial states), 199-240 (measurements), 976-992 (tokenizer)
//   ContractNodes  src/Network.h:715-864
//   gate tables    src/Node.h:197-898, built from U (x) U* with the same expressions
// The arithmetic of a contraction runs on the GPU (qt_contract_pair).
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/qtorch/qtorch.hpp"
#include "core.h"

namespace qtorch {

// ===========================================================================
// gate tensors

namespace {

constexpr double kPi = 3.14159265358979323846;   // src/Node.h:45

inline std::complex<double> mul_conj(std::complex<double> x, std::complex<double> y) {
    // x * conj(y) rounded as std::complex<double>::operator* (no fused multiply-add)
    const double ar = x.real(), ai = x.imag(), br = y.real(), bi = -y.imag();
    volatile double p1 = ar * br, p2 = ai * bi, p3 = ar * bi, p4 = ai * br;
    return {p1 - p2, p3 + p4};
}

// T[in + 4*out], in = 2r + c, out = 2r' + c', T = U[r'][r] conj(U[c'][c])
void superop1(const std::complex<double> *u, std::complex<double> *t) {
    for (int in = 0; in < 4; in++)
        for (int out = 0; out < 4; out++) {
            const int r = in >> 1, c = in & 1, rp = out >> 1, cp = out & 1;
            t[in + 4 * out] = mul_conj(u[2 * rp + r], u[2 * cp + c]);
        }
}

// wires [in_q1, in_q2, out_q1, out_q2]; T = U[2r1'+r2'][2r1+r2] conj(U[2c1'+c2'][2c1+c2])
void superop2(const std::complex<double> *u, std::complex<double> *t) {
    for (int i1 = 0; i1 < 4; i1++)
        for (int i2 = 0; i2 < 4; i2++)
            for (int o1 = 0; o1 < 4; o1++)
                for (int o2 = 0; o2 < 4; o2++) {
                    const int rowr = 2 * (o1 >> 1) + (o2 >> 1), colr = 2 * (i1 >> 1) + (i2 >> 1);
                    const int rowc = 2 * (o1 & 1) + (o2 & 1), colc = 2 * (i1 & 1) + (i2 & 1);
                    t[i1 + 4 * i2 + 16 * o1 + 64 * o2] = mul_conj(u[4 * rowr + colr], u[4 * rowc + colc]);
                }
}

inline void fold_negative_zero(std::vector<std::complex<double>> &v) {
    for (auto &x : v) x = {x.real() + 0.0, x.imag() + 0.0};
}

class GateNode : public Node {
public:
    GateNode(int rank, GateType type, const std::string &name, double angle = 0.0) : Node(rank), mAngle(angle) {
        mType = type;
        mStringType = name;
    }
    std::vector<std::complex<double>> &Vals() { return mVals; }
    double mAngle;
};

void set1(std::vector<std::complex<double>> &t, int in, int out, std::complex<double> v) { t[in + 4 * out] = v; }

}  // namespace

std::shared_ptr<Node> MakeGateNode(const std::string &kind, double param) {
    using C = std::complex<double>;
    if (kind == "INIT" || kind == "T" || kind == "MX" || kind == "MY" || kind == "MZ" || kind == "M0" || kind == "M1") {
        // rank-1 vectors over s = 2r + c (src/Node.h ZeroStateNode .. ProjectZero)
        GateType ty = kind == "INIT" ? GateType::INITSTATE : GateType::MEASURETRACE;
        const char *label = kind == "INIT" ? "|0><0|" : kind == "T" ? "Trace" : kind == "MX" ? "X measure"
                          : kind == "MY" ? "Y measure" : kind == "MZ" ? "Z measure" : kind == "M0" ? "|0><0| measure"
                          : "|1><1| measure";
        auto n = std::make_shared<GateNode>(1, ty, label);
        auto &v = n->Vals();
        if (kind == "INIT" || kind == "M0") v[0] = 1.0;
        else if (kind == "M1") v[3] = 1.0;
        else if (kind == "T") { v[0] = 1.0; v[3] = 1.0; }
        else if (kind == "MZ") { v[0] = 1.0; v[3] = -1.0; }
        else if (kind == "MX") { v[1] = 1.0; v[2] = 1.0; }
        else { v[1] = C(0, 1.0); v[2] = C(0, -1.0); }
        return n;
    }
    if (kind == "Rx" || kind == "Ry") {
        // the parser narrows the angle with std::stof (src/Network.h:342, 383)
        const double th = (double) (float) param;
        const double cc = std::pow(std::cos(th / 2.0), 2);
        const double ss = std::pow(std::sin(th / 2.0), 2);
        const double sh = std::sin(th) / 2.0;
        auto n = std::make_shared<GateNode>(2, kind == "Rx" ? GateType::RX : GateType::RY, kind, param);
        auto &t = n->Vals();
        set1(t, 0, 0, cc); set1(t, 1, 1, cc); set1(t, 2, 2, cc); set1(t, 3, 3, cc);
        if (kind == "Rx") {
            set1(t, 0, 3, ss); set1(t, 1, 2, ss); set1(t, 2, 1, ss); set1(t, 3, 0, ss);
            set1(t, 0, 1, C(0, sh)); set1(t, 1, 0, C(0, sh)); set1(t, 2, 3, C(0, sh)); set1(t, 3, 2, C(0, sh));
            set1(t, 0, 2, C(0, -1.0 * sh)); set1(t, 1, 3, C(0, -1.0 * sh));
            set1(t, 2, 0, C(0, -1.0 * sh)); set1(t, 3, 1, C(0, -1.0 * sh));
        } else {
            const double mss = -1.0 * std::pow(std::sin(th / 2), 2);
            const double msh = -1.0 * std::sin(th) / 2.0;
            set1(t, 0, 3, ss); set1(t, 3, 0, ss); set1(t, 1, 2, mss); set1(t, 2, 1, mss);
            set1(t, 0, 1, sh); set1(t, 0, 2, sh); set1(t, 1, 3, sh); set1(t, 2, 3, sh);
            set1(t, 1, 0, msh); set1(t, 2, 0, msh); set1(t, 3, 1, msh); set1(t, 3, 2, msh);
        }
        return n;
    }
    if (kind == "Rz" || kind == "PHASE") {
        const double th = (double) (float) param;
        auto n = std::make_shared<GateNode>(2, kind == "Rz" ? GateType::RZ : GateType::PHASE, kind == "Rz" ? "Rz" : "Phase",
                                            param);
        auto &t = n->Vals();
        set1(t, 0, 0, 1.0);
        set1(t, 3, 3, 1.0);
        set1(t, 1, 1, C(std::cos(th), -1.0 * std::sin(th)));
        set1(t, 2, 2, C(std::cos(th), std::sin(th)));
        return n;
    }
    if (kind == "H" || kind == "X" || kind == "Y" || kind == "Z") {
        C u[4];
        GateType ty = GateType::HADAMARD;
        if (kind == "H") { u[0] = 1; u[1] = 1; u[2] = 1; u[3] = -1; }
        else if (kind == "X") { u[0] = 0; u[1] = 1; u[2] = 1; u[3] = 0; ty = GateType::X; }
        else if (kind == "Y") { u[0] = 0; u[1] = C(0, -1); u[2] = C(0, 1); u[3] = 0; ty = GateType::Y; }
        else { u[0] = 1; u[1] = 0; u[2] = 0; u[3] = -1; ty = GateType::Z; }
        auto n = std::make_shared<GateNode>(2, ty, kind);
        superop1(u, n->Vals().data());
        if (kind == "H")
            for (auto &x : n->Vals()) x *= 0.5;   // entries are exactly +-1/2
        fold_negative_zero(n->Vals());
        return n;
    }
    if (kind == "CNOT" || kind == "CZ" || kind == "SWAP") {
        C u[16];
        for (auto &x : u) x = 0.0;
        for (int x = 0; x < 4; x++) {
            const int q1 = x >> 1, q2 = x & 1;   // basis index 2*q1 + q2
            if (kind == "CNOT") u[4 * (2 * q1 + (q2 ^ q1)) + x] = 1.0;
            else if (kind == "SWAP") u[4 * (2 * q2 + q1) + x] = 1.0;
            else u[4 * x + x] = (q1 && q2) ? -1.0 : 1.0;
        }
        auto n = std::make_shared<GateNode>(4, kind == "CNOT" ? GateType::CNOT : kind == "CZ" ? GateType::CZ : GateType::SWAP, kind);
        superop2(u, n->Vals().data());
        fold_negative_zero(n->Vals());
        return n;
    }
    if (kind == "CPHASE" || kind == "CRk") {
        // controlled phase diag(1,1,1,e^{i phi}) (src/Node.h CPhaseNode, CRkNode)
        C em, ep;
        if (kind == "CPHASE") {
            em = C(std::cos(param), -1.0 * std::sin(param));
            ep = C(std::cos(param), std::sin(param));
        } else {
            // exp(2 pi (0,-1) / 2^(k+1)), k = the control qubit index (src/Network.h:571)
            em = std::exp(2.0 * kPi * C(0, -1) / std::pow(2, param + 1.0));
            ep = std::exp(2.0 * kPi * C(0, 1) / std::pow(2, param + 1.0));
        }
        auto n = std::make_shared<GateNode>(4, kind == "CPHASE" ? GateType::CPHASE : GateType::CRK,
                                            kind == "CPHASE" ? "CPhase" : "CRk", param);
        auto &t = n->Vals();
        for (int i1 = 0; i1 < 4; i1++)
            for (int i2 = 0; i2 < 4; i2++) {
                const bool rowph = (i1 >> 1) && (i2 >> 1), colph = (i1 & 1) && (i2 & 1);
                C v = 1.0;
                if (rowph && !colph) v = ep;
                else if (!rowph && colph) v = em;
                t[i1 + 4 * i2 + 16 * i1 + 64 * i2] = v;
            }
        return n;
    }
    throw InvalidFileFormat();
}

double GateAngle(const Node &n) {
    const auto *g = dynamic_cast<const GateNode *>(&n);
    return g ? g->mAngle : 0.0;
}

std::shared_ptr<Node> MakeArbitraryNode(const std::string &path, const std::string &name, bool twoQubit) {
    std::ifstream in(path);
    if (!in.is_open()) throw InvalidFile();
    const int nv = twoQubit ? 16 : 4;
    std::vector<std::complex<double>> u(nv);
    for (int i = 0; i < nv; i++) {
        if (in.eof()) throw InvalidFileFormat();
        in >> u[i];   // "(re,im)" or "re", as the reference reads them
        if (in.fail()) throw InvalidFileFormat();
    }
    auto n = std::make_shared<GateNode>(twoQubit ? 4 : 2,
                                        twoQubit ? GateType::ARBITRARYTWOQUBITUNITARY : GateType::ARBITRARYONEQUBITUNITARY, name);
    if (twoQubit) superop2(u.data(), n->Vals().data());
    else superop1(u.data(), n->Vals().data());
    return n;
}

// ===========================================================================
// Node

Node::Node(int rank) : mRank(rank) {
    if (rank < 0 || rank > qtg::kMaxWires) throw InvalidFunctionInput();
    mVals.assign((size_t) 1 << (2 * rank), std::complex<double>(0.0));
}

Node::Node(int rank, NoData) : mRank(rank) {
    if (rank < 0 || rank > qtg::kMaxWires) throw InvalidFunctionInput();
    mHostValid = false;
}

Node::~Node() {
    if (mDevice && mCtx) qt_tensor_free(mCtx, mDevice);
}

const std::complex<double> &Node::Access(const std::vector<int> &idx) {
    unsigned long long s = 0;
    for (size_t i = 0; i < idx.size(); i++) s += (unsigned long long) idx[i] << (2 * i);
    return GetTensorVals().at(s);
}

const std::complex<double> &Node::Access(const long long &index) { return GetTensorVals().at(index); }

std::complex<double> &Node::Index(const std::vector<int> &idx) {
    unsigned long long s = 0;
    for (size_t i = 0; i < idx.size(); i++) s += (unsigned long long) idx[i] << (2 * i);
    auto &v = GetTensorVals();
    if (mDevice && mCtx) { qt_tensor_free(mCtx, mDevice); mDevice = nullptr; }   // host copy becomes the truth
    return v[s];
}

std::complex<double> &Node::Index(const long long &index) {
    auto &v = GetTensorVals();
    if (mDevice && mCtx) { qt_tensor_free(mCtx, mDevice); mDevice = nullptr; }
    return v[index];
}

void Node::ClearNodeData() {
    mVals = std::vector<std::complex<double>>();
    mHostValid = false;
    if (mDevice && mCtx) qt_tensor_free(mCtx, mDevice);
    mDevice = nullptr;
}

std::vector<std::complex<double>> &Node::GetTensorVals() {
    if (!mHostValid && mDevice && mCtx) {
        mVals.resize((size_t) 1 << (2 * mRank));
        qt_status s = qt_tensor_download(mCtx, mDevice, mVals.data(), mVals.size() * sizeof(std::complex<double>));
        if (s != QT_OK) throw EngineFailure(s);
        mHostValid = true;
    }
    return mVals;
}

qt_tensor *Node::DeviceTensor(qt_ctx *ctx) {
    if (mDevice) return mDevice;
    if (!mHostValid) throw InvalidFunctionInput();   // Network.h:938-940
    qt_tensor *t = nullptr;
    qt_status s = qt_tensor_create(ctx, mRank, QT_C128, &t);
    if (s != QT_OK) throw EngineFailure(s);
    s = qt_tensor_upload(ctx, t, mVals.data(), mVals.size() * sizeof(std::complex<double>));
    if (s != QT_OK) {
        qt_tensor_free(ctx, t);
        throw EngineFailure(s);
    }
    mDevice = t;
    mCtx = ctx;
    return t;
}

void Node::AdoptDeviceTensor(qt_ctx *ctx, qt_tensor *t) {
    if (mDevice && mCtx) qt_tensor_free(mCtx, mDevice);
    mDevice = t;
    mCtx = ctx;
    mHostValid = false;
    mVals = std::vector<std::complex<double>>();
}

// ===========================================================================
// Network

static std::mutex g_default_ctx_lock;
static qt_ctx *g_default_ctx = nullptr;

qt_ctx *Network::DefaultContext() {
    std::lock_guard<std::mutex> g(g_default_ctx_lock);
    if (!g_default_ctx) {
        qt_status s = qt_ctx_create(0, nullptr, &g_default_ctx);
        if (s != QT_OK) throw EngineFailure(s);
    }
    return g_default_ctx;
}

Network::Network() {}

Network::~Network() {}

static bool read_file(const std::string &path, std::string &out) {
    std::ifstream in(path, std::ios::binary);
    if (!in.is_open()) return false;
    std::stringstream ss;
    ss << in.rdbuf();
    out = ss.str();
    return true;
}

Network::Network(const std::string &inputFile, const std::string &measureFile, qt_ctx *ctx)
    : mInputFile(inputFile), mMeasureFile(measureFile), mCtx(ctx) {
    if (!read_file(inputFile, mQasmText)) {
        mFailure = true;
        throw InvalidFile();
    }
    // an unreadable measurement file traces every qubit out (Network.h:286-288)
    if (!read_file(measureFile, mMeasureText)) mMeasureText.clear();
    ParseNetwork(mQasmText);
}

std::shared_ptr<Network> Network::FromText(const std::string &qasm, const std::string &measure,
                                           const std::string &gateDir, qt_ctx *ctx) {
    auto n = std::make_shared<Network>();
    n->mCtx = ctx;
    n->mQasmText = qasm;
    n->mMeasureText = measure;
    n->mGateDir = gateDir;
    n->ParseNetwork(qasm);
    return n;
}

void Network::Reset() {
    mParsingWires.clear();
    mFinalVal = 0.0;
    mNumberOfQubits = 0;
    mDone = false;
    mFailure = false;
    mAllNodes.clear();
    mNodesByWire.clear();
    mUncontractedNodes.clear();
    mArbitraryOneQubitGates.clear();
    mArbitraryTwoQubitGates.clear();
    mSteps.clear();
    mLeaves.clear();
    mNextTensorId = 0;
    ParseNetwork(mQasmText);
}

void Network::CreateInitialStates() {
    for (int i = 0; i < mNumberOfQubits; i++) {
        auto n = MakeGateNode("INIT", 0.0);
        auto w = std::make_shared<Wire>(n, nullptr, i);
        n->GetWires().push_back(w);
        mParsingWires.push_back(w);
        mAllNodes.push_back(n);
        n->AddWireNumber(i);
        mNodesByWire[i].push_back(n);
        n->mID = (int) mAllNodes.size() - 1;
    }
}

void Network::AddMeasurementsOrTrace(const std::string &measureText) {
    // one non-space character per qubit, missing entries trace out (Network.h:290-298)
    size_t pos = 0;
    for (int i = 0; i < mNumberOfQubits; i++) {
        while (pos < measureText.size() && std::isspace((unsigned char) measureText[pos])) pos++;
        char ch = 'T';
        if (pos < measureText.size()) ch = measureText[pos++];
        const char *kind = ch == 'X' ? "MX" : ch == 'Y' ? "MY" : ch == 'Z' ? "MZ" : ch == '0' ? "M0" : ch == '1' ? "M1" : "T";
        auto n = MakeGateNode(kind, 0.0);
        mParsingWires[i]->SetNodeB(n);
        n->GetWires().push_back(mParsingWires[i]);
        mAllNodes.push_back(n);
        n->AddWireNumber(i);
        mNodesByWire[i].push_back(n);
        n->mID = (int) mAllNodes.size() - 1;
    }
}

// std::stoi / std::stof / std::stod that report failure instead of throwing
static bool to_int(const std::string &s, int &v) {
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    long x = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || errno) return false;
    v = (int) x;
    return true;
}

static bool to_float(const std::string &s, float &v) {
    char *end = nullptr;
    errno = 0;
    float x = std::strtof(s.c_str(), &end);
    if (end == s.c_str() || errno == ERANGE) return false;
    v = x;
    return true;
}

static bool to_double(const std::string &s, double &v) {
    char *end = nullptr;
    errno = 0;
    double x = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || errno == ERANGE) return false;
    v = x;
    return true;
}

// Network.h:976-992: split on single spaces keeping empty tokens, dropping an
// empty final piece; lines starting with '#' are comments
static void tokenize(const std::string &line, std::vector<std::string> &out) {
    out.clear();
    if (line.empty() || line[0] == '#') return;
    size_t start = 0;
    for (;;) {
        size_t sp = line.find(' ', start);
        if (sp == std::string::npos) {
            if (start < line.size()) out.push_back(line.substr(start));
            break;
        }
        out.push_back(line.substr(start, sp - start));
        start = sp + 1;
    }
}

void Network::Attach(const std::shared_ptr<Node> &n, const int *q, int nq) {
    for (int i = 0; i < nq; i++) {
        n->GetWires().push_back(mParsingWires[q[i]]);
        mParsingWires[q[i]]->SetNodeB(n);
    }
    for (int i = 0; i < nq; i++) {
        auto w = std::make_shared<Wire>(n, nullptr, q[i]);
        mParsingWires[q[i]] = w;
        n->GetWires().push_back(w);
    }
    for (int i = 0; i < nq; i++) n->AddWireNumber(q[i]);
    if (nq == 1) n->mIndexOfPreviousNode = (int) mNodesByWire[q[0]].size() - 1;
    for (int i = 0; i < nq; i++) mNodesByWire[q[i]].push_back(n);
}

void Network::ParseNode(std::string &line) {
    std::vector<std::string> t;
    tokenize(line, t);
    if (t.empty()) return;
    const std::string &g = t[0];
    const int nq = mNumberOfQubits;
    std::shared_ptr<Node> node;
    int q[2];
    auto one_qubit = [&](size_t qi) {
        if (t.size() <= qi || !to_int(t[qi], q[0]) || q[0] > nq - 1 || q[0] < 0) throw InvalidFileFormat();
    };
    auto two_qubit = [&](size_t qi) {
        if (t.size() <= qi + 1 || !to_int(t[qi], q[0]) || !to_int(t[qi + 1], q[1])) throw InvalidFileFormat();
        if (q[0] > nq - 1 || q[1] > nq - 1 || q[0] == q[1] || q[0] < 0 || q[1] < 0) throw InvalidFileFormat();
    };
    if (g == "Rx" || g == "RX" || g == "Ry" || g == "RY" || g == "Rz" || g == "RZ" || g == "PHASE") {
        float th;
        if (t.size() < 2 || !to_float(t[1], th)) throw InvalidFileFormat();
        const char *kind = (g == "Rx" || g == "RX") ? "Rx" : (g == "Ry" || g == "RY") ? "Ry" : g == "PHASE" ? "PHASE" : "Rz";
        node = MakeGateNode(kind, (double) th);
        one_qubit(2);
        Attach(node, q, 1);
    } else if (g == "H" || g == "X" || g == "Y" || g == "Z") {
        node = MakeGateNode(g, 0.0);
        one_qubit(1);
        Attach(node, q, 1);
    } else if (g == "CNOT" || g == "SWAP" || g == "CRk" || g == "CZ") {
        two_qubit(1);
        node = MakeGateNode(g, (double) q[0]);   // CRk phase from the control index (Network.h:571)
        Attach(node, q, 2);
    } else if (g == "CPHASE") {
        double th;
        if (t.size() < 2 || !to_double(t[1], th)) throw InvalidFileFormat();
        two_qubit(2);
        node = MakeGateNode("CPHASE", th);
        Attach(node, q, 2);
    } else if (g == "def1" || g == "def2") {
        if (t.size() < 3) throw InvalidFileFormat();
        auto &m = g == "def1" ? mArbitraryOneQubitGates : mArbitraryTwoQubitGates;
        m.insert({t[1], t[2]});   // the first definition wins, as unordered_map::insert does
        return;
    } else if (mArbitraryOneQubitGates.count(g)) {
        std::string path = mArbitraryOneQubitGates[g];
        if (!mGateDir.empty() && !path.empty() && path[0] != '/') path = mGateDir + "/" + path;
        node = MakeArbitraryNode(path, g, false);
        one_qubit(1);
        Attach(node, q, 1);
    } else if (mArbitraryTwoQubitGates.count(g)) {
        std::string path = mArbitraryTwoQubitGates[g];
        if (!mGateDir.empty() && !path.empty() && path[0] != '/') path = mGateDir + "/" + path;
        node = MakeArbitraryNode(path, g, true);
        two_qubit(1);
        Attach(node, q, 2);
    } else {
        throw InvalidFileFormat();
    }
    mAllNodes.push_back(node);
    node->mID = (int) mAllNodes.size() - 1;
}

void Network::ParseNetwork(const std::string &qasm) {
    mAllNodes.reserve(1024);
    size_t pos = qasm.find('\n');
    std::string first = qasm.substr(0, pos);
    int nq;
    if (!to_int(first, nq) || nq < 0) {
        mFailure = true;
        throw InvalidFileFormat();
    }
    mNumberOfQubits = nq;
    mNodesByWire.assign(nq, {});
    CreateInitialStates();
    while (pos != std::string::npos) {
        size_t next = qasm.find('\n', pos + 1);
        std::string line = qasm.substr(pos + 1, next == std::string::npos ? std::string::npos : next - pos - 1);
        ParseNode(line);
        pos = next;
    }
    AddMeasurementsOrTrace(mMeasureText);
    mParsingWires.clear();
    mUncontractedNodes = mAllNodes;
    mLeaves = mAllNodes;
    for (auto &n : mAllNodes) n->mTensorId = mNextTensorId++;
}

void Network::ContractNetworkLinearly() {
    while (!mDone) {
        auto &w = mUncontractedNodes[0]->GetWires()[0];
        auto a = w->GetNodeA().lock(), b = w->GetNodeB().lock();
        if (!a || !b) throw InvalidContractionMethod();
        ContractNodes(a, b, 1000);
    }
}

void Network::FindAndRemove(std::vector<std::shared_ptr<Node>> &v, const std::shared_ptr<Node> &x) {
    for (size_t i = 0; i < v.size(); i++)
        if (v[i] == x) {
            v.erase(v.begin() + i);
            return;
        }
}

void Network::FindAndReplace(std::vector<std::shared_ptr<Node>> &v, const std::shared_ptr<Node> &x,
                             const std::shared_ptr<Node> &y) {
    for (auto &e : v)
        if (e == x) {
            e = y;
            return;
        }
}

void Network::FindAndReplace(std::vector<std::vector<std::shared_ptr<Node>>> &v, const std::shared_ptr<Node> &x,
                             const std::shared_ptr<Node> &y) {
    int count = 0;
    for (auto &row : v)
        for (auto &e : row) {
            if (e == x) {
                e = y;
                count++;
            }
            if (count >= 2) break;
        }
}

std::shared_ptr<Node> Network::ContractNodes(std::shared_ptr<Node> nodeA, std::shared_ptr<Node> nodeB, int threshold) {
    std::unique_lock<std::mutex> guard(mLocker);
    if (!nodeA || !nodeB || nodeA->mContracted || nodeB->mContracted) return nullptr;
    std::vector<int> indicesA, indicesB;
    std::vector<std::pair<bool, int>> indicesC;
    std::vector<std::shared_ptr<Wire>> connected, remaining;
    auto &wa = nodeA->GetWires();
    auto &wb = nodeB->GetWires();
    for (int i = 0; i < (int) wa.size(); i++) {
        auto &w = wa[i];
        if (w->GetNodeB().lock() == nodeB || w->GetNodeA().lock() == nodeB) {
            indicesA.push_back(i);
            connected.push_back(w);
        } else {
            indicesC.push_back({true, i});
            remaining.push_back(w);
        }
    }
    for (auto &cw : connected)
        for (int k = 0; k < (int) wb.size(); k++)
            if (cw == wb[k]) indicesB.push_back(k);
    for (int j = 0; j < (int) wb.size(); j++) {
        auto &w = wb[j];
        if (!(w->GetNodeB().lock() == nodeA || w->GetNodeA().lock() == nodeA)) {
            indicesC.push_back({false, j});
            remaining.push_back(w);
        }
    }
    // refusal rule of Network.h:772-777
    if ((indicesA.empty() && !indicesC.empty() && !mAllowOuter) ||
        (int) remaining.size() > std::max(nodeA->mRank, nodeB->mRank) + threshold)
        return nullptr;
    if (indicesA.size() != indicesB.size()) return nullptr;   // a wire listed twice: not a tensor network edge
    std::vector<std::pair<int, int>> pairs(indicesA.size());
    for (size_t k = 0; k < indicesA.size(); k++) pairs[k] = {indicesA[k], indicesB[k]};

    auto nodeC = std::make_shared<Node>((int) indicesC.size(), Node::NoData{});
    nodeC->mTensorId = mNextTensorId++;
    for (auto &w : remaining) {
        nodeC->GetWires().push_back(w);
        if (w->GetNodeA().lock() == nodeA || w->GetNodeA().lock() == nodeB) w->SetNodeA(nodeC);
        else if (w->GetNodeB().lock() == nodeA || w->GetNodeB().lock() == nodeB) w->SetNodeB(nodeC);
    }
    nodeA->mContracted = true;
    nodeB->mContracted = true;
    for (auto &w : connected) w->SetIsContracted(true);

    mNumFloatOps += (long long) 1 << (2 * (indicesC.size() + pairs.size()));
    const bool rank0 = indicesC.empty();
    const bool finishes = rank0 && mUncontractedNodes.size() == 2;
    StepRecord rec;
    rec.a = nodeA->mTensorId;
    rec.b = nodeB->mTensorId;
    rec.c = nodeC->mTensorId;
    rec.idA = nodeA->mID;
    rec.idB = nodeB->mID;
    rec.rankA = nodeA->mRank;
    rec.rankB = nodeB->mRank;
    rec.freeIdx = indicesC;
    rec.sumIdx = pairs;
    rec.done = finishes;
    mSteps.push_back(rec);

    if (mCtx) {
        // the arithmetic: one pairwise contraction on the device
        std::vector<uint8_t> ffa(indicesC.size());
        std::vector<int32_t> fi(indicesC.size()), sa(pairs.size()), sb(pairs.size());
        for (size_t i = 0; i < indicesC.size(); i++) {
            ffa[i] = indicesC[i].first ? 1 : 0;
            fi[i] = indicesC[i].second;
        }
        for (size_t j = 0; j < pairs.size(); j++) {
            sa[j] = pairs[j].first;
            sb[j] = pairs[j].second;
        }
        qt_tensor *ta = nodeA->DeviceTensor(mCtx);
        qt_tensor *tb = nodeB->DeviceTensor(mCtx);
        qt_tensor *tc = nullptr;
        qt_status s = qt_contract_pair(mCtx, ta, tb, (int) ffa.size(), ffa.data(), fi.data(), (int) sa.size(),
                                       sa.data(), sb.data(), &tc);
        if (s != QT_OK) {
            if (s == QT_ERR_INVALID_FUNCTION_INPUT) throw InvalidFunctionInput();
            throw EngineFailure(s);
        }
        nodeC->AdoptDeviceTensor(mCtx, tc);
        if (rank0) {
            // final-value rule (Network.h:961-969)
            const std::complex<double> v = nodeC->GetTensorVals()[0];
            if ((std::abs(mFinalVal.real()) <= 1.0e-30 && std::abs(mFinalVal.imag()) <= 1.0e-30) ||
                (nodeA->mRank == 0 && nodeB->mRank == 0))
                mFinalVal = v;
        }
    } else {
        nodeC->ClearNodeData();   // symbolic: no values
    }
    if (rank0 && mUncontractedNodes.size() == 2) mDone = true;

    if (mDone) {
        auto t = std::make_shared<Node>(0);
        t->mID = (int) mAllNodes.size();
        t->mCreatedFrom = {nodeA->mID, nodeB->mID};
        mAllNodes.push_back(t);
        FindAndRemove(mUncontractedNodes, nodeA);
        FindAndReplace(mUncontractedNodes, nodeB, nodeC);
        nodeA->ClearNodeData();
        nodeB->ClearNodeData();
        return nullptr;
    }
    nodeC->mID = (int) mAllNodes.size();
    nodeC->mCreatedFrom = {nodeA->mID, nodeB->mID};
    mAllNodes.push_back(nodeC);
    nodeA->ClearNodeData();
    nodeB->ClearNodeData();
    FindAndRemove(mUncontractedNodes, nodeA);
    FindAndReplace(mUncontractedNodes, nodeB, nodeC);
    return nodeC;
}

}  // namespace qtorch
