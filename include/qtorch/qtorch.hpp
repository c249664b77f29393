// qtorch C++ API on the GB300 engine.
//
// The classes keep the names, members and call semantics of qTorch's public
// API (src/Node.h, src/Wire.h, src/Network.h, src/ContractionTools.h,
// src/LineGraph.h, src/Exceptions.h) so that code written against the
// reference compiles against this header.  What changes is where tensors live:
// a Node's values are a device tensor of the engine; GetTensorVals() brings a
// host copy on demand, and Network::ContractNodes runs the pairwise
// contraction on the GPU through the C ABI (qtorch_gb300.h).
#pragma once

#include <array>
#include <complex>
#include <cstdint>
#include <exception>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../qtorch_gb300.h"

namespace qtorch {

// ---- exceptions (src/Exceptions.h:24-59) --------------------------------
class InvalidFile : public std::exception {
public:
    const char *what() const noexcept override { return "Invalid Input or Output File Path"; }
};
class InvalidFileFormat : public std::exception {
public:
    const char *what() const noexcept override { return "Invalid File Format."; }
};
class InvalidTensorNetwork : public std::exception {
public:
    const char *what() const noexcept override { return "QASM File Does Not Entangle All Qubits"; }
};
class ContractionFailure : public std::exception {
public:
    const char *what() const noexcept override { return "Contraction Failed."; }
};
class InvalidUserContractionSequence : public std::exception {
public:
    const char *what() const noexcept override { return "Invalid User Defined Contraction Sequence."; }
};
class InvalidFunctionInput : public std::exception {
public:
    const char *what() const noexcept override { return "Input to Function Invalid."; }
};
class NumWiresVsNodeRank : public std::exception {
public:
    const char *what() const noexcept override { return "Number of wires different than tensor rank."; }
};
class InvalidContractionMethod : public std::exception {
public:
    const char *what() const noexcept override { return "Invalid Contraction Method."; }
};
class QbbFailure : public std::exception {
public:
    const char *what() const noexcept override { return "Line graph ordering failure."; }
};
// raised when the engine itself fails (CUDA error, out of memory, deadline)
class EngineFailure : public std::exception {
public:
    explicit EngineFailure(qt_status s) : mStatus(s) {}
    const char *what() const noexcept override { return qt_status_string(mStatus); }
    qt_status status() const noexcept { return mStatus; }
private:
    qt_status mStatus;
};

// ---- gate types (src/Node.h:85-105) -------------------------------------
enum class GateType {
    CNOT, SWAP, HADAMARD, RX, RY, RZ, X, Y, Z, PHASE, DEPOLARIZER, CRK, CZ, CPHASE,
    INITSTATE, MEASURETRACE, INTERMEDIATESTATE, ARBITRARYONEQUBITUNITARY, ARBITRARYTWOQUBITUNITARY
};

class Node;

// ---- Wire (src/Wire.h:26-60) ---------------------------------------------
class Wire {
public:
    Wire(std::shared_ptr<Node> nodeA, std::shared_ptr<Node> nodeB, int qubitNum)
        : mNodeA(nodeA), mNodeB(nodeB), mQubitNumber(qubitNum) {}
    void SetNodeA(std::shared_ptr<Node> n) { mNodeA = n; }
    void SetNodeB(std::shared_ptr<Node> n) { mNodeB = n; }
    int GetQubitNumber() const { return mQubitNumber; }
    void SetQubitNumber(int q) { mQubitNumber = q; }
    std::weak_ptr<Node> GetNodeA() const { return mNodeA; }
    std::weak_ptr<Node> GetNodeB() const { return mNodeB; }
    void SetWireID(int id) { mWireID = id; }
    int GetWireID() const { return mWireID; }
    void SetIsContracted(bool c) { mContractedFlag = c; }
    bool IsContracted() const { return mContractedFlag; }
private:
    std::weak_ptr<Node> mNodeA, mNodeB;
    int mWireID{-1};
    int mQubitNumber;
    bool mContractedFlag{false};
};

// ---- Node (src/Node.h:108-194) -------------------------------------------
class Node {
public:
    int mRank;
    int mID{0};
    int mIndexOfPreviousNode{0};
    bool mContracted{false};
    std::pair<int, int> mCreatedFrom{0, 0};
    bool mSelectedInCostContractionAlgorithm{false};

    explicit Node(int rank);
    // a node whose values come later: a contraction's result, adopted from the
    // device, or a node of a symbolic network (no host array of 4^rank values)
    struct NoData {};
    Node(int rank, NoData);
    virtual ~Node();
    Node(const Node &) = delete;
    Node &operator=(const Node &) = delete;

    const std::complex<double> &Access(const std::vector<int> &indexVect);
    const std::complex<double> &Access(const long long &index);
    std::complex<double> &Index(const std::vector<int> &indexVect);
    std::complex<double> &Index(const long long &index);
    const std::vector<int> &GetWireNumber() const { return mWireNumbers; }
    void AddWireNumber(int w) { mWireNumbers.push_back(w); }
    void SetWireNumber(int i, int w) { mWireNumbers[i] = w; }
    GateType GetTypeOfNode() const { return mType; }
    void SetTypeOfNode(GateType t) { mType = t; }
    void SetTypeOfNodeString(const std::string &s) { mStringType = s; }
    const std::string &GetTypeOfNodeString() const { return mStringType; }
    void ClearNodeData();
    std::vector<std::shared_ptr<Wire>> &GetWires() { return mWires; }
    // host copy of the values (downloaded from the device when it holds the data)
    std::vector<std::complex<double>> &GetTensorVals();
    bool HasData() const { return mHostValid || mDevice != nullptr; }

    // ---- engine state
    // device tensor (uploaded lazily from the host values for leaves)
    qt_tensor *DeviceTensor(qt_ctx *ctx);
    void AdoptDeviceTensor(qt_ctx *ctx, qt_tensor *t);
    int64_t mTensorId{-1};     // creation order, used by the planner

protected:
    GateType mType{GateType::INTERMEDIATESTATE};
    std::string mStringType{"INTERMEDIATESTATE"};
    std::vector<std::complex<double>> mVals;
    bool mHostValid{true};
    qt_tensor *mDevice{nullptr};
    qt_ctx *mCtx{nullptr};
private:
    std::vector<std::shared_ptr<Wire>> mWires;
    std::vector<int> mWireNumbers;
};

// gate tensors built on the host with the reference's expressions
std::shared_ptr<Node> MakeGateNode(const std::string &kind, double param);
std::shared_ptr<Node> MakeArbitraryNode(const std::string &path, const std::string &name, bool twoQubit);
// the angle a rotation gate node was built with (0 for other nodes)
double GateAngle(const Node &n);

// ---- one recorded contraction (what the planner lowers) -------------------
struct StepRecord {
    int64_t a, b, c;            // tensor ids (Node::mTensorId)
    int idA, idB;               // mID of the operands (mAllNodes index)
    int rankA, rankB;
    std::vector<std::pair<bool, int>> freeIdx;   // toNotSumOn
    std::vector<std::pair<int, int>> sumIdx;     // toSumOn
    bool done;                  // this step finished the network
};

// ---- Network (src/Network.h:54-140) --------------------------------------
class Network {
public:
    Network();
    // ctx == nullptr builds a symbolic network (ranks and wires only, no device work)
    Network(const std::string &inputFile, const std::string &measureFile, qt_ctx *ctx = DefaultContext());
    static std::shared_ptr<Network> FromText(const std::string &qasm, const std::string &measure,
                                             const std::string &gateDir, qt_ctx *ctx);
    ~Network();

    std::shared_ptr<Node> ContractNodes(std::shared_ptr<Node> nodeA, std::shared_ptr<Node> nodeB, int threshold);
    const std::complex<double> &GetFinalValue() const noexcept { return mFinalVal; }
    void ContractNetworkLinearly();
    const std::vector<std::shared_ptr<Node>> &GetAllNodes() const noexcept { return mAllNodes; }
    void SetNumThreads(int n) noexcept { mNumberOfThreads = n; }
    int GetNumQubits() const noexcept { return mNumberOfQubits; }
    const std::vector<std::shared_ptr<Node>> &GetUncontractedNodes() const noexcept { return mUncontractedNodes; }
    bool IsDone() const noexcept { return mDone; }
    void ReduceCircuit();
    bool HasFailed() const noexcept { return mFailure; }
    void Reset();
    const std::string &GetInputQasm() const noexcept { return mInputFile; }
    void resetFloatCounter() noexcept { mNumFloatOps = 0; }
    long long getNumFloatOps() const noexcept { return mNumFloatOps; }

    // ---- engine additions
    qt_ctx *Context() const { return mCtx; }
    bool IsSymbolic() const { return mCtx == nullptr; }
    const std::vector<StepRecord> &Steps() const { return mSteps; }
    const std::vector<std::shared_ptr<Node>> &Leaves() const { return mLeaves; }
    static qt_ctx *DefaultContext();
    // Index slicing (no reference counterpart): a network whose sliced wires
    // were cut from their leaves replays its recorded sequence, and a pair that
    // shared only cut wires is then an outer product instead of a refusal.
    void AllowOuterProducts(bool allow) noexcept { mAllowOuter = allow; }

private:
    void ParseNetwork(const std::string &qasmText);
    void ParseNode(std::string &line);
    void CreateInitialStates();
    void AddMeasurementsOrTrace(const std::string &measureText);
    void Attach(const std::shared_ptr<Node> &n, const int *qubits, int nq);
    void FindAndRemove(std::vector<std::shared_ptr<Node>> &v, const std::shared_ptr<Node> &x);
    void FindAndReplace(std::vector<std::shared_ptr<Node>> &v, const std::shared_ptr<Node> &x,
                        const std::shared_ptr<Node> &y);
    void FindAndReplace(std::vector<std::vector<std::shared_ptr<Node>>> &v, const std::shared_ptr<Node> &x,
                        const std::shared_ptr<Node> &y);

    std::string mInputFile, mMeasureFile, mQasmText, mMeasureText, mGateDir;
    std::complex<double> mFinalVal{0.0};
    std::mutex mLocker;
    int mNumberOfQubits{0};
    bool mDone{false};
    bool mFailure{false};
    std::vector<std::shared_ptr<Node>> mAllNodes;
    std::vector<std::vector<std::shared_ptr<Node>>> mNodesByWire;
    std::vector<std::shared_ptr<Node>> mUncontractedNodes;
    std::vector<std::shared_ptr<Wire>> mParsingWires;
    std::unordered_map<std::string, std::string> mArbitraryOneQubitGates, mArbitraryTwoQubitGates;
    long long mNumFloatOps{0};
    int mNumberOfThreads{8};
    qt_ctx *mCtx{nullptr};
    std::vector<StepRecord> mSteps;
    std::vector<std::shared_ptr<Node>> mLeaves;
    int64_t mNextTensorId{0};
    bool mAllowOuter{false};
};

// ---- ContractionTools (src/ContractionTools.h:52-123) ----------------------
enum ContractionType { Stochastic, FromEdges, CostContractSimple, CostContractBruteForce };

class ContractionTools {
public:
    explicit ContractionTools(const std::string &inputFile, const std::string &measureFile, int numThreads = 8);
    explicit ContractionTools(std::shared_ptr<Network> network);
    std::complex<double> GetFinalVal() const noexcept { return mFinalVal; }
    // Stochastic is the supported ordering; the cost-based ones are not built
    std::shared_ptr<Network> Contract(ContractionType type, int pValue = 1, int numSamples = 1);
    std::shared_ptr<Network> ContractUserDefinedSequenceOfWires(const std::string &userInputFilePath);
    std::shared_ptr<Network> ContractUserDefinedSequenceText(const std::string &text);
    std::shared_ptr<Network> ContractGivenSequence(const std::vector<std::pair<int, int>> &sequence);
    void Reset(const std::string &inputFile, const std::string &measureFile, int numThreads = 8);
    void Reset();
    void Reset(std::shared_ptr<Network> network) { mNetwork = network; mCopyCreated = true; }
    // the reference seeds from std::random_device; a fixed seed makes the ordering reproducible
    void Seed(uint64_t seed) { mRandGen.seed((std::mt19937::result_type) seed); }
private:
    std::shared_ptr<Network> Acquire();
    std::shared_ptr<Network> ParallelContract(std::mt19937 &gen);
    std::string mString, mMeasureFile;
    std::complex<double> mFinalVal{0.0};
    std::shared_ptr<Network> mNetwork;
    std::mt19937 mRandGen;
    bool mCopyCreated{false};
    int mNumThreadsInNetwork{8};
};

// ---- preProcess (src/preprocess.h:28-52) ----------------------------------
// The reference retries its randomly seeded stochastic ordering up to 100
// times and keeps the first sequence whose contraction finishes under a time
// limit.  This build scores each seeded try by what sets the GPU's time and
// memory -- the rank of its largest intermediate, then its complex MACs --
// over a symbolic copy of the network (no contraction is run) and keeps the
// best of `tries` seeds (seed, seed + 1, ...); with maxMacs > 0 it stops at
// the first try of at most that many MACs, as the reference stops at the
// first fast enough.  The sequence is the mCreatedFrom walk of the reference
// (preprocess.h:41-46), replayable with ContractGivenSequence.
struct PreProcessResult {
    uint64_t seed = 0;
    int tries = 0;          // tries run
    int peakRank = 0;
    long long flops = 0;    // complex MACs (getNumFloatOps)
    std::vector<std::pair<int, int>> sequence;
};
bool preProcess(const std::string &qasmText, const std::string &measureText, const std::string &gateDir,
                uint64_t seed, int tries, long long maxMacs, PreProcessResult &best);

// ---- Size-greedy ordering (no reference counterpart) ------------------------
// For networks too large for the line graph's min-fill walk (circuits of
// 20-30 qubits and depth 8-20 make line graphs of 10^3-10^4 wires): pairs of
// nodes that share a wire are merged in order of the size change the merge
// causes, 4^rank(C) - 4^rank(A) - 4^rank(B), so merges that shrink the network
// (a trace into the gate before it, a one-qubit gate into its neighbour) come
// first and growth is postponed.  Try 0 is deterministic; tries 1.. add seeded
// noise to the scores; the try with the smallest largest intermediate, then the
// fewest MACs, is kept and replayed on `net` with ContractNodes.  Leftover
// rank-0 nodes of unconnected groups are multiplied in list order, as
// LGContract does.
struct GreedyResult {
    int peakRank = 0;
    double macs = 0;        // complex MACs
    int height = 0;         // height of the contraction tree
    int tries = 0;
};
GreedyResult GreedyContract(Network &net, uint64_t seed, int tries);
// The planner's default for requests of any size: the greedy walk, and for line
// graphs of at most maxMinFillWires wires also the min-fill walk, the better by
// largest intermediate and estimated GPU time.
GreedyResult AutoContract(std::shared_ptr<Network> net, uint64_t seed, int tries, int maxMinFillWires);

// ---- LineGraph (src/LineGraph.h:28-85) -------------------------------------
// The reference asks the closed QuickBB binary for an elimination order; this
// build computes a min-fill elimination order of the line graph itself.
class LineGraph {
public:
    explicit LineGraph(std::shared_ptr<Network> network);
    void Reset(std::shared_ptr<Network> network = nullptr);
    // 1-based wire elimination order (the content of qbb.out's ordering line)
    const std::vector<int> &MinFillOrdering();
    bool LGContract();                                   // uses MinFillOrdering()
    bool LGContract(const std::vector<int> &order1Based); // replays a given order
    int NumWires() const { return (int) mGraphWires.size(); }
    const std::vector<std::array<int, 2>> &Edges() const { return mEdges; }
private:
    void Build();
    std::shared_ptr<Network> mNetwork;
    std::vector<std::shared_ptr<Wire>> mGraphWires;
    std::vector<std::array<int, 2>> mEdges;
    std::vector<int> mOrder;
};

}  // namespace qtorch
