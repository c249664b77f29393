// .inp scripts (src/leviParser.hpp:41-104 and the flow of src/main.cpp:42-309):
// ">type name value" lines configure a run that parses a QASM circuit and a
// measurement file, reduces the circuit (ReduceCircuit), contracts it with the
// chosen method and writes the result file.
//   contractmethod  linegraph-qbb | simple-stoch | user-defined
//   qbbonly         write the line-graph elimination order (qbb.out format) and stop
//   readqbbresonly  contract with the order stored in output/qbb.out
// The line-graph order is this build's min-fill order (the reference runs the
// QuickBB binary); it is written in QuickBB's output format so either side can
// replay it.  `>int seed` fixes the stochastic ordering (the reference seeds from
// std::random_device).
#include <sys/stat.h>

#include <chrono>
#include <fstream>
#include <map>
#include <sstream>

#include "../../include/qtorch/qtorch.hpp"
#include "core.h"

namespace {

struct InpVars {
    std::map<std::string, std::string> str;
    std::map<std::string, bool> boolean;
    std::map<std::string, int> integer;
    std::map<std::string, double> dbl;
};

bool read_inp(const std::string &path, InpVars &v) {
    std::ifstream f(path);
    if (!f.is_open()) return false;
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] != '>') continue;
        std::stringstream ss(line);
        std::string type, name, val;
        ss >> type >> name;
        if (type == ">string") {
            ss >> val;
            v.str[name] = val;
        } else if (type == ">bool") {
            ss >> val;
            if (val == "1" || val == "true" || val == "True" || val == "yes" || val == "Yes") v.boolean[name] = true;
            else if (val == "0" || val == "false" || val == "False" || val == "no" || val == "No") v.boolean[name] = false;
        } else if (type == ">int") {
            int i = 0;
            ss >> i;
            v.integer[name] = i;
        } else if (type == ">double") {
            double d = 0;
            ss >> d;
            v.dbl[name] = d;
        }
    }
    return true;
}

std::vector<int> read_qbb_order(const std::string &path, int n_wires) {
    // the line after " The optimal ordering is " holds the 1-based wire order (LineGraph.h:322-333)
    std::ifstream f(path);
    if (!f) throw qtorch::QbbFailure();
    std::string line;
    while (std::getline(f, line)) {
        if (line == " The optimal ordering is ") {
            std::getline(f, line);
            std::stringstream ss(line);
            std::vector<int> order;
            for (int i = 0; i < n_wires; i++) {
                int w;
                if (!(ss >> w)) break;
                order.push_back(w);
            }
            return order;
        }
    }
    throw qtorch::QbbFailure();
}

void write_qbb_order(const std::string &path, const std::vector<int> &order) {
    std::ofstream f(path);
    f << " The optimal ordering is \n";
    for (size_t i = 0; i < order.size(); i++) f << order[i] << (i + 1 < order.size() ? " " : "\n");
}

}  // namespace

extern "C" qt_status qt_run_inp(qt_ctx *ctx, const char *inp_path, double *value, int64_t *flops) {
    if (!inp_path) return QT_ERR_INVALID_ARGUMENT;
    InpVars v;
    // defaults of main.cpp:316-336
    v.integer["quickbbseconds"] = 20;
    v.integer["threads"] = 2;
    v.boolean["qbbonly"] = false;
    v.boolean["readqbbresonly"] = false;
    v.str["outputpath"] = "output/qtorch.out";
    if (!read_inp(inp_path, v)) return qtg::set_error(ctx, QT_ERR_INVALID_FILE, "cannot open the .inp file");
    mkdir("output", 0755);
    std::ofstream out(v.str["outputpath"]);
    if (!out) return qtg::set_error(ctx, QT_ERR_INVALID_FILE, "invalid output file path");
    const auto t0 = std::chrono::steady_clock::now();
    try {
        auto net = std::make_shared<qtorch::Network>(v.str["qasm"], v.str["measurement"], ctx);
        net->ReduceCircuit();
        const std::string method = v.str["contractmethod"];
        if (method == "linegraph-qbb") {
            qtorch::LineGraph lg(net);
            const std::string qbb = "output/qbb.out";
            if (v.boolean["qbbonly"]) {
                write_qbb_order(qbb, lg.MinFillOrdering());
                if (value) value[0] = value[1] = 0.0;
                if (flops) *flops = 0;
                return QT_OK;
            }
            std::vector<int> order;
            if (v.boolean["readqbbresonly"]) {
                order = read_qbb_order(qbb, lg.NumWires());
            } else {
                order = lg.MinFillOrdering();
                write_qbb_order(qbb, order);
            }
            lg.LGContract(order);
        } else if (method == "simple-stoch" || method == "user-defined") {
            qtorch::ContractionTools t(net);
            if (v.integer.count("seed")) t.Seed((uint64_t) v.integer["seed"]);
            if (method == "user-defined" && v.str.count("user-contract-seq"))
                t.ContractUserDefinedSequenceOfWires(v.str["user-contract-seq"]);
            else
                t.Contract(qtorch::Stochastic);
        } else {
            throw qtorch::InvalidContractionMethod();
        }
        const std::complex<double> fv = net->GetFinalValue();
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        out << "Result of Contraction: " << fv << "\n";
        out << "Number of floating point ops in full contraction: " << net->getNumFloatOps() << "\n";
        out << "Contraction complete.  { " << std::to_string(secs) << " } \n";
        if (value) {
            value[0] = fv.real();
            value[1] = fv.imag();
        }
        if (flops) *flops = net->getNumFloatOps();
        return QT_OK;
    } catch (const qtorch::InvalidFile &) {
        out << "Invalid Input or Output File Path\n";
        return qtg::set_error(ctx, QT_ERR_INVALID_FILE, "invalid file");
    } catch (const qtorch::InvalidFileFormat &) {
        out << "Invalid File Format.\n";
        return qtg::set_error(ctx, QT_ERR_INVALID_FILE_FORMAT, "invalid file format");
    } catch (const qtorch::InvalidContractionMethod &) {
        return qtg::set_error(ctx, QT_ERR_INVALID_CONTRACTION_METHOD, "contractmethod: bad option");
    } catch (const qtorch::QbbFailure &) {
        return qtg::set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "cannot read the line-graph order");
    } catch (const qtorch::ContractionFailure &) {
        return qtg::set_error(ctx, QT_ERR_CONTRACTION_FAILURE, "contraction failed");
    } catch (const qtorch::InvalidUserContractionSequence &) {
        return qtg::set_error(ctx, QT_ERR_INVALID_USER_SEQUENCE, "invalid user contraction sequence");
    } catch (const qtorch::EngineFailure &e) {
        return e.status();
    } catch (const std::exception &e) {
        return qtg::set_error(ctx, QT_ERR_INVALID_ARGUMENT, e.what());
    }
}
