// A C++ program written against include/qtorch/qtorch.hpp the way a qTorch
// user writes against src/qtorch.hpp: files in, ContractionTools /
// LineGraph / Network out.  It links libqtorch_gb300.so and nothing else, and
// every contraction runs on the GPU.  For each case (qasm file, measurement
// file, recorded sequence file) it prints one line:
//   <case> <given-sequence re im> <seeded stochastic re im> <line-graph re im> <flops>
// and, for a missing file, the what() of the exception the reference throws.
#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "qtorch/qtorch.hpp"

static std::vector<std::pair<int, int>> read_sequence(const std::string &path) {
    std::vector<std::pair<int, int>> seq;
    std::ifstream f(path);
    int a, b;
    while (f >> a >> b) seq.push_back({a, b});
    return seq;
}

int main(int argc, char **argv) {
    if (argc >= 2 && std::string(argv[1]) == "missing") {
        try {
            qtorch::ContractionTools t("no/such/file.qasm", "no/such/measure.txt");
            t.Contract(qtorch::Stochastic);
            std::printf("no exception\n");
        } catch (const std::exception &e) {
            std::printf("exception %s\n", e.what());
        }
        return 0;
    }
    for (int i = 1; i + 2 < argc; i += 3) {
        const std::string qasm = argv[i], meas = argv[i + 1];
        // ContractGivenSequence (src/ContractionTools.h:392-411)
        qtorch::ContractionTools given(qasm, meas);
        auto net = given.ContractGivenSequence(read_sequence(argv[i + 2]));
        const std::complex<double> v1 = given.GetFinalVal();
        // the stochastic ordering, seeded (the reference draws from random_device)
        qtorch::ContractionTools stoch(qasm, meas);
        stoch.Seed(7);
        stoch.Contract(qtorch::Stochastic);
        const std::complex<double> v2 = stoch.GetFinalVal();
        // LineGraph::LGContract (src/LineGraph.h:357-376)
        auto lgnet = std::make_shared<qtorch::Network>(qasm, meas);
        qtorch::LineGraph lg(lgnet);
        lg.LGContract();
        const std::complex<double> v3 = lgnet->GetFinalValue();
        std::printf("case %d %.17g %.17g %.17g %.17g %.17g %.17g %lld\n", (i - 1) / 3, v1.real(), v1.imag(), v2.real(),
                    v2.imag(), v3.real(), v3.imag(), net->getNumFloatOps());
    }
    return 0;
}
