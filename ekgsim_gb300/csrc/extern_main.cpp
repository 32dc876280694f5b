// ekgsim_extern [--in NAME] [--out NAME] [dir] -- the evaluation command for AMS-DEMO's
// ExternalEvaluation.
//
// ExternalEvaluation (AMS-DEMO/ExternalEvaluation.h:85-152) writes <dir>/input.txt (a '#' comment
// line, then one gene per line), runs `<command> <dir>` and reads <dir>/output.txt: the criteria
// whitespace-separated, '#' lines skipped, and "# violation v" setting the violation; a non-zero
// exit status makes it throw.  This program reads simulator.ini from the working directory (as
// ekgSim does), evaluates the genes on the GPU and writes output.txt in that format.  Errors go to
// stderr with exit status 1.  ExternalEvaluation appends the directory (process<rank> under MPI,
// nothing in the sequential build, GeneralOptimizationAlgorithm.cpp:262-281), so it defaults to the
// working directory; --in / --out take the "input file name" / "output file name" of the
// [evaluation] section when they are not input.txt / output.txt.
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "ekgsim.h"

int main(int argc, char **argv) {
    std::string dir = ".", in_name = "input.txt", out_name = "output.txt";
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--in" && i + 1 < argc) in_name = argv[++i];
        else if (a == "--out" && i + 1 < argc) out_name = argv[++i];
        else if (!a.empty()) dir = a;
    }
    std::vector<double> genes;
    {
        std::ifstream in((dir + "/" + in_name).c_str());
        if (!in) {
            std::cerr << "cannot read " << dir << "/" << in_name << "\n";
            return 1;
        }
        std::string line;
        while (std::getline(in, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream s(line);
            double v;
            if (s >> v) genes.push_back(v);
        }
    }
    ekg_engine *eng = nullptr;
    ekg_heart *heart = nullptr;
    int rc = ekg_engine_create(0, &eng);
    if (rc == EKG_OK) rc = ekg_heart_from_ini(eng, "simulator.ini", nullptr, &heart);
    int32_t ng = 0, nc = 0;
    if (rc == EKG_OK) rc = ekg_eval_shape(heart, &ng, &nc);
    std::vector<double> crit(nc > 0 ? nc : 1);
    double viol = 0;
    if (rc == EKG_OK) rc = ekg_eval(heart, genes.data(), (int32_t)genes.size(), crit.data(), &viol, nullptr, nullptr,
                                    nullptr);
    if (rc != EKG_OK) {
        std::cerr << "ekgsim_extern: " << ekg_last_error() << "\n";
        return 1;
    }
    std::ofstream out((dir + "/" + out_name).c_str());
    out << "# file generated by ekgsim_extern\n";
    out << std::setprecision(17);
    for (int i = 0; i < nc; ++i) out << crit[i] << "\n";
    out << "# violation " << viol << "\n";
    ekg_heart_destroy(heart);
    ekg_engine_destroy(eng);
    return out ? 0 : 1;
}
