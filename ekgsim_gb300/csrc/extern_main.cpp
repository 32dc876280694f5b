// ekgsim_extern <dir> -- the evaluation command for AMS-DEMO's ExternalEvaluation.
//
// ExternalEvaluation (AMS-DEMO/ExternalEvaluation.h:85-152) writes <dir>/input.txt (a '#' comment
// line, then one gene per line), runs `<command> <dir>` and reads <dir>/output.txt: the criteria
// whitespace-separated, '#' lines skipped, and "# violation v" setting the violation; a non-zero
// exit status makes it throw.  This program reads simulator.ini from the working directory (as
// ekgSim does), evaluates the genes on the GPU and writes output.txt in that format.  Errors go to
// stderr with exit status 1.
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "ekgsim.h"

int main(int argc, char **argv) {
    if (argc < 2) {
        std::cerr << "usage: ekgsim_extern <dir>\n";
        return 2;
    }
    const std::string dir = argv[1];
    std::vector<double> genes;
    {
        std::ifstream in((dir + "/input.txt").c_str());
        if (!in) {
            std::cerr << "cannot read " << dir << "/input.txt\n";
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
    std::ofstream out((dir + "/output.txt").c_str());
    out << "# file generated by ekgsim_extern\n";
    out << std::setprecision(17);
    for (int i = 0; i < nc; ++i) out << crit[i] << "\n";
    out << "# violation " << viol << "\n";
    ekg_heart_destroy(heart);
    ekg_engine_destroy(eng);
    return out ? 0 : 1;
}
