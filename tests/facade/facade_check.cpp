// facade_check.cpp -- drives the C++ facades (include/ekgsim.hpp, include/ekgsim_amsdemo.hpp) the
// way the reference's callers would, in a working directory holding simulator.ini and its files,
// and prints what each returns, one line per result, for tests/test_gpu_facades.py to compare:
//   single i c0 c1 ... viol done     ekgsim::Evaluation::operator() + simulationDone()
//   batch i c0 c1 ... viol           Evaluation::evaluateBatch (one device pass)
//   plugin i c0 c1 ... viol          GpuOptimizationFunction through a VirtualOptimizationFunction&
//   queue i c0 c1 ... viol           GenerationQueue driving a master with AMS-DEMO's job interface
//   ecg i d                          EkgSim (loadFromIni, setAps, setMeasuringPoints, run,
//                                    getMeasurement): max |difference| to ekg_eval's ECG
// Chromosomes are read from genes.txt (one per line, comma separated).
// With EKGSIM_WITH_AMSDEMO the real AMS-DEMO header supplies VirtualOptimizationFunction; the
// compile-only test uses that to check the plugin against the reference's own declaration.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#ifdef EKGSIM_WITH_AMSDEMO
#include "GeneralOptimizationAlgorithm.h"
#else
// AMS-DEMO's in-process evaluation interface, declared here with the same members
// (AMS-DEMO/GeneralOptimizationAlgorithm.h:83-93) so that the check builds without AMS-DEMO.
struct VirtualOptimizationFunction {
    typedef std::vector<double> Value;
    typedef std::vector<double> Input;
    typedef std::vector<double> Properties;
    bool geneBounds;
    VirtualOptimizationFunction() : geneBounds(true) {}
    virtual ~VirtualOptimizationFunction() {}
    virtual void operator()(const Input &solution, Value &result, double &violation, Properties &properties) const = 0;
    virtual void normalize(Input &) const {}
};
#endif

#include "ekgsim.hpp"
#include "ekgsim_amsdemo.hpp"

namespace {
void print(const char *tag, size_t i, const std::vector<double> &c, double v, int done = -1) {
    std::printf("%s %zu", tag, i);
    for (double x : c) std::printf(" %.17g", x);
    std::printf(" %.17g", v);
    if (done >= 0) std::printf(" %d", done);
    std::printf("\n");
}

// A master with AMS-DEMO's job interface over a fixed list of chromosomes.
struct Individual {
    std::vector<double> chromosome, criteria;
    double violation = 0;
};
struct ListMaster {
    std::vector<std::vector<double>> jobs;
    size_t generated = 0;
    std::map<int, size_t> index_of_id;
    std::map<size_t, Individual> results;
    int moreJobs(int preferred) {
        const size_t left = jobs.size() - generated;
        return (int)std::min<size_t>(left, (size_t)preferred);
    }
    std::vector<double> generateJob(int id) {
        index_of_id[id] = generated;
        return jobs[generated++];
    }
    bool newResult(Individual &out, int id, int, double, double) {
        results[index_of_id.at(id)] = out;
        return false;
    }
};
}  // namespace

int main() {
    try {
        std::vector<std::vector<double>> genes;
        std::ifstream in("genes.txt");
        for (std::string line; std::getline(in, line);) {
            if (line.empty()) continue;
            std::vector<double> g;
            std::stringstream ss(line);
            for (std::string tok; std::getline(ss, tok, ',');) g.push_back(std::stod(tok));
            genes.push_back(g);
        }
        ekgsim::Engine engine(0);
        ekgsim::Evaluation ev(engine, "simulator.ini", ".");
        for (size_t i = 0; i < genes.size(); ++i) {
            std::vector<double> r, p;
            double v = 0;
            ev(genes[i], r, v, p);
            print("single", i, r, v, ev.simulationDone() ? 1 : 0);
        }
        std::vector<std::vector<double>> rs;
        std::vector<double> vs;
        ev.evaluateBatch(genes, rs, vs);
        for (size_t i = 0; i < genes.size(); ++i) print("batch", i, rs[i], vs[i]);
        {
            ekgsim::GpuOptimizationFunction<VirtualOptimizationFunction> plugin(0, "simulator.ini", ".");
            const VirtualOptimizationFunction &f = plugin;
            for (size_t i = 0; i < genes.size(); ++i) {
                std::vector<double> r, p, g = genes[i];
                double v = 0;
                f.normalize(g);
                f(g, r, v, p);
                print("plugin", i, r, v);
            }
        }
        {
            ListMaster master;
            master.jobs = genes;
            ekgsim::GenerationQueue<ListMaster, Individual> q(master, ev, 2);
            const size_t n = q.run();
            if (n != genes.size()) throw std::runtime_error("queue evaluated a different number of jobs");
            for (size_t i = 0; i < n; ++i) print("queue", i, master.results.at(i).criteria, master.results.at(i).violation);
        }
        {
            ekgsim::EkgSim sim(engine);
            sim.loadFromIni("simulator.ini");
            ekg_heart_info info{};
            ekgsim::check(ekg_heart_get_info(ev.heart(), &info));
            for (size_t i = 0; i < genes.size(); ++i) {
                std::vector<double> lk((size_t)info.n_layers * 9), leads((size_t)info.n_leads * 3),
                    ecg((size_t)info.n_leads * info.steps), crit(64);
                double v = 0;
                ekgsim::check(ekg_eval(ev.heart(), genes[i].data(), (int32_t)genes[i].size(), crit.data(), &v,
                                       ecg.data(), lk.data(), leads.data()));
                std::vector<std::vector<double>> aps;
                for (int L = 0; L < info.n_layers; ++L) aps.emplace_back(lk.begin() + 9 * L, lk.begin() + 9 * L + 9);
                sim.setAps(aps);
                sim.setMeasuringPoints(leads);
                sim.run();
                double d = 0, m = 0;
                for (size_t l = 0; l < sim.numMeasurements(); ++l) {
                    const std::vector<double> e = sim.getMeasurement(l);
                    for (size_t t = 0; t < e.size(); ++t) {
                        d = std::max(d, std::fabs(e[t] - ecg[l * info.steps + t]));
                        m = std::max(m, std::fabs(ecg[l * info.steps + t]));
                    }
                }
                std::printf("ecg %zu %.17g %.17g\n", i, d, m);
            }
        }
    } catch (const std::exception &e) {
        std::printf("error %s\n", e.what());
        return 1;
    }
    return 0;
}
