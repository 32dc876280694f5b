// ekgsim.hpp -- header-only C++ facade over the C ABI (ekgsim.h), mirroring the reference's
// simulator interfaces so that C++ callers can switch with few edits:
//
//   ekgsim::EkgSim            ~ SimLib::EkgSim (simlib/sim_lib.h:93-287): loadSettings, loadShape,
//                               simExcitationSequence, setAps, run, getMeasurement, ...
//   ekgsim::Evaluation        ~ OptimizationFunction (sim.h:97-123): operator()(solution, result,
//                               violation, properties), getGeneParams, getEvolutionaryParams,
//                               normalize, plus evaluateBatch for a generation at once
//
// Errors are thrown as std::runtime_error with the engine's message, as the reference throws.
// Not thread-safe per object (as the reference); one engine per process and GPU.
#ifndef EKGSIM_HPP_INCLUDED
#define EKGSIM_HPP_INCLUDED

#include <stdexcept>
#include <string>
#include <vector>

#include "ekgsim.h"

namespace ekgsim {

inline void check(int rc) {
    if (rc != EKG_OK) throw std::runtime_error(ekg_last_error());
}

class Engine {
    ekg_engine *e_ = nullptr;

public:
    explicit Engine(int device = 0) { check(ekg_engine_create(device, &e_)); }
    ~Engine() { ekg_engine_destroy(e_); }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    ekg_engine *get() const { return e_; }
};

// One resident heart built from a simulator.ini, evaluated like SimImplementation (sim.cpp:322-1043).
class Evaluation {
    Engine &eng_;
    ekg_heart *h_ = nullptr;
    int32_t genes_ = 0, criteria_ = 0;
    std::vector<double> gmin_, gmax_;

public:
    typedef std::vector<double> Input, Value, Properties;
    Evaluation(Engine &eng, const std::string &ini = "simulator.ini", const std::string &out_dir = ".") : eng_(eng) {
        check(ekg_heart_from_ini(eng.get(), ini.c_str(), out_dir.empty() ? nullptr : out_dir.c_str(), &h_));
        check(ekg_eval_shape(h_, &genes_, &criteria_));
        gmin_.resize(genes_);
        gmax_.resize(genes_);
        check(ekg_eval_gene_bounds(h_, gmin_.data(), gmax_.data()));
    }
    ~Evaluation() { ekg_heart_destroy(h_); }
    Evaluation(const Evaluation &) = delete;
    Evaluation &operator=(const Evaluation &) = delete;

    // OptimizationFunction::operator() (sim.cpp:1101-1106)
    void operator()(const Input &solution, Value &result, double &violation, Properties &) const {
        result.resize(criteria_);
        check(ekg_eval(h_, solution.data(), (int32_t)solution.size(), result.data(), &violation, nullptr, nullptr,
                       nullptr));
    }
    // a whole generation in one device pass (the batched form)
    void evaluateBatch(const std::vector<Input> &solutions, std::vector<Value> &results,
                       std::vector<double> &violations) const {
        const int32_t n = (int32_t)solutions.size();
        std::vector<double> g((size_t)n * genes_), c((size_t)n * criteria_);
        violations.resize(n);
        for (int32_t i = 0; i < n; ++i) {
            // the reference's messages for too few and for a wrong number of genes (sim.cpp:458-459, :835-841)
            if ((int32_t)solutions[i].size() < genes_) throw std::runtime_error("Solution does not contain enough values");
            if ((int32_t)solutions[i].size() != genes_)
                throw std::runtime_error("chromosome size does not agree with the combination of the number of free "
                                         "Wohlfart parameters and the selected interpolation procedure");
            std::copy(solutions[i].begin(), solutions[i].end(), g.begin() + (size_t)i * genes_);
        }
        check(ekg_eval_batch(h_, n, g.data(), genes_, c.data(), violations.data(), nullptr));
        results.assign(n, Value(criteria_));
        for (int32_t i = 0; i < n; ++i)
            std::copy(c.begin() + (size_t)i * criteria_, c.begin() + (size_t)(i + 1) * criteria_, results[i].begin());
    }
    // a generation queued while the previous one runs (ekg_eval_batch_submit / _wait): the
    // outputs must stay allocated until waitBatch returns
    int64_t submitBatch(const std::vector<double> &genes_flat, int32_t n, double *criteria, double *violations,
                        double *ecg = nullptr) const {
        if ((int64_t)genes_flat.size() != (int64_t)n * genes_)
            throw std::runtime_error("genes_flat must hold n chromosomes of the heart's gene count");
        int64_t t = 0;
        check(ekg_eval_batch_submit(h_, n, genes_flat.data(), genes_, criteria, violations, ecg, &t));
        return t;
    }
    void waitBatch(int64_t ticket) const { check(ekg_eval_batch_wait(h_, ticket)); }
    // whether the last operator() ran its simulation (false when the fast-approximation gate skipped
    // it: SimImplementation::simulationDone, sim.cpp:712-748)
    bool simulationDone() const {
        int32_t v = 1;
        check(ekg_eval_simulated(h_, &v));
        return v != 0;
    }
    // getGeneParams (sim.cpp:523-580)
    void getGeneParams(size_t &numGenes, size_t &numCriteria, std::vector<double> &gMin, std::vector<double> &gMax) const {
        numGenes = genes_;
        numCriteria = criteria_;
        gMin = gmin_;
        gMax = gmax_;
    }
    // OptimizationFunction::normalize (sim.cpp:1123-1128)
    void normalize(Input &solution) const {
        for (size_t i = 0; i < gmin_.size() && i < solution.size(); ++i)
            if (solution[i] < gmin_[i]) solution[i] = gmin_[i];
        for (size_t i = 0; i < gmax_.size() && i < solution.size(); ++i)
            if (solution[i] > gmax_[i]) solution[i] = gmax_[i];
    }
    ekg_heart *heart() const { return h_; }
};

// SimLib::EkgSim-style use: load a heart, set layer APs, run, read measurements.
class EkgSim {
    Engine &eng_;
    ekg_heart *h_ = nullptr;
    ekg_heart_info info_{};
    std::vector<double> aps_, leads_, out_;

public:
    explicit EkgSim(Engine &eng) : eng_(eng) {}
    ~EkgSim() { ekg_heart_destroy(h_); }
    EkgSim(const EkgSim &) = delete;
    EkgSim &operator=(const EkgSim &) = delete;

    // loadSettings + loadTransferMatrix + loadMeasuringPoints + loadShape + simExcitationSequence
    // + applySettings in one step (simlib/sim_lib.h:111-229)
    void loadFromIni(const std::string &ini = "simulator.ini") {
        check(ekg_heart_from_ini(eng_.get(), ini.c_str(), nullptr, &h_));
        check(ekg_heart_get_info(h_, &info_));
    }
    // explicit model (layers [z][y][x], conduction matrix, leads (z,y,x)) as EkgSim's loaders would read
    void load(const ekg_heart_desc &desc) {
        check(ekg_heart_create(eng_.get(), &desc, &h_));
        check(ekg_heart_get_info(h_, &info_));
    }
    size_t requiredAps() const { return (size_t)info_.n_layers; }
    // setApsDestructive: one WohlfartPlus k vector (9 values) per layer
    void setAps(const std::vector<std::vector<double>> &layer_k) {
        aps_.clear();
        for (const auto &k : layer_k) aps_.insert(aps_.end(), k.begin(), k.end());
    }
    // moveMeasuringPoints result (z,y,x per lead); empty = loaded positions
    void setMeasuringPoints(const std::vector<double> &zyx) { leads_ = zyx; }
    void run() {
        if (aps_.size() != (size_t)info_.n_layers * 9) throw std::runtime_error("need one AP per layer");
        out_.assign((size_t)info_.n_leads * info_.steps, 0.0);
        check(ekg_simulate(h_, aps_.data(), leads_.empty() ? nullptr : leads_.data(), out_.data()));
    }
    size_t numMeasurements() const { return (size_t)info_.n_leads; }
    std::vector<double> getMeasurement(size_t n) const {
        return std::vector<double>(out_.begin() + n * info_.steps, out_.begin() + (n + 1) * info_.steps);
    }
    std::vector<double> activationTimes() const {
        std::vector<double> at((size_t)info_.n_cells);
        check(ekg_heart_activation(h_, at.data()));
        return at;
    }
    ekg_heart *heart() const { return h_; }
};

}  // namespace ekgsim

#endif  // EKGSIM_HPP_INCLUDED
