// ekgsim_amsdemo.hpp -- bindings of the GPU engine to AMS-DEMO's two evaluation paths, header-only
// over ekgsim.hpp, with no dependency on AMS-DEMO's own headers (its types enter as template
// parameters, so this header compiles with or without them):
//
//   ekgsim::GpuOptimizationFunction<Base>
//       the in-process plugin: a subclass of AMS-DEMO's VirtualOptimizationFunction
//       (AMS-DEMO/GeneralOptimizationAlgorithm.h:83-93) evaluating on the GPU, for the
//       `internalFunction` slot that the reference fills with OptimizationFunction (sim.h:97-123).
//
//   ekgsim::GenerationQueue<Controller>
//       the job queue: drives a master that offers jobs the way ParallelNumericOptimizer offers them
//       to PFramework (moreJobs / generateJob / newResult, AMS-DEMO/ParallelNumericOptimizer.h:509-599,
//       called from PFramework::execute, AMS-DEMO/ParallelFramework.h:286) and evaluates the jobs a
//       batch at a time on the device instead of shipping one chromosome per MPI message.  Each job
//       is normalised and evaluated as EvaluationJob does (ParallelNumericOptimizer.h:361-379); the
//       next batch is generated and queued while the current one runs on the device (two batches
//       in flight, as PFramework keeps worker queues filled ahead of the results).
#ifndef EKGSIM_AMSDEMO_HPP_INCLUDED
#define EKGSIM_AMSDEMO_HPP_INCLUDED

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "ekgsim.hpp"

namespace ekgsim {

// Base: AMS-DEMO's VirtualOptimizationFunction (or a type with the same virtual members).
template <class Base>
struct GpuOptimizationFunction : public Base {
    typedef typename Base::Input Input;
    typedef typename Base::Value Value;
    typedef typename Base::Properties Properties;
    Engine engine;     // one per process (MPI rank) and GPU
    Evaluation eval;   // reads simulator.ini as SimImplementation's constructor does (sim.cpp:362-431)

    explicit GpuOptimizationFunction(int device = 0, const std::string &ini = "simulator.ini",
                                     const std::string &out_dir = ".")
        : engine(device), eval(engine, ini, out_dir) {
        this->geneBounds = false;  // the engine's getGeneParams bounds are reported instead
    }
    void operator()(const Input &solution, Value &result, double &violation, Properties &properties) const override {
        eval(solution, result, violation, properties);
    }
    void normalize(Input &solution) const override { eval.normalize(solution); }
    // OptimizationFunction::getGeneParams (sim.cpp:1109-1116)
    void getGeneParams(size_t &numGenes, size_t &numCriteria, std::vector<double> &gMin,
                       std::vector<double> &gMax) const {
        eval.getGeneParams(numGenes, numCriteria, gMin, gMax);
    }
};

// Controller: the master's job interface, as ParallelNumericOptimizer offers it --
//   int moreJobs(int preferred)          jobs the master wants created now (< 0: finished)
//   Input generateJob(int id)            the chromosome of job `id`
//   bool newResult(Individual &out, int id, int rank, double evolTime, double lifeTime)
// Individual: a type with chromosome, criteria and violation members (AMS-DEMO's IndividualStruc).
template <class Controller, class Individual>
class GenerationQueue {
    Controller &ctl_;
    const Evaluation &eval_;
    int batch_;
    int next_id_ = 0;
    struct Batch {
        std::vector<int> ids;
        std::vector<std::vector<double>> chromosomes;
        std::vector<double> genes, criteria, violations;
        int64_t ticket = 0;
        bool busy = false;
    };
    Batch slots_[2];

    // hands a finished batch's results to the master in job order
    void deliver(Batch &b) {
        if (!b.busy) return;
        b.busy = false;
        eval_.waitBatch(b.ticket);
        size_t ng = 0, nc = 0;
        std::vector<double> lo, hi;
        eval_.getGeneParams(ng, nc, lo, hi);
        for (size_t i = 0; i < b.ids.size(); ++i) {
            Individual out;
            out.chromosome = b.chromosomes[i];
            out.criteria.assign(b.criteria.begin() + i * nc, b.criteria.begin() + (i + 1) * nc);
            out.violation = b.violations[i];
            ctl_.newResult(out, b.ids[i], 0, 0.0, 0.0);
        }
    }

public:
    GenerationQueue(Controller &ctl, const Evaluation &eval, int batch = 256) : ctl_(ctl), eval_(eval), batch_(batch) {
        if (batch_ < 1) throw std::runtime_error("batch size must be positive");
    }
    // Runs until the master wants no more jobs; returns the number of evaluations.
    size_t run() {
        size_t ng = 0, nc = 0, total = 0;
        std::vector<double> lo, hi;
        eval_.getGeneParams(ng, nc, lo, hi);
        int cur = 0;
        for (;;) {
            const int n = ctl_.moreJobs(batch_);
            if (n <= 0) break;
            Batch &b = slots_[cur];
            deliver(b);  // the batch that used this slot two rounds ago
            b.ids.resize(n);
            b.chromosomes.resize(n);
            b.genes.resize((size_t)n * ng);
            b.criteria.resize((size_t)n * nc);
            b.violations.resize(n);
            for (int i = 0; i < n; ++i) {
                b.ids[i] = ++next_id_;
                std::vector<double> c = ctl_.generateJob(b.ids[i]);
                eval_.normalize(c);
                if (c.size() != ng) throw std::runtime_error("Solution does not contain enough values");
                std::copy(c.begin(), c.end(), b.genes.begin() + (size_t)i * ng);
                b.chromosomes[i] = std::move(c);
            }
            b.ticket = eval_.submitBatch(b.genes, n, b.criteria.data(), b.violations.data());
            b.busy = true;
            total += (size_t)n;
            cur ^= 1;
            deliver(slots_[cur]);  // the previous batch, while this one runs
        }
        deliver(slots_[cur ^ 1]);
        deliver(slots_[cur]);
        return total;
    }
};

}  // namespace ekgsim

#endif  // EKGSIM_AMSDEMO_HPP_INCLUDED
