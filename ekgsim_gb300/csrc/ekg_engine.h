// Engine and heart objects behind the C ABI.
#pragma once

#include <functional>

#include "ekg_internal.h"
#include "host_model.h"

enum { EKG_CONTRACT_BAND = 0, EKG_CONTRACT_DENSE_UMMA = 1, EKG_CONTRACT_DENSE_CUDA = 2 };

struct ekg_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    int chunk_len = 512;  // APs per K chunk of the contraction (multiple of 64)
    // per-simulation contraction: band form (default), dense on the tensor cores (EKG_CONTRACT=umma)
    // or dense on the CUDA cores (EKG_CONTRACT=cuda)
    int contract = 0;
    bool batched = true;  // separable batched form for multi-simulation passes (EKG_BATCHED=0 disables)
    int batch_ctas = 0;   // target CTAs of the moved-lead GEMM (0 = one wave)
    bool graphs = true;   // replay repeated passes as CUDA graphs (EKG_GRAPHS=0 disables)
    // rounds after which the activation-time relaxation gives up with EKG_ERR_CA_NOT_CONVERGED
    // (0 = the default bound from the grid size; EKG_CA_ROUND_CAP sets it, e.g. to test that error)
    int ca_round_cap = 0;
    // activation-time relaxation: 0 = by time buckets where the lags allow it (else tile rounds),
    // 1 = tile rounds always (EKG_CA=tiles)
    int ca_mode = 0;
    // autotuning of the batched form's launch shapes: EKG_TUNE=1 tunes every new pass shape on its
    // first pass (ekg_heart_tune does it on request); EKG_TUNE_CACHE names a file that keeps the
    // choices across processes
    bool tune = false;
    std::string tune_cache;
};

namespace ekg {
struct EvalSettings {
    GeneModel gm;
    bool optimize_points = false, peak = false, fast_is_crit = false;
    int criteria_mode = 1, comparison_mode = 2;
    double fast_delay = 0, fast_limit = 2, endo_epi_delay = -1;
    std::vector<std::vector<double>> targets;
    std::vector<double> target_offsets;
    std::vector<int> target_peak;
    std::vector<double> disp_min_v, disp_max_v;
    int n_crit_leads = 0, n_criteria = 0, n_genes = 0;
};
}  // namespace ekg

namespace ekg {
// Per-heart state of the batched form: the static-lead Taylor basis (cached per set of per-layer
// k1, k4) and per-batch buffers.
struct BatchState {
    bool basis_ok = false;
    std::vector<double> key;               // k1, k4 per layer the basis was built for
    std::vector<double> single_key;        // k1, k4 of the last single-simulation pass
    int J = 0;                             // Taylor terms stored
    std::vector<double> centre, scale;     // per layer
    DBuf<float> Q1, Q2;                    // [nl][L*J][steps]
    DBuf<double> d_centre, d_scale;
    DBuf<int32_t> lc0, lc1;                // chunk range of each layer
    // band structure of the moved-lead GEMM for the same key, per layer L and 128-step tile j
    int ntt = 0;                           // tiles
    int max_ent = 1;                       // steady entries per layer (max)
    std::vector<int32_t> band_s0, band_s1; // [nl][ntt] band in 32-AP stages [s0, s1)
    DBuf<int32_t> ls0, ls1;                // [nl] 32-AP stage range of each layer
    DBuf<int32_t> nent, esplit;            // [nl], [nl][8]: entries, steady prefix ends (stages)
    DBuf<float2> tref;                     // [stages] last finite activation time of the stage (hi, lo)
    DBuf<int64_t> goff;                    // [nl][8] offsets into gtab
    DBuf<float> gtab;                      // exp(-k4 (t0_e - tref[st])) for the steady stages of entry e
    DBuf<int32_t> ent;                     // [nl][ntt] entry of each tile (-1: layer without APs)
    DBuf<float> E;                         // [nl][steps] exp(-k4 (t - t0 of the tile's entry))
    // per batch
    DBuf<uint8_t> Bt;                      // tiled BF16 hi/lo moved-lead weights
    DBuf<float2> P1;                       // [stages][rows] steady sums per 32-AP stage
    DBuf<int> work;                        // work counter of the operand kernel
    DBuf<float2> U, Up;                    // [rows][nl][max_ent] steady sums (U0, U1), per K part
    DBuf<float> partial;                   // [items][rows][128] raw accumulators (x2 with two bases)
    // resting-potential term (k0 differing between layers): per-part unscaled field sums of the
    // moved rows, the per-row and per-(simulation, static lead) constants, and per heart the
    // layer sums of the resident lead field (K0s, valid while the band tables are)
    DBuf<float> P2;                        // [stages * 4][rows_used]
    DBuf<double> cmov, cst;                // [rows_used], [S][L]
    DBuf<double> K0s;                      // [nl][L]
    bool k0s_ok = false;
};
// Launch shape of the batched form's moved-lead kernels, chosen by the autotuner (0 / -1 = the
// built-in choice): the band GEMM's row tile (32, 128 or 256 rows of (simulation, moved lead)),
// its work-item target in CTAs per SM, and the operand kernel's form (1: one thread per (AP,
// simulation); 0: the persistent kernel with four rows per thread).
struct TuneChoice {
    int tile_rows = 0, cta_mult = 0, op_small = -1;
    int op_bps = 0;       // persistent operand kernel: blocks per SM (0 = as many as fit)
    double ms = 0;        // device time of one pass with this shape (CUDA events)
    int candidates = 0;   // shapes timed when it was chosen
};
// What one device pass does, decided on the host from the batch's layer APs and lead positions.
struct PassPlan {
    bool batch = false;                    // separable batched form
    int n_sims = 0, nmove = 0, J = 0, two_bases = 0;
    int rows_used = 0, rows = 0, ntiles = 0, nitems = 0;
    int tile_rows = 0, op_small = 0, op_bps = 0;  // launch shape (see TuneChoice)
    bool k0 = false;                       // some simulation's k0 differs between layers
    std::vector<double> k3;                // [S][nl]
    std::vector<int4> items;               // band GEMM work items, grouped by tile
    std::vector<int32_t> ti0, ti1;         // [ntt][nl] item range of each (tile, layer)
    std::vector<float> k5l;                // [S][nl]
    std::vector<float4> lrel;              // [S][nmove]
    float4 hc[256];
};
}  // namespace ekg

struct ekg_heart {
    ekg_engine *eng = nullptr;
    cudaStream_t stream = nullptr;    // this heart's device passes run here
    cudaStream_t copy_stream = nullptr;  // early device->host copies overlapping the rest of a pass
    cudaEvent_t static_done = nullptr;   // static-lead ECG rows complete (batched form)
    cudaEvent_t moved_done = nullptr;    // moved-lead ECG rows complete (batched form)
    // the batched form's static-lead combine and steady-sum reduction run on a second stream beside
    // the moved-lead operand kernel and GEMM (fork and join by events; captured into the graphs)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_op = nullptr, ev_join = nullptr;
    uint32_t *err_host = nullptr;     // pinned copy of the kernels' error word
    // device passes captured as CUDA graphs, keyed by everything their launches depend on
    struct PassGraph {
        std::vector<uint64_t> sig;
        cudaGraphExec_t exec = nullptr;
        uint64_t used = 0;
        bool seen_once = false;  // the first pass with a signature runs directly
    };
    PassGraph graphs[4];
    uint64_t graph_clock = 0;
    // the small per-pass inputs, packed into one pinned host buffer and copied with one transfer into
    // one device buffer (both grow only, so the device addresses the graphs hold stay valid); two
    // of them, so that a pass can be prepared while the one before runs
    struct PassInputs {
        const double *layer_k = nullptr, *cpre = nullptr, *leads = nullptr, *k3 = nullptr;
        const float *k5l = nullptr;
        const float4 *hconst = nullptr, *lrel = nullptr;
        const int4 *items = nullptr;
        const int32_t *ti0 = nullptr, *ti1 = nullptr;
    };
    struct Staging {
        uint8_t *host = nullptr;
        ekg::DBuf<uint8_t> dev;
        size_t cap = 0;
        PassInputs in;
    };
    Staging stg[2];
    int cur = 0;  // staging buffer (and pending slot) of the next pass
    const PassInputs &in() const { return stg[cur].in; }
    // batched evaluations in flight (submitted, results not yet handed over), one per staging buffer
    struct Pending {
        bool busy = false;
        int64_t ticket = 0;
        cudaEvent_t done = nullptr;        // the pass and its copies to the host are complete
        uint32_t *err = nullptr;           // pinned error word of the pass
        double *crit2 = nullptr;           // pinned per-lead criterion values and peaks
        size_t crit2_cap = 0;
        int n_sims = 0;
        bool single = false;               // an ekg_eval call (sets simulationDone when handed over)
        std::vector<double> lk_all, leads_all, viol, acrit, endo_epi;
        std::vector<char> done_flags;
        std::vector<std::vector<double>> approx;
        double *criteria = nullptr, *violation = nullptr;  // the caller's outputs
    };
    Pending pend[2];
    int64_t next_ticket = 0;
    cudaEvent_t copies_done = nullptr;  // the last pass's copies to the host are complete
    cudaEvent_t pass_end = nullptr;     // the last pass's work on the heart's stream is complete
    bool copies_pending = false;
    // whether the simulation of the last single evaluation (ekg_eval) ran (false when the
    // fast-approximation gate skipped it: SimImplementation::simulationDone, sim.cpp:743-748)
    bool last_simulated = true;
    ~ekg_heart() {
        for (PassGraph &g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (Staging &g : stg)
            if (g.host) cudaFreeHost(g.host);
        for (Pending &p : pend) {
            if (p.done) cudaEventDestroy(p.done);
            if (p.err) cudaFreeHost(p.err);
            if (p.crit2) cudaFreeHost(p.crit2);
        }
        if (copies_done) cudaEventDestroy(copies_done);
        if (pass_end) cudaEventDestroy(pass_end);
        if (static_done) cudaEventDestroy(static_done);
        if (moved_done) cudaEventDestroy(moved_done);
        for (cudaEvent_t e : {ev_fork, ev_op, ev_join})
            if (e) cudaEventDestroy(e);
        if (aux_stream) cudaStreamDestroy(aux_stream);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
        if (err_host) cudaFreeHost(err_host);
    }
    std::mutex mu;
    int nz = 0, ny = 0, nx = 0, nhood = 0;
    int64_t ncell = 0, nvox = 0, naps = 0;
    double start = 0, length = 0, dt = 1;
    int ca_rounds = 0;
    bool ca_buckets = false;  // the relaxation ran by time buckets (else tile rounds)
    double ca_ms = 0, setup_ms = 0;
    std::vector<double> t;            // time axis
    std::vector<double> leads0;       // loaded lead positions (z,y,x)
    std::vector<double> lead_uv;      // their displacement frames [n][u, v]
    std::vector<double> at_host;      // activation time per cell (copied from the device on first use)
    std::vector<uint8_t> layer_host;  // layer id per cell (stimulus flag stripped)
    std::vector<int64_t> ap_index_ref;    // reference AP numbering per cell (built on demand)
    std::vector<int32_t> vox_cell;        // cell of each voxel, voxels in AP order
    std::vector<int32_t> vox_group_start; // [naps + 1] first voxel of each AP
    ekg::HeartDev dev;
    ekg::EvalDev ev;
    ekg::DBuf<double> at_cells;       // device activation times per cell
    ekg::DBuf<double> leads0_dev;
    ekg::DBuf<float> W0;              // [L][apad] lead field at the loaded positions
    ekg::DBuf<double> W0_layer;       // [nl][L] per-layer sums of W0 (the per-simulation form's k0 term)
    bool W0_layer_ok = false;
    ekg::EvalSettings es;
    ekg::BatchState bs;
    int sm_count = 152;
    bool has_eval = false;
    bool any_k0 = false;              // some layer AP of the current pass has k0 != 0
    bool cpre_on = false;             // the current pass's repolarisation constants come from the host
    ekg::SimConfig cfg;
    // autotuned launch shapes by pass shape (tune_key), and a shape forced while the tuner times it
    std::map<std::string, ekg::TuneChoice> tuned;
    const ekg::TuneChoice *tune_force = nullptr;
    std::vector<ekg::TuneChoice> tune_last;  // every candidate of the last tuning, with its time
};
