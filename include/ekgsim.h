/*
 * ekgsim.h -- C ABI of the GB300 engine for the EkgSim simulation path.
 *
 * The reference simulator is a C++ class library driven per evaluation (simlib/sim_lib.h:93-287,
 * sim.cpp:322-1129).  This header is the thin boundary between C++ (or any FFI) host code and
 * the CUDA engine: plain pointers, sizes and int status codes, no CUDA or torch types.
 *
 * Conventions
 *   - Every call returns an int status: EKG_OK (0) or a negative EKG_ERR_* code; the message of
 *     the last failure on the calling thread is available from ekg_last_error().
 *   - The caller owns every host buffer; the engine owns all device state.
 *   - Coordinates follow the reference: grids are [z][y][x] with x fastest; lead positions are
 *     (z, y, x) in voxel units from the grid's (0,0,0) corner (the points file holds x, y, z,
 *     simlib/simulator.cpp:374-381).
 *   - One engine per process and GPU.  Calls on one heart are serialised internally; the served
 *     form (ekg_server_*) is safe to call from several host threads.
 */
#ifndef EKGSIM_H_INCLUDED
#define EKGSIM_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define EKG_OK 0
#define EKG_ERR_BAD_INPUT -1        /* invalid argument, size or file content */
#define EKG_ERR_OUT_OF_MEMORY -2    /* device allocation failed or admission refused */
#define EKG_ERR_CA_NOT_CONVERGED -3 /* activation-time relaxation hit its sweep cap */
#define EKG_ERR_DEVICE -4           /* CUDA error (message has the detail) */
#define EKG_ERR_TIMEOUT -5          /* a bounded device wait ran out (kernel error flag set) */
#define EKG_ERR_NO_START -6         /* model has no stimulus voxel (simlib/simulator.cpp:275-278) */
#define EKG_ERR_TRANSFER -7         /* conduction matrix misses a layer (simlib/simulator.cpp:234-238) */
#define EKG_ERR_IO -8               /* file could not be opened or parsed */
#define EKG_ERR_NOT_FOUND -9        /* unknown request id / heart id */
#define EKG_ERR_BUSY -10            /* request not finished yet (poll again) */

/* neighbourhood codes of the [simulation] "neighbourhood type" key (simlib/sim_lib.h:131-147) */
#define EKG_NHOOD_3D4 0  /* 8 body diagonals (simlib/simulator.h:353-360) */
#define EKG_NHOOD_CUBE 1 /* "3D8" / "cube": 26 neighbours (simlib/simulator.h:363-369) */
#define EKG_NHOOD_2D4 2  /* in-plane diagonals (simlib/simulator.h:336-343) */
#define EKG_NHOOD_2D8 3  /* in-plane 8 (simlib/simulator.h:345-351) */

typedef struct ekg_engine ekg_engine;
typedef struct ekg_heart ekg_heart;
typedef struct ekg_server ekg_server;

/* Message of the last failed call on this thread (empty string when none).  Replaces the
 * std::runtime_error messages the reference prints from main (main.cpp:405-413). */
const char *ekg_last_error(void);

/* ------------------------------------------------------------------ engine */
/* Create the engine on CUDA device `device` (streams, event pool, kernel configuration).
 * Replaces nothing in the reference: its process is CPU-only (main.cpp:387). */
int ekg_engine_create(int device, ekg_engine **out);
int ekg_engine_destroy(ekg_engine *e);
/* Free device memory currently usable by the engine (cudaMemGetInfo minus its reserve). */
int ekg_engine_free_bytes(ekg_engine *e, uint64_t *free_bytes);

/* ------------------------------------------------------------------ heart */
typedef struct {
    int32_t nz, ny, nx;
    const int32_t *layers;     /* [nz][ny][nx]: 0 empty, L>0 layer, -L stimulus voxel of layer L */
    int32_t n_transfer;        /* conduction matrix is n_transfer x n_transfer */
    const double *transfer;    /* row-major, ms; T[src][dst] (simlib/simulator.cpp:239) */
    int32_t n_leads;
    const double *leads_zyx;   /* n_leads x 3, as loaded (before any displacement) */
    int32_t nhood;             /* EKG_NHOOD_* for the dipole neighbourhood */
    double start;              /* [simulation] start (ms) */
    double length;             /* [simulation] length (ms) */
    double dt;                 /* [simulation] time step (ms) */
    const double *activation_in; /* NULL: compute the activation times; else [nz][ny][nx] times (ms,
                                  * finite and >= 0 in non-empty cells) used instead, as the
                                  * reference does with "[model] excitation sequence"
                                  * (Simulation::loadExcitationSequence, simlib/simulator.cpp:288-367;
                                  * no stimulus voxel or conduction matrix is needed then) */
} ekg_heart_desc;

typedef struct {
    int64_t n_cells;           /* nz*ny*nx */
    int64_t n_voxels;          /* non-empty voxels */
    int64_t n_aps;             /* unique (layer, activation time) pairs (simlib/simulator.cpp:561-621) */
    int32_t n_layers;          /* highest layer id */
    int32_t n_leads;
    int32_t steps;             /* ceil(length / dt) */
    int32_t ca_rounds;         /* steps of the activation relaxation: time buckets, or tile rounds
                                * where the lags do not allow buckets (a zero lag) */
    int64_t device_bytes;      /* device memory held by this heart */
    double ca_ms;              /* device time of the activation relaxation */
    double setup_ms;           /* host wall time of ekg_heart_create */
    int32_t ca_buckets;        /* 1: the relaxation ran by time buckets, 0: by tile rounds (or loaded) */
} ekg_heart_info;

/* Upload a heart, compute its activation times on the device (bit-exact FP64 equivalent of
 * Simulation::calculateExcitationSequence, simlib/simulator.cpp:212-286), de-duplicate the cell
 * APs (Simulation::setApIndices, simlib/simulator.cpp:561-621) and build the resident lead field.
 * Replaces EkgSim::loadShape + loadTransferMatrix + loadMeasuringPoints + simExcitationSequence
 * + applySettings (simlib/sim_lib.h:131-229). */
int ekg_heart_create(ekg_engine *e, const ekg_heart_desc *desc, ekg_heart **out);
int ekg_heart_destroy(ekg_heart *h);
int ekg_heart_get_info(ekg_heart *h, ekg_heart_info *info);
/* Simulation window of the heart: start, length and time step in ms. */
int ekg_heart_time_axis(ekg_heart *h, double *start, double *length, double *dt);
/* Activation times [nz][ny][nx] (0 = empty or unreachable), the excitationDelay field of the
 * reference's ShapeElement after calculateExcitationSequence (simlib/matrix.h:82-102). */
int ekg_heart_activation(ekg_heart *h, double *at_out);
/* apIndex of every cell [nz][ny][nx] in the reference's numbering (first appearance in raster
 * order, -1 for empty cells; simlib/simulator.cpp:570-590). */
int ekg_heart_ap_index(ekg_heart *h, int64_t *ap_index_out);

/* Plain simulation: layer APs in, ECG out.  Replaces EkgSim::setApsDestructive + run +
 * getMeasurement (simlib/sim_lib.h:152-155, :258-260, :268-270 -> Simulation::run,
 * simlib/simulator.cpp:452-550).
 *   layer_k:   n_layers x 9 WohlfartPlus coefficients (layer 1 first, k8 unshifted)
 *   leads_zyx: n_leads x 3 lead positions for this run, or NULL for the loaded positions
 *   ecg_out:   n_leads x steps doubles (lead-major) */
int ekg_simulate(ekg_heart *h, const double *layer_k, const double *leads_zyx, double *ecg_out);

/* Device timing of the simulation itself, inputs resident in device memory: uploads layer_k
 * (n_sims x n_layers x 9) and leads (n_sims x n_leads x 3, NULL = loaded positions) once, runs
 * `warmup` untimed and `iters` timed device passes, and writes up to n_out values:
 * [0] total ms of the timed passes (back to back, as replayed evaluation passes; CUDA events on
 * the heart's stream), then over `iters` more passes with events between their parts: [1] ms in
 * the lead contraction kernel, [2] ms in lead field / AP factors, [3] ms in reduction + criteria,
 * [4] kernel launches per pass, [5] leads whose lead field is recomputed per pass,
 * [6] 1 when the pass used the separable batched form, 0 for the per-simulation form,
 * batched form with moved leads only (else 0): [7] ms in the moved-lead operand kernel,
 * [8] tensor flops the band GEMM executes per pass, [9] bytes the operand kernel moves per pass;
 * per-simulation form with the band-form contraction (else 0): [10] bytes that contraction has to
 * move per pass (W' read, per-chunk FP64 partial sums written, activation times read).
 * No counterpart in the reference (it has no device); used by the benchmark. */
int ekg_heart_benchmark(ekg_heart *h, int32_t n_sims, const double *layer_k, const double *leads, int32_t warmup,
                        int32_t iters, double *out, int32_t n_out);

/* Autotuner of the batched form's launch shapes (no counterpart in the reference, which has no
 * device).  For a pass of n_sims simulations with these inputs (as ekg_heart_benchmark takes them)
 * it times every candidate shape of the moved-lead kernels -- band GEMM row tile 32 / 128 / 256,
 * GEMM work-item target of 1 / 2 / 4 CTAs per SM, for up to 64 simulations the operand kernel's
 * per-(AP, simulation) or persistent form, and the persistent form's blocks per SM (as many as fit,
 * or 4) -- with CUDA events on the heart's stream
 * (`reps` passes each after one untimed pass), keeps the fastest for every later pass of this
 * shape on this heart, and appends it to the file named by the EKG_TUNE_CACHE environment variable
 * (read at engine creation; engines read it back for the same pass shape).  With EKG_TUNE=1 every
 * new pass shape is tuned on its first batched pass.  out (n_out values at most): [0] row tile,
 * [1] CTAs per SM, [2] operand form (1 per-(AP, simulation), 0 persistent), [3] ms per pass of the
 * choice, [4] ms per pass of the built-in shape, [5] candidates timed (0: the pass has no moved
 * leads or is not in the batched form, so there is nothing to tune), [6] operand blocks per SM
 * (0 = as many as fit); then per candidate five values: row tile, CTAs per SM, operand form,
 * operand blocks per SM, ms per pass.  Results of every shape are within the engine's tolerance of
 * one another (the shapes change FP32 summation order only). */
int ekg_heart_tune(ekg_heart *h, int32_t n_sims, const double *layer_k, const double *leads, int32_t reps,
                   double *out, int32_t n_out);
/* The candidate shapes the tuner times for a pass (host only; no counterpart in the reference): shapes_out receives up to
 * max_shapes quadruples (row tile, CTAs per SM, operand form, operand blocks per SM), *n_out their
 * number. */
int ekg_tune_candidates(int32_t two_bases, int32_t rows_used, int32_t n_sims, int32_t *shapes_out,
                        int32_t max_shapes, int32_t *n_out);
/* The tuner's cache file (host only; no counterpart in the reference): one line per pass shape, "key rows ctas form ms candidates
 * blocks", later lines winning.  _put appends a shape (quadruple as above) for `key` (no spaces);
 * _get reads the last valid one (EKG_ERR_NOT_FOUND when there is none). */
int ekg_tune_cache_put(const char *path, const char *key, const int32_t *shape, double ms);
int ekg_tune_cache_get(const char *path, const char *key, int32_t *shape_out, double *ms_out);

/* ------------------------------------------------------------------ evaluation */
/* Everything SimImplementation reads from simulator.ini beyond the heart itself
 * (SimSettings, SimSettings.h:77-357) plus the loaded targets (sim.cpp:999-1042). */
typedef struct {
    int32_t interpolation;       /* 1 = endo-epi, 2 = endo-mid-epi (sim.cpp:389-396) */
    double mid_position;         /* "mid AP position" */
    int32_t n_base_aps;
    const double *base_aps;      /* n_base_aps x 9 ("base ap N") */
    const double *k_min;         /* 9 */
    const double *k_max;         /* 9 */
    uint32_t free_k_mask;        /* bit i: k_i is a gene ("free k") */
    int32_t optimize_points;     /* "optimize measuring points" */
    int32_t criteria_mode;       /* 1 every lead, 9 leads sum ("mode") */
    int32_t comparison_mode;     /* 1 rms, 2 1-pearson, 3 devFromLinear, 4 1-vector-corr */
    int32_t peak_is_criterion;
    int32_t fast_is_criterion;
    double fast_delay;           /* "fast approximation epi delay" */
    double fast_limit;           /* "fast approximation limit" */
    double endo_epi_delay;       /* "endo-epi minimization criterion epi delay" (<0 off) */
    int32_t n_targets;
    const int64_t *target_len;   /* n_targets */
    const double *targets;       /* concatenated target columns (already scaled/resampled) */
    const double *target_offsets;/* n_targets */
    int32_t n_disp_min;          /* "displacement min" values (bounds of the lead genes) */
    const double *disp_min;
    int32_t n_disp_max;          /* "displacement max" values */
    const double *disp_max;
} ekg_eval_config;

/* Set the evaluation settings of a heart: what SimImplementation's constructor takes from
 * simulator.ini and the target file (sim.cpp:362-431, targets sim.cpp:999-1042).  Evaluations in
 * flight complete with the settings they started with. */
int ekg_heart_set_eval(ekg_heart *h, const ekg_eval_config *cfg);
/* Number of genes and criteria (SimImplementation::getGeneParams, sim.cpp:523-580). */
int ekg_eval_shape(ekg_heart *h, int32_t *n_genes, int32_t *n_criteria);
/* Gene bounds (n_genes each) as getGeneParams reports them (sim.cpp:523-580). */
int ekg_eval_gene_bounds(ekg_heart *h, double *gene_min, double *gene_max);

/* One evaluation: OptimizationFunction::operator() (sim.cpp:1101-1106 -> SimImplementation::eval,
 * sim.cpp:443-492).  criteria_out has n_criteria entries; ecg_out (n_leads x steps) and
 * layer_k_out (n_layers x 9) and leads_out (n_leads x 3, z,y,x) may be NULL. */
int ekg_eval(ekg_heart *h, const double *genes, int32_t n_genes, double *criteria_out,
             double *violation_out, double *ecg_out, double *layer_k_out, double *leads_out);
/* 1 when the last ekg_eval on this heart ran the simulation, 0 when the fast-approximation gate
 * skipped it (SimImplementation::simulationDone, sim.cpp:712-748): its criteria then come from the
 * approximation and the reference writes no ECG rows (ecg_out still receives the simulated ECG). */
int ekg_eval_simulated(ekg_heart *h, int32_t *simulated_out);

/* Batched evaluation of n_sims gene vectors on one resident heart (the reference's MPI farm of
 * independent evaluations, AMS-DEMO/ParallelFramework.h:226-520, folded into one device pass).
 * genes: n_sims x n_genes; criteria_out: n_sims x n_criteria; violation_out: n_sims;
 * ecg_out: n_sims x n_leads x steps or NULL. */
int ekg_eval_batch(ekg_heart *h, int32_t n_sims, const double *genes, int32_t n_genes,
                   double *criteria_out, double *violation_out, double *ecg_out);

/* The same, queued: returns once the host part of the evaluation is done (genes may be reused)
 * and its device pass is queued; *ticket_out identifies it.  The outputs are complete after
 * ekg_eval_batch_wait(ticket).  Two evaluations per heart can be in flight, so a caller can
 * prepare the next batch while the device runs the current one (the reference's master process
 * hands out the next generation's jobs the same way, AMS-DEMO/ParallelFramework.h:226-520); a
 * third submission first completes the oldest.  Copies into pageable output memory block the
 * calling thread; ekg_host_register the output buffers to let the copies run asynchronously. */
int ekg_eval_batch_submit(ekg_heart *h, int32_t n_sims, const double *genes, int32_t n_genes,
                          double *criteria_out, double *violation_out, double *ecg_out, int64_t *ticket_out);
int ekg_eval_batch_wait(ekg_heart *h, int64_t ticket);

/* Page-locks (and releases) caller memory so that device copies into it run asynchronously
 * (cudaHostRegister).  The memory must stay allocated while it is registered. */
int ekg_host_register(void *ptr, int64_t bytes);
int ekg_host_unregister(void *ptr);

/* ------------------------------------------------------------------ served form */
typedef struct {
    int32_t max_batch;           /* most requests packed into one device pass (default 256) */
    int32_t max_wait_us;         /* longest a request waits for others to join while nothing of its
                                  * heart is on the device (default 200) */
    uint64_t hbm_reserve_bytes;  /* free memory kept back from admission (default 2 GiB) */
    int32_t no_ecg;              /* 1: results carry criteria and violation only (no ECG copies to
                                  * the host); polling for an ECG is then an error.  0 (default) keeps them */
} ekg_server_opts;

typedef struct {
    double queue_ms;             /* submit -> start of its device pass */
    double total_ms;             /* submit -> result available */
    int32_t batch_size;          /* requests in its device pass */
} ekg_request_stats;

/* Request loop with continuous batching over resident hearts; replaces the MPI master/worker
 * job queue of AMS-DEMO (AMS-DEMO/ParallelFramework.h:109-520) on one GPU.  Every heart has its
 * own queue and dispatcher: while one pass of a heart runs on the device the next one is prepared
 * and queued behind it, so requests that arrive during a pass join the next; hearts overlap on the
 * device.  A request with the wrong gene count or non-finite genes fails alone (EKG_ERR_BAD_INPUT,
 * the reference's messages of sim.cpp:458-459 and :835-841); a pass that does not fit the free
 * device memory minus the reserve is halved until it does (EKG_ERR_OUT_OF_MEMORY when not even one
 * simulation fits). */
int ekg_server_create(ekg_engine *e, const ekg_server_opts *opts, ekg_server **out);
int ekg_server_destroy(ekg_server *s);
/* Register a heart (with its eval config set); returns its id.  The heart must outlive the server
 * (destroy the server first), and its evaluation settings must not change while it is registered. */
int ekg_server_add_heart(ekg_server *s, ekg_heart *h, int32_t *heart_id);
int ekg_server_submit(ekg_server *s, int32_t heart_id, const double *genes, int32_t n_genes,
                      uint64_t *request_id);
/* Wait up to wait_ms (0 = poll) for a result; EKG_ERR_BUSY if not ready.  ecg_out may be NULL. */
int ekg_server_poll(ekg_server *s, uint64_t request_id, int32_t wait_ms, double *criteria_out,
                    double *violation_out, double *ecg_out, ekg_request_stats *stats);
/* Many requests in one call (as the reference's master hands out a generation of jobs,
 * AMS-DEMO/ParallelNumericOptimizer.h:509-599): heart_ids and request_ids have n entries, genes is
 * n x n_genes. */
int ekg_server_submit_many(ekg_server *s, int32_t n, const int32_t *heart_ids, const double *genes,
                           int32_t n_genes, uint64_t *request_ids);
/* Wait up to wait_ms until all n requests are finished, then hand over the finished ones: per
 * request status_out[i] (EKG_OK, its error code, or EKG_ERR_BUSY when not finished), its criteria at
 * criteria_out + i * crit_stride (at most crit_stride values), violation_out[i] and stats_out[i]
 * (criteria_out, violation_out and stats_out may be NULL).  Returns EKG_ERR_BUSY when some request
 * is not finished, else EKG_OK (each request's own outcome is in status_out). */
int ekg_server_poll_many(ekg_server *s, int32_t n, const uint64_t *request_ids, int32_t wait_ms,
                         int32_t crit_stride, double *criteria_out, double *violation_out,
                         int32_t *status_out, ekg_request_stats *stats_out);

/* Test hook (no counterpart in the reference): replace the free-device-memory query the admission
 * check uses (fn returns free bytes; NULL restores cudaMemGetInfo).  Lets tests refuse admission
 * without filling the GPU. */
int ekg_server_set_free_bytes_provider(ekg_server *s, uint64_t (*fn)(void *ctx), void *ctx);

/* Activation times without any device allocation, for callers that cannot call cudaMalloc (for
 * example code running under a framework's memory pool or a real-time loop that forbids new
 * device allocations after start-up).  No counterpart in the reference, which has no device.
 *   d_layers: device buffer, nz*ny*nx int32 cells with the ekg_heart_desc.layers convention
 *             (0 empty, L > 0 layer, -L stimulus voxel of layer L); layer ids at most 31
 *   transfer: host buffer, n_transfer x n_transfer conduction matrix (ms)
 *   d_at:     device buffer, nz*ny*nx doubles; receives the activation times (0 = empty or
 *             unreachable), bit-identical to ekg_heart_activation
 * Scratch is one fixed device array inside the library (about 600 KB per GPU that loads it, held
 * until the process exits); grids of more than 65536 tiles of 8x8x8 cells are rejected with
 * EKG_ERR_BAD_INPUT.  The first call on a device looks the array's device address up.  Every call
 * makes synchronous copies and waits for its kernels on the legacy default stream, so it must not
 * be called while any stream capture is in progress in the process.  The calls do not wait for
 * work on other streams: finish (or synchronise) every write to d_layers and every use of d_at
 * before the call.  A call returns when the result is in d_at; calls in one process are
 * serialised, and device work of two calls must not overlap (they share the array). */
int ekg_activation_noalloc(int32_t nz, int32_t ny, int32_t nx, const int32_t *d_layers, int32_t n_transfer,
                           const double *transfer, double *d_at, int32_t *rounds_out);

/* Self-test of the kernels' bounded device waits, for failure-detection tests that must not hang
 * or fault the GPU.  No counterpart in the reference (it has no device).  One block takes tensor
 * memory, waits on an mbarrier that nothing arrives on for at most wait_limit polls (the
 * contraction kernels' own wait helper, whose limit is 2^22 polls), records the timeout bit in the
 * error word, releases the tensor memory and returns; the host reads the word.  Returns
 * EKG_ERR_TIMEOUT when the wait ran out (the expected outcome), after which the device stays
 * usable. */
int ekg_selftest_bounded_wait(int32_t device, uint32_t wait_limit);

/* ------------------------------------------------------------------ files */
/* Build a heart and its eval config from a simulator.ini and the files it names, as the
 * SimImplementation constructor does (sim.cpp:362-431): settings, transfer matrix, measuring
 * points, shape, excitation sequence, targets (target_chk.column is written to `out_dir`
 * when it is not NULL, as sim.cpp:1031-1039 does).  "[model] excitation sequence" loads the
 * activation times from that .matrix file instead of computing them, and "[output files]
 * excitation sequence" writes them (3 decimals) to that file, as simlib/sim_lib.h:224-231 with
 * simlib/simulator.cpp:71-106 and :288-367 do. */
int ekg_heart_from_ini(ekg_engine *e, const char *ini_path, const char *out_dir, ekg_heart **out);

/* Lead positions after moving them by per-lead (u, v) displacements (n_leads x 2) in the
 * plane basis of EkgSim::loadMeasuringPoints / moveMeasuringPoints (simlib/sim_lib.h:167-208). */
int ekg_move_leads(int32_t n_leads, const double *orig_zyx, const double *disp_uv, double *out_zyx);

/* Value at time t of the AP of a cell activated at time `at` (WohlfartPlus with k8 shifted by at,
 * simlib/simulator.cpp:154-170 and simlib/Wohlfart.h:195-203), FP64 on the host.  Used for the
 * layer_aps / cell_aps outputs (sim.cpp:939-991). */
double ekg_ap_value(const double *k9, double at, double t);
/* Layer (1-based) and activation time of the cell AP with the reference's apIndex `index`
 * (first appearance in raster order, simlib/simulator.cpp:570-590). */
int ekg_heart_cell_ap(ekg_heart *h, int64_t index, int32_t *layer_out, double *at_out);

/* Layer APs from the Wohlfart genes (sim.cpp:751-916 with nonlinearFit.h:92-168) under the
 * interpolation settings of `cfg` (targets are not read); also the violation (sim.cpp:582-596).
 * Host-only: needs no device. */
int ekg_layer_aps(const ekg_eval_config *cfg, int32_t n_layers, const double *wohlfart_genes, double *layer_k_out,
                  double *violation_out);

#ifdef __cplusplus
}
#endif
#endif /* EKGSIM_H_INCLUDED */
