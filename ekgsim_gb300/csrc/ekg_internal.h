// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <condition_variable>
#include <functional>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/ekgsim.h"

namespace ekg {

// ------------------------------------------------------------------ errors
void set_error(const std::string &msg);
struct Error {
    int code;
    std::string msg;
};
#define EKG_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t err_ = (call);                                                          \
        if (err_ != cudaSuccess)                                                            \
            throw ::ekg::Error{EKG_ERR_DEVICE, std::string(#call) + ": " + cudaGetErrorString(err_)}; \
    } while (0)
#define EKG_CHECK(cond, code, msg)                                                          \
    do {                                                                                    \
        if (!(cond)) throw ::ekg::Error{(code), (msg)};                                     \
    } while (0)

// Runs f, mapping a thrown Error / std::exception to a status code and the thread's last error.
int guard(const std::function<void()> &f);

// Kernel error word bits (written by bounded device waits, read by the host after a pass).
enum : uint32_t { KERR_MBAR_TIMEOUT = 1u, KERR_TMEM = 2u };

// Float-float ("double-single") arithmetic with error-free transformations (Knuth's two-sum, an
// FMA two-product): about 48 significant bits on the FP32 pipe, for sums where GB300's FP64 rate
// would dominate.  The hi part is the float nearest the value, lo the remainder.  The _rn
// intrinsics keep the compiler from contracting a product into the error-free steps.
#ifdef __CUDACC__
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 ff_norm(float h, float e) {
    const float s = __fadd_rn(h, e);
    return make_float2(s, __fsub_rn(e, __fsub_rn(s, h)));
}
__device__ __forceinline__ float2 ff_add(float2 x, float2 y) {
    const float2 s = ff_two_sum(x.x, y.x);
    return ff_norm(s.x, __fadd_rn(__fadd_rn(s.y, x.y), y.y));
}
__device__ __forceinline__ float2 ff_add_f(float2 x, float b) {
    const float2 s = ff_two_sum(x.x, b);
    return ff_norm(s.x, __fadd_rn(s.y, x.y));
}
__device__ __forceinline__ float2 ff_mul(float2 x, float2 y) {
    const float p = __fmul_rn(x.x, y.x);
    const float e = fmaf(x.x, y.y, fmaf(x.y, y.x, fmaf(x.x, y.x, -p)));
    return ff_norm(p, e);
}
__device__ __forceinline__ float2 ff_neg(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ double ff_to_double(float2 x) { return (double)x.x + (double)x.y; }
__device__ __forceinline__ float2 ff_from_double(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
#endif

// device buffer owning helper
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DBuf &operator=(DBuf &&o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            throw Error{EKG_ERR_OUT_OF_MEMORY, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
        }
        n = count;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// ------------------------------------------------------------------ CA (ca.cu)
struct CaResult {
    int rounds = 0;        // tile rounds, or bucket launches of the bucketed relaxation
    float ms = 0.f;
    bool buckets = false;  // the bucketed relaxation ran
};
// Bucketed relaxation (Dijkstra by time buckets); false when it does not apply and ca_run must run.
bool ca_run_buckets(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_layers, const uint8_t *d_start,
                    const std::vector<double> &lag_h, int nl1, const double *d_lag, double *d_at, int64_t nvox,
                    int round_cap, int sm_count, CaResult &res);
// layers_u8: stripped layer per cell; start flags in `is_start`; lag: [nl1][nl1][3] FP64 with
// lag[s][d][k-1] = T[s][d] * sqrt(k).  at_out: FP64 per cell (0 for empty / unreachable).
CaResult ca_run(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_layers, const uint8_t *d_start,
                const std::vector<int32_t> &start_tiles, int nl1, const double *d_lag, double *d_at, int round_cap,
                int sm_count);

// ------------------------------------------------------------------ ECG kernels (ecg.cu)
// Heart-resident device arrays used by the simulation kernels.
struct HeartDev {
    int nz = 0, ny = 0, nx = 0;
    int64_t nvox = 0, naps = 0, apad = 0;  // apad: A rounded to a multiple of 64 per layer (K tiles)
    int nlayers = 0, nleads = 0, steps = 0, nhood = 0;
    int nchunks = 0;                        // K chunks (each inside one layer)
    int chunk_max = 0;                      // APs of the longest chunk
    // per-AP (ordered by (layer, at), padded per layer to a multiple of 64)
    DBuf<float2> at_hilo;   // [apad] activation time split hi+lo (pad: +inf -> H = 0)
    DBuf<double> at;        // [apad]
    DBuf<int32_t> a_layer;  // [apad] layer index 0-based (pad: layer of its chunk)
    DBuf<int64_t> a_vox_begin;  // [apad + 1] voxel ranges (voxels sorted by AP)
    // per voxel (sorted by AP)
    DBuf<int32_t> vox_zyx;  // [nvox] packed z<<20 | y<<10 | x  (each < 1024)
    DBuf<uint32_t> vox_nb;  // [nvox] bits 0..25: in-neighbour mask, (unused high bits)
    DBuf<uint32_t> vox_nbo; // [nvox] out-neighbour mask
    DBuf<float4> vox_pos;   // [nvox] bordered position relative to `centre` (z,y,x) + in-mask bits in .w
    DBuf<float4> vox_out;   // [nvox] sum of the out-neighbour offsets (z,y,x), .w = 1 if any
    DBuf<float4> stage_box; // [2 * apad / 32] per 32-AP stage: lowest and highest voxel position (z,y,x)
    DBuf<int32_t> stage_order;  // [apad / 32] stages by descending voxel count (field kernels' item order)
    double centre[3] = {0, 0, 0};
    // K chunks
    DBuf<int32_t> chunk_a0, chunk_a1, chunk_layer;  // [nchunks]
    DBuf<int32_t> layer_c0, layer_c1;               // [nlayers] chunk range of each layer (empty: 0, 0)
    // neighbourhood offsets (z,y,x) as int8 triples
    int nnb = 0;
    int8_t nb_dif[26 * 3];
    DBuf<int8_t> difs;      // [nnb*3] device copy of nb_dif
    // closed form of the field of a voxel with every neighbour present (moved-lead operand):
    // coefficients A0, A1, B0, B1, B2 of rho u^2 [(A0 + u B0) + u^2 (P (A1 + u B1) + u^2 B2 Q)];
    // mask 0 when the set lacks cube symmetry
    float interior_c[5] = {0, 0, 0, 0, 0};
    uint32_t interior_mask = 0;
    int64_t n_interior = 0;  // voxels flagged interior
    // time axis
    DBuf<double> t;         // [steps]
    DBuf<float2> t_hilo;    // [steps]
};

// De-duplication of a heart's voxels into APs on the device (setup.cu): the voxels sorted by
// (layer, activation time, cell), the first voxel of every AP, and per present layer (in order)
// its first AP, AP count and base in the padded (multiple of 64) per-layer K layout.
struct DedupResult {
    int64_t nvox = 0, naps = 0, apad = 0;
    std::vector<int> pl_layer, pfirst, pcount;  // per present layer: id (1-based), first AP, APs
    std::vector<int64_t> pbase;                  // per present layer: first padded AP slot
    DBuf<int> cell;                              // [nvox] cell of each sorted voxel
    DBuf<int> gstart;                            // [naps (+1)] first sorted voxel of each AP
    DBuf<uint64_t> key;                          // [nvox] activation-time bits of each sorted voxel
    DBuf<uint8_t> vl;                            // [nvox] layer of each sorted voxel
};
void setup_voxels_device(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_lay, const double *d_at_cells,
                         int nl, DedupResult &r);
// at / at_hilo / a_layer [apad], a_vb [apad + 1]
void setup_ap_arrays_device(cudaStream_t s, const DedupResult &r, const double *d_at_cells, double *at,
                            float2 *at_hilo, int32_t *a_layer, int64_t *a_vb);
// per-voxel records of the dipole kernels; returns the number of voxels flagged interior
// Bounding box of each 32-AP stage's voxel positions (empty stages: an inverted box).
void setup_stage_boxes_device(cudaStream_t s, int64_t apad, const int64_t *a_vox_begin, const float4 *vox_pos,
                              float4 *stage_box);
int64_t setup_voxel_records_device(cudaStream_t s, const DedupResult &r, int nz, int ny, int nx, const uint8_t *d_lay,
                                   const HeartDev &D, int few_max, int32_t *vzyx, uint32_t *vin, uint32_t *vout,
                                   float4 *vpos, float4 *vosum);

// Per-evaluation scratch (sized for n_sims simulations).
struct EvalDev {
    int cap_sims = 0;
    DBuf<float> layer_c;    // [S][nl][4]: k1*log2e, k4*log2e, 1-k3, k3 (FP32 H constants)
    DBuf<double> F;         // [S][nl][steps]
    DBuf<float> Ff;         // [S][nl][steps] the same in FP32 (batched form)
    DBuf<double> k0w;       // [S][L] constant k0 term
    DBuf<float> W;          // [S][L][apad] lead field for this eval's positions
    DBuf<float> Wp;         // [S][L][apad] W * exp(k5 at)
    DBuf<double> partial;   // [S][nchunks][L][steps] (dense contractions)
    DBuf<float> band;       // [S][nchunks][L][steps] band-step values (band contraction)
    DBuf<float2> csum;      // [S][nchunks][L] steady sums (S0, S1)
    DBuf<int4> cinfo;       // [S][nchunks] (first band step, first steady step, amax bits, 0)
    DBuf<int> work;         // work-item counter of the moved-row field kernel
    DBuf<float> coef;       // [S][nl][J] static-lead Taylor coefficients (batched form)
    DBuf<double> ecg;       // [S][L][steps]
    DBuf<float2> ecg_ff;    // [S][L][steps] the same as float-float (hi, lo), read by the criteria
    DBuf<double> crit;      // [S][ncrit]
    DBuf<double> targets;   // concatenated targets
    DBuf<float2> targets_ff;  // the same as float-float
    DBuf<int64_t> target_len;
    DBuf<double> target_off;
    DBuf<uint32_t> err;     // [1]
};

void launch_lead_field(cudaStream_t s, const HeartDev &h, const double *d_leads, int nleads_in, int lead_stride,
                       int n_sims, float *d_W, int w_lead_stride);
void launch_layer_factors(cudaStream_t s, const HeartDev &h, const double *d_layer_k, const double *d_cpre,
                          int n_sims, double *d_F, float *d_Ff, float *d_layer_c, const double *d_centre = nullptr,
                          const double *d_scale = nullptr, int J = 0, float *d_coef = nullptr);
// per-simulation form: W and (Wp not null) W' = W exp(k5 at) of the moved rows from the lead
// positions, and with static_rows W' of the other rows from the resident field W0 (batch.cu)
void launch_sim_lead_field(cudaStream_t s, const HeartDev &h, const double *d_leads, int nmove, int lead_stride,
                           int n_sims, const double *d_layer_k, const float *W0, float *W, float *Wp,
                           bool static_rows);
// the same W of the moved rows for many simulations, with the batched operand kernel's work split;
// work: a device counter (zeroed here)
void launch_sim_lead_field_rows(cudaStream_t s, const HeartDev &h, const double *d_leads, int nmove, int lead_stride,
                                int n_sims, float *W, int *work, int sm_count);
// k0w[s][l] = sum_a k0_{layer(a)} W[s][l][a] for the first `rows` leads
void launch_k0_term(cudaStream_t s, const HeartDev &h, const float *d_W, const double *d_layer_k, int n_sims,
                    double *d_k0w, int rows);
// out[L][l] = sum_{a in layer L} W0[l][a] in FP64 (batch.cu)
void launch_w0_layer_sums(cudaStream_t s, const HeartDev &h, const float *W0, double *out);
void launch_contract_cuda(cudaStream_t s, const HeartDev &h, const float *d_Wp, const float *d_layer_c,
                          const double *d_F, int n_sims, double *d_partial);
// band form (zero / steady / band steps per chunk) for chunks of up to CONTRACT_BAND_CAP APs
constexpr int CONTRACT_BAND_CAP = 512;
// band[S][nchunks][L][steps] (band steps only), csum[S][nchunks][L], cinfo[S][nchunks]; the field
// is Wm [S][L][apad] (unscaled) for rows l < wrows and the resident W0 for the others
void launch_contract_band(cudaStream_t s, const HeartDev &h, const float *d_Wm, int wrows, const float *d_W0,
                          const double *d_layer_k, const float *d_layer_c, int n_sims, float *d_band, float2 *d_csum,
                          int4 *d_cinfo);
// ecg (and its float-float copy) from the band contraction's outputs plus k0w
void launch_reduce_chunks(cudaStream_t s, const HeartDev &h, const float *d_layer_c, const double *d_F,
                          const float *d_band, const float2 *d_csum, const int4 *d_cinfo, const double *d_k0w,
                          int n_sims, double *d_ecg, float2 *d_ecg_ff);
void launch_contract_umma(cudaStream_t s, const HeartDev &h, const float *d_Wp, const float *d_layer_c,
                          const double *d_F, int n_sims, double *d_partial, uint32_t *d_err);
// Explicit-argument form: `rows` weight rows (leads) per simulation, Wp [S][rows][apad],
// layer_c [S][nl] float4, F [S][nl][steps], partial [S][nchunks][rows][steps].
struct ContractArgs {
    int steps = 0, rows = 0, nl = 0, nchunks = 0, n_sims = 1;
    int64_t apad = 0;
    const float2 *t_hilo = nullptr, *at_hilo = nullptr;
    const int32_t *chunk_a0 = nullptr, *chunk_a1 = nullptr, *chunk_layer = nullptr;
    const float *Wp = nullptr, *layer_c = nullptr;
    const double *F = nullptr;
    double *partial = nullptr;
    uint32_t *err = nullptr;
};
void launch_contract_umma_args(cudaStream_t s, const ContractArgs &a);

// ------------------------------------------------------------------ batched form (batch.cu)
struct BatchArgs {
    int steps = 0, nl = 0, nkt = 0, rows = 0, rows_used = 0, nmove = 0, n_sims = 0, ntiles = 0, nitems = 0,
        two_bases = 0, tile_rows = 0;
    const float2 *t_hilo = nullptr, *at_hilo = nullptr;
    const int4 *items = nullptr;  // (t tile, first stage, end stage, layer), stages of 32 APs
    const float4 *hconst = nullptr;
    const uint8_t *Bt = nullptr;
    float *partial = nullptr;     // [items][rows][128] raw accumulators (x2 with two bases)
    uint32_t *err = nullptr;
};
// Steady part of the moved-lead ECG and the final reduction (batch.cu k_batch_lead_field,
// k_band_u, k_reduce_band).
struct BandArgs {
    int n_sims = 0, nmove = 0, nl = 0, ntt = 0, steps = 0, rows = 0, rows_used = 0, nleads = 0;
    int max_ent = 1, nb = 1;
    const int32_t *ti0 = nullptr, *ti1 = nullptr;  // [ntt][nl] item range of (tile, layer)
    const float2 *tref = nullptr;                   // [stages] last finite activation time of each 32-AP stage
    const int32_t *stage_order = nullptr;           // [stages] by descending voxel count (HeartDev's)
    const int32_t *nent = nullptr, *esplit = nullptr, *ls0 = nullptr, *ls1 = nullptr;  // stage units
    const int32_t *ent = nullptr;
    const int64_t *goff = nullptr;
    const float *gtab = nullptr;
    const float *E = nullptr, *F = nullptr, *partial = nullptr;
    const double *k3 = nullptr;
    float2 *P1 = nullptr;            // [stages][rows] steady sums per 32-AP stage
    float *P2 = nullptr;             // [stages * 4][rows] unscaled field sums per 8-AP part, or null
    const double *cmov = nullptr;    // [rows'] resting-potential constant of each moved-lead row, or null
    float2 *Up = nullptr;            // [band_u_parts()][rows][nl][max_ent]
    float2 *U = nullptr;             // [rows][nl][max_ent]
    double *ecg = nullptr;
    float2 *ecg_ff = nullptr;
};
int batch_tile_rows(int two_bases, int rows_used);
int small_operand_sims();  // passes up to this many simulations use the per-(AP, simulation) operand kernel
void launch_taylor_w(cudaStream_t s, const HeartDev &h, const float *W0, int J, const double *centre,
                     const double *scale, float *Wt);
void launch_reduce_layers(cudaStream_t s, int steps, int rows, int nl, const int32_t *lc0, const int32_t *lc1,
                          const double *partial, float *Q);
void launch_static_combine(cudaStream_t s, const HeartDev &h, int J, int Jb, int nmove, int n_sims, const float *F,
                           const float *coef, const double *k3, const float *Q1, const float *Q2, double *ecg,
                           float2 *ecg_ff, const double *cst = nullptr);
void launch_batch_lead_field(cudaStream_t s, const HeartDev &h, int tile_rows, bool small, int blocks_per_sm,
                             const float *k5l,
                             const float4 *hconst, const float4 *lrel, int nmove, int n_sims, const BandArgs &B,
                             uint8_t *Bt, int *work, int sm_count);
void launch_batch_gemm(cudaStream_t s, const BatchArgs &a);
int band_u_parts();
void launch_band_u(cudaStream_t s, const BandArgs &a);
// Resting-potential term of the batched form where k0 differs between layers:
//   moved rows   cmov[l * S + s] = sum_L (k0_L - k0_0) sum_{a in L} W_s[l][a]   (from P2)
//   static leads K0s[L][l] = sum_{a in L} W0[l][a] (per heart), cst[s][l] = sum_L (k0_L - k0_0) K0s[L][l]
void launch_k0_moved(cudaStream_t s, const BandArgs &a, const int32_t *ls0, const int32_t *ls1,
                     const double *layer_k, double *cmov);
void launch_k0_static_sums(cudaStream_t s, int nleads, int64_t apad, int nl, const int32_t *ls0,
                           const int32_t *ls1, const float *W0, double *K0s);
// cst[s][l] (l >= nmove) = sum_L (k0_L - k0_0) K0s[L][l], or sum_L k0_L K0s[L][l] when !relative
void launch_k0_static(cudaStream_t s, int n_sims, int nleads, int nmove, int nl, const double *K0s,
                      const double *layer_k, double *cst, bool relative = true);
void launch_reduce_band(cudaStream_t s, const BandArgs &a);
void launch_reduce_ecg(cudaStream_t s, const HeartDev &h, const double *d_partial, const double *d_k0w,
                       int n_sims, double *d_ecg, float2 *d_ecg_ff);
// criteria of the criterion leads [i0, i1) of every simulation
void launch_criteria(cudaStream_t s, const HeartDev &h, const double *d_ecg, const float2 *d_ecg_ff, int n_sims,
                     int ncrit_stride, int i0, int i1, int mode, const double *d_targets, const float2 *d_targets_ff,
                     const int64_t *d_tlen, const double *d_toff, double *d_crit);

}  // namespace ekg
