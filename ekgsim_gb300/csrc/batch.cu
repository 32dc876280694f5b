// batch.cu -- the batched form: many parameter vectors on one resident heart.
//
// Within a batch every simulation shares the heart (activation times, de-duplicated APs) and the
// per-layer AP shape coefficients k1 and k4, which the genes never change (they are interpolated
// between base APs, sim.cpp:705-709, and left alone by the steepest-descent fit, whose step vector
// is zero for them, sim.cpp:873-874).  With tau = t - at_a the cell AP factors as
//     AP_a(t) - k0 = F_L(t) exp(k5 at_a) [(1 - k3) B1_a(t) + k3 B2_a(t)],
//     B1_a(t) = sigma(k1 tau) exp(-k4 tau),   B2_a(t) = sigma(k1 tau),
// where only F_L (per layer and step), k5 and k3 depend on the simulation.  Hence:
//
// * Leads at their loaded position (the same lead field W0 for every simulation): exp(k5 at) is
//   expanded around the layer's mid activation time c_L, with u_a = (at_a - c_L)/s_L in [-1, 1]:
//       exp(k5 at_a) = exp(k5 c_L) sum_{j<J} (k5 s_L)^j / j! u_a^j   (truncation bound <= 1e-12),
//   so per heart the basis Q_{b,L,j}[l,t] = sum_{a in L} W0[l,a] u_a^j B_b,a(t) is contracted once
//   (tensor cores, ecg path), and each simulation's static-lead ECG is a short FP64 combination.
// * Moved leads (lead genes): one GEMM per batch on the tensor cores,
//       Y_b[(s,l), t] = sum_{a in L} W'_s[l,a] B_b,a(t),   W'_s = W_s exp(k5_s at_a),
//   with M = 128 steps, N = 256 (or 128) rows (simulation, moved lead), K = APs of one layer.
//   The B operand W' is written per batch in BF16 hi+lo, already tiled in the UMMA canonical
//   layout, and streamed into shared memory with 1-D bulk copies (TMA engine, mbarrier tx
//   counts); the A operand B_b,a(t) is evaluated by all 256 threads in FP32 per K stage.  The
//   epilogue forms ((1-k3) Y1 + k3 Y2) F_L(t) per row in FP64.  With a batch-uniform k3 the two
//   bases collapse into one (N = 256, three MMAs per K step instead of six).
#include <cmath>
#include <cstdio>

#include "ekg_internal.h"
#include "umma_ptx.h"

namespace ekg {

using namespace ptx;

namespace {

constexpr int BM = 128, BKT = 64, BTHREADS = 256;

__device__ __forceinline__ float ex2a(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcpa(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void split2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float r0 = x0 - __bfloat162float(h.x), r1 = x1 - __bfloat162float(h.y);
    __nv_bfloat162 l = __floats2bfloat162_rn(r0, r1);
    hi = *reinterpret_cast<uint32_t *>(&h);
    lo = *reinterpret_cast<uint32_t *>(&l);
}

// ------------------------------------------------------------------ Taylor basis weights
// Wt[(l*J + j)][a] = W0[l][a] * u_a^j, u_a = (at_a - c_L) / s_L  (0 for padding APs)
__global__ void k_taylor_w(int64_t apad, int nleads, int J, const float *__restrict__ W0,
                           const double *__restrict__ at, const int32_t *__restrict__ a_layer,
                           const double *__restrict__ centre, const double *__restrict__ scale, float *__restrict__ Wt) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (a >= apad) return;
    const double aa = at[a];
    const int L = a_layer[a];
    const double u = isinf(aa) ? 0.0 : (aa - centre[L]) / scale[L];
    const float w = W0[(size_t)l * apad + a];
    double p = 1.0;
    for (int j = 0; j < J; ++j) {
        Wt[((size_t)l * J + j) * apad + a] = isinf(aa) ? 0.f : (float)((double)w * p);
        p *= u;
    }
}

// Q[L][row][t] = sum over the chunks of layer L of partial[c][row][t] (chunks of a layer are
// contiguous, [lc0[L], lc1[L])); block per (row, 32 steps), warps split chunks, fixed order.
__global__ void k_reduce_layers(int steps, int rows, int nl, const int32_t *__restrict__ lc0,
                                const int32_t *__restrict__ lc1, const double *__restrict__ partial,
                                double *__restrict__ Q) {
    __shared__ double red[8][33];
    const int tt = blockIdx.x * 32 + (threadIdx.x & 31);
    const int w = threadIdx.x >> 5;
    const int row = blockIdx.y;
    for (int L = 0; L < nl; ++L) {
        double acc = 0.0;
        if (tt < steps)
            for (int c = lc0[L] + w; c < lc1[L]; c += 8) acc += partial[((size_t)c * rows + row) * steps + tt];
        red[w][threadIdx.x & 31] = acc;
        __syncthreads();
        if (w == 0 && tt < steps) {
            double r = 0.0;
            for (int i = 0; i < 8; ++i) r += red[i][threadIdx.x];
            Q[((size_t)L * rows + row) * steps + tt] = r;
        }
        __syncthreads();
    }
}

// Static leads: ecg[s][l][t] = sum_L F[s][L][t] sum_j coef[s][L][j] ((1-k3) Q1 + k3 Q2)[L][l*J+j][t]
__global__ void k_static_combine(int steps, int nleads, int nl, int J, int Jb, int nmove, int n_sims,
                                 const double *__restrict__ F, const double *__restrict__ coef,
                                 const double *__restrict__ k3, const double *__restrict__ Q1,
                                 const double *__restrict__ Q2, double *__restrict__ ecg) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = nmove + blockIdx.y, s = blockIdx.z;
    if (t >= steps || l >= nleads) return;
    const int rows = nleads * Jb;  // the basis stores Jb terms per lead
    double acc = 0.0;
    for (int L = 0; L < nl; ++L) {
        const double kk = k3[(size_t)s * nl + L];
        const double *c = coef + ((size_t)s * nl + L) * J;
        double v = 0.0;
        for (int j = 0; j < J; ++j) {
            const size_t q = ((size_t)L * rows + (size_t)l * Jb + j) * steps + t;
            v += c[j] * ((1.0 - kk) * Q1[q] + kk * Q2[q]);
        }
        acc += F[((size_t)s * nl + L) * steps + t] * v;
    }
    ecg[((size_t)s * nleads + l) * steps + t] = acc;
}

// ------------------------------------------------------------------ moved-lead operand
// W'_s[l][a] for the moved leads l < nmove, written as BF16 hi/lo into the tiled B layout:
// [N tile][K tile][part hi/lo][N*128 bytes], element (row n, k) of a tile at byte
// ((k/8) * (N/8) + n/8) * 128 + (n%8) * 16 + (k%8) * 2.
// Block = up to 128 simulations (one per thread) x one chunk of 8 consecutive APs, so the voxel
// data of the chunk is a broadcast load for the warp and each thread writes one 16-byte row
// segment per part; a warp's 32 simulations x nmove rows are contiguous in the tile.
// g at p = v + d uses |m - d|^2 = |m|^2 - 2 m.d + |d|^2 with m = r - v, and g.d = (m.d - |d|^2) f,
// f = |m - d|^-3: one rsqrt and a handful of FMAs per neighbour.
// w(v) for one lead relative position r (both relative to the same centre), general neighbourhood.
__device__ __forceinline__ float voxel_w_general(float4 pos, float4 out, float rz, float ry, float rx, int nnb,
                                                 const float *s_d) {
    const float mz = rz - pos.x, my = ry - pos.y, mx = rx - pos.z;
    const uint32_t mi = __float_as_uint(pos.w);
    const float s0 = fmaf(mz, mz, fmaf(my, my, mx * mx));
    float w = 0.f;
    for (int n = 0; n < nnb; ++n) {
        if (!(mi & (1u << n))) continue;
        const float4 d = reinterpret_cast<const float4 *>(s_d)[n];
        const float md = fmaf(mz, d.x, fmaf(my, d.y, mx * d.z));
        const float rs = rsqrtf(fmaf(-2.f, md, s0 + d.w));
        w = fmaf(rs * rs * rs, md - d.w, w);
    }
    if (out.w != 0.f) {
        const float rs = rsqrtf(s0);
        w = fmaf(-(rs * rs * rs), fmaf(mz, out.x, fmaf(my, out.y, mx * out.z)), w);
    }
    return w;
}

// Same for the 8 body diagonals ("3D4", creation order (-1,-1,-1) ... (1,1,1)): with p = my + mx and
// q = my - mx the eight m.d are -mz-p, -mz-q, -mz+q, -mz+p, mz-p, mz-q, mz+q, mz+p; |d|^2 = 3.
// Missing neighbours are masked by multiplying their term by 0 (branch-free).
__device__ __forceinline__ float voxel_w_diag(float4 pos, float4 out, float rz, float ry, float rx) {
    const float mz = rz - pos.x, my = ry - pos.y, mx = rx - pos.z;
    const uint32_t mi = __float_as_uint(pos.w);
    const float s0 = fmaf(mz, mz, fmaf(my, my, mx * mx));
    const float s3 = s0 + 3.f;
    const float p = my + mx, q = my - mx;
    const float md[8] = {-mz - p, -mz - q, -mz + q, -mz + p, mz - p, mz - q, mz + q, mz + p};
    float w = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float rs = rsqrtf(fmaf(-2.f, md[n], s3));
        const float t = (rs * rs * rs) * (md[n] - 3.f);
        w += ((mi >> n) & 1u) ? t : 0.f;
    }
    const float rs0 = rsqrtf(s0);
    w = fmaf(-(rs0 * rs0 * rs0) * out.w, fmaf(mz, out.x, fmaf(my, out.y, mx * out.z)), w);
    return w;
}

template <int N, bool DIAG>
__global__ void __launch_bounds__(128) k_batch_lead_field(
    int64_t apad, int nkt, const int64_t *__restrict__ a_vox_begin, const float4 *__restrict__ vox_pos,
    const float4 *__restrict__ vox_out, int nnb, const int8_t *__restrict__ difs, const double *__restrict__ at,
    const int32_t *__restrict__ a_layer, const double *__restrict__ layer_k, int nl, const double *__restrict__ leads,
    double cz, double cy, double cx, int nleads, int nmove, int n_sims, uint8_t *__restrict__ Bt) {
    __shared__ float s_d[26 * 4];
    if (threadIdx.x < nnb) {
        const float dz = difs[3 * threadIdx.x], dy = difs[3 * threadIdx.x + 1], dx = difs[3 * threadIdx.x + 2];
        s_d[4 * threadIdx.x] = dz;
        s_d[4 * threadIdx.x + 1] = dy;
        s_d[4 * threadIdx.x + 2] = dx;
        s_d[4 * threadIdx.x + 3] = dz * dz + dy * dy + dx * dx;
    }
    __syncthreads();
    const int64_t a0 = (int64_t)blockIdx.x * 8;
    const int s = blockIdx.y * blockDim.x + threadIdx.x;
    if (s >= n_sims) return;
    const int kt = (int)(a0 / BKT), kc = (int)((a0 % BKT) / 8);
    float e[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const double aa = at[a0 + j];
        e[j] = isinf(aa) ? 0.f : expf((float)(layer_k[((size_t)s * nl + a_layer[a0 + j]) * 9 + 5] * aa));
    }
    // leads in pairs: the voxel data of the chunk is loaded once per pair
    for (int l0 = 0; l0 < nmove; l0 += 2) {
        const bool two = l0 + 1 < nmove;
        float r0[3], r1[3] = {0.f, 0.f, 0.f};
        {
            // lead positions relative to the same centre as vox_pos (difference taken in FP64)
            const double *r = leads + ((size_t)s * nleads + l0) * 3;
            r0[0] = (float)(r[0] - cz);
            r0[1] = (float)(r[1] - cy);
            r0[2] = (float)(r[2] - cx);
            if (two) {
                r1[0] = (float)(r[3] - cz);
                r1[1] = (float)(r[4] - cy);
                r1[2] = (float)(r[5] - cx);
            }
        }
        float w0[8], w1[8];
        int64_t v = a_vox_begin[a0];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t ve = a_vox_begin[a0 + j + 1];
            float acc0 = 0.f, acc1 = 0.f;
            for (; v < ve; ++v) {
                const float4 pos = vox_pos[v], out = vox_out[v];
                if (DIAG) {
                    acc0 += voxel_w_diag(pos, out, r0[0], r0[1], r0[2]);
                    if (two) acc1 += voxel_w_diag(pos, out, r1[0], r1[1], r1[2]);
                } else {
                    acc0 += voxel_w_general(pos, out, r0[0], r0[1], r0[2], nnb, s_d);
                    if (two) acc1 += voxel_w_general(pos, out, r1[0], r1[1], r1[2], nnb, s_d);
                }
            }
            w0[j] = acc0 * e[j];
            w1[j] = acc1 * e[j];
        }
        for (int q = 0; q < (two ? 2 : 1); ++q) {
            const float *wv = q ? w1 : w0;
            uint4 hv, lv;
            split2(wv[0], wv[1], hv.x, lv.x);
            split2(wv[2], wv[3], hv.y, lv.y);
            split2(wv[4], wv[5], hv.z, lv.z);
            split2(wv[6], wv[7], hv.w, lv.w);
            const int row = s * nmove + l0 + q;
            const int nt = row / N, n = row % N;
            const size_t tile = ((size_t)nt * nkt + kt) * 2;
            const size_t off = (size_t)(kc * (N / 8) + n / 8) * 128 + (n % 8) * 16;
            *reinterpret_cast<uint4 *>(Bt + tile * (N * 128) + off) = hv;
            *reinterpret_cast<uint4 *>(Bt + (tile + 1) * (N * 128) + off) = lv;
        }
    }
}

// ------------------------------------------------------------------ batch GEMM
// Warp-specialised: warps 0-7 produce the A operand (B_b,a(t) in BF16 hi/lo) and drain the
// accumulators; one lane of warp 8 streams the B operand with 1-D bulk copies; one lane of warp 9
// issues the MMAs.  Rings: SA stages of A, SB stages of B (32 APs per stage); full/empty mbarrier
// pairs per stage; two TMEM accumulator sets with full/empty barriers for the segment drains.
// The tensor core's FP32 accumulation loses accuracy over long K (measured: relative ECG error
// grows with the K length of one accumulation), so the K range is cut into segments of DRAIN
// stages (512 APs): segment g accumulates in TMEM set g % 2 and is drained into FP32 registers
// (each producer thread owns one row and half of the columns) while segment g + 1 accumulates.
constexpr int WKT = 32;              // APs per stage
constexpr int SA = 3, SB = 4;        // ring depths
constexpr int DRAIN = 512 / WKT;     // stages per accumulation segment
constexpr int WS_THREADS = 320;      // 8 producer warps + bulk-copy warp + MMA warp

template <int NB, int N>
struct BatchSmem {
    alignas(1024) uint8_t a[SA][NB][2][BM * WKT * 2];  // [stage][basis][hi/lo]
    alignas(1024) uint8_t b[SB][2][N * WKT * 2];       // [stage][hi/lo]
    alignas(8) uint64_t a_full[SA], a_empty[SA], b_full[SB], b_empty[SB], acc_full[2], acc_empty[2];
    uint32_t tmem_base;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// grid (t tiles, N tiles, K chunks).  Chunk c covers 64-AP tiles [ck0[c], ck1[c]) inside layer cl[c].
template <int NB, int N>
__global__ void __launch_bounds__(WS_THREADS, 1) k_batch_umma(
    int steps, int nl, int nkt, int rows, int nmove, int n_sims, const float2 *__restrict__ t_hilo,
    const float2 *__restrict__ at_hilo, const int32_t *__restrict__ ck0, const int32_t *__restrict__ ck1,
    const int32_t *__restrict__ cl, const float4 *__restrict__ hconst, const double *__restrict__ k3,
    const double *__restrict__ F, const uint8_t *__restrict__ Bt, double *__restrict__ partial,
    uint32_t *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    BatchSmem<NB, N> &S =
        *reinterpret_cast<BatchSmem<NB, N> *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr uint32_t SET = NB * N;        // columns of one accumulator set
    constexpr uint32_t TCOLS = 2 * SET;     // 512
    constexpr uint32_t IDESC = idesc_bf16(BM, N);
    constexpr uint32_t A_LBO = (BM / 8) * 128, A_SBO = 128;
    constexpr uint32_t B_LBO = (N / 8) * 128, B_SBO = 128;
    constexpr uint32_t BTILE = N * BKT * 2;  // one part of a 64-AP tile in global memory
    constexpr uint32_t BSTAGE = N * WKT * 2; // one part of a 32-AP stage
    constexpr int HALF = N / 2;
    constexpr int NACC = NB * HALF;         // 128
    constexpr int NPROD = 256;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int t0 = blockIdx.x * BM, nt = blockIdx.y, c = blockIdx.z;
    const int st0 = 2 * ck0[c], nk = 2 * (ck1[c] - ck0[c]), L = cl[c];
    const int nseg = (nk + DRAIN - 1) / DRAIN;

    if (tid == 0) {
        for (int i = 0; i < SA; ++i) {
            mbar_init(&S.a_full[i], NPROD);
            mbar_init(&S.a_empty[i], 1);
        }
        for (int i = 0; i < SB; ++i) {
            mbar_init(&S.b_full[i], 1);
            mbar_init(&S.b_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&S.acc_full[i], 1);
            mbar_init(&S.acc_empty[i], NPROD);
        }
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(&S.tmem_base, TCOLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    bool ok = true;

    if (warp < 8) {
        // ---------------- producers and drains
        const float4 hc = hconst[L];
        const int q = warp & 3, ch = warp >> 2;  // TMEM lane quadrant, column half
        const int row = tid & (BM - 1), half = tid >> 7;
        const float2 th = t_hilo[min(t0 + row, steps - 1)];
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
        float acc[NACC];
#pragma unroll
        for (int i = 0; i < NACC; ++i) acc[i] = 0.f;
        int drained = 0;
        auto drain = [&](int g) {
            if (!mbar_wait(&S.acc_full[g & 1], (uint32_t)((g >> 1) & 1))) {
                ok = false;
                return;
            }
            tc_fence_after();
            const uint32_t base = lane_addr + (uint32_t)((g & 1) * SET);
#pragma unroll
            for (int bsi = 0; bsi < NB; ++bsi)
#pragma unroll
                for (int cb = 0; cb < HALF; cb += 16) {
                    float v[16];
                    tmem_ld16(base + (uint32_t)(bsi * N + ch * HALF + cb), v);
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj) acc[bsi * HALF + cb + jj] += v[jj];
                }
            tc_fence_before();
            mbar_arrive(&S.acc_empty[g & 1]);
        };
        for (int i = 0; i < nk && ok; ++i) {
            const int sa = i % SA, u = i / SA;
            // drain segment g once production is SA stages into segment g + 1
            if (i >= SA && (i - SA) % DRAIN == 0 && (i - SA) >= DRAIN) {
                drain(drained);
                ++drained;
                if (!ok) break;
            }
            if (u > 0 && !mbar_wait(&S.a_empty[sa], (uint32_t)((u - 1) & 1))) {
                ok = false;
                break;
            }
            const float2 *atp = at_hilo + (size_t)(st0 + i) * WKT + half * 16;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int kc8 = half * 2 + j;
                float v1[8], v2[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float2 at = __ldg(atp + j * 8 + e);
                    const float tau = (th.x - at.x) + (th.y - at.y);
                    const float e1 = ex2a(-hc.x * tau);
                    const float sg = rcpa(1.0f + e1);
                    const float e4 = ex2a(-hc.y * tau);
                    if (NB == 1) {
                        const float h = sg * fmaf(hc.z, e4, hc.w);
                        v1[e] = sg == 0.f ? 0.f : h;
                    } else {
                        const float h = sg * e4;
                        v1[e] = sg == 0.f ? 0.f : h;
                        v2[e] = sg;
                    }
                }
                const uint32_t off = (uint32_t)((kc8 * (BM / 8) + row / 8) * 128 + (row % 8) * 16);
                uint4 hv, lv;
                split2(v1[0], v1[1], hv.x, lv.x);
                split2(v1[2], v1[3], hv.y, lv.y);
                split2(v1[4], v1[5], hv.z, lv.z);
                split2(v1[6], v1[7], hv.w, lv.w);
                *reinterpret_cast<uint4 *>(S.a[sa][0][0] + off) = hv;
                *reinterpret_cast<uint4 *>(S.a[sa][0][1] + off) = lv;
                if (NB == 2) {
                    split2(v2[0], v2[1], hv.x, lv.x);
                    split2(v2[2], v2[3], hv.y, lv.y);
                    split2(v2[4], v2[5], hv.z, lv.z);
                    split2(v2[6], v2[7], hv.w, lv.w);
                    *reinterpret_cast<uint4 *>(S.a[sa][NB - 1][0] + off) = hv;
                    *reinterpret_cast<uint4 *>(S.a[sa][NB - 1][1] + off) = lv;
                }
            }
            fence_proxy_async_smem();
            mbar_arrive(&S.a_full[sa]);
        }
        while (ok && drained < nseg) {
            drain(drained);
            ++drained;
        }
        if (ok && nk > 0) {
            const int t = t0 + 32 * q + lane;
            if (t < steps) {
#pragma unroll
                for (int jj = 0; jj < HALF; ++jj) {
                    const int r = nt * N + ch * HALF + jj;
                    const int s = r / nmove;
                    if (s >= n_sims) continue;
                    const double f = F[((size_t)s * nl + L) * steps + t];
                    double v;
                    if (NB == 2) {
                        const double kk = k3[(size_t)s * nl + L];
                        v = ((1.0 - kk) * (double)acc[jj] + kk * (double)acc[HALF + jj]) * f;
                    } else {
                        v = (double)acc[jj] * f;
                    }
                    partial[((size_t)c * rows + r) * steps + t] = v;
                }
            }
        }
    } else if (warp == 8 && lane == 0) {
        // ---------------- B operand: 32-AP halves of the tiled 64-AP layout, one bulk copy per part
        for (int i = 0; i < nk; ++i) {
            const int sb = i % SB, v = i / SB;
            if (v > 0 && !mbar_wait(&S.b_empty[sb], (uint32_t)((v - 1) & 1))) {
                ok = false;
                break;
            }
            const int st = st0 + i;
            const uint8_t *src = Bt + ((size_t)nt * nkt + st / 2) * 2 * BTILE + (size_t)(st & 1) * BSTAGE;
            mbar_expect_tx(&S.b_full[sb], 2 * BSTAGE);
            bulk_g2s(S.b[sb][0], src, BSTAGE, &S.b_full[sb]);
            bulk_g2s(S.b[sb][1], src + BTILE, BSTAGE, &S.b_full[sb]);
        }
    } else if (warp == 9 && lane == 0) {
        // ---------------- MMA issue
        for (int i = 0; i < nk; ++i) {
            const int sa = i % SA, sb = i % SB, g = i / DRAIN;
            if (!mbar_wait(&S.a_full[sa], (uint32_t)((i / SA) & 1)) ||
                !mbar_wait(&S.b_full[sb], (uint32_t)((i / SB) & 1))) {
                ok = false;
                break;
            }
            const bool first = (i % DRAIN) == 0;
            if (first && g >= 2 && !mbar_wait(&S.acc_empty[g & 1], (uint32_t)(((g - 2) >> 1) & 1))) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t set = (uint32_t)((g & 1) * SET);
            const uint32_t bh = smem_u32(S.b[sb][0]), bl = smem_u32(S.b[sb][1]);
#pragma unroll
            for (int j = 0; j < WKT / 16; ++j) {
                const uint64_t dbh = sdesc(bh + j * 2 * B_LBO, B_LBO, B_SBO);
                const uint64_t dbl = sdesc(bl + j * 2 * B_LBO, B_LBO, B_SBO);
#pragma unroll
                for (int qb = 0; qb < NB; ++qb) {
                    const uint32_t ah = smem_u32(S.a[sa][qb][0]), al = smem_u32(S.a[sa][qb][1]);
                    const uint64_t dah = sdesc(ah + j * 2 * A_LBO, A_LBO, A_SBO);
                    const uint64_t dal = sdesc(al + j * 2 * A_LBO, A_LBO, A_SBO);
                    const uint32_t d = tmem + set + (uint32_t)(qb * N);
                    mma_bf16(d, dah, dbh, IDESC, (first && j == 0) ? 0u : 1u);
                    mma_bf16(d, dah, dbl, IDESC, 1u);
                    mma_bf16(d, dal, dbh, IDESC, 1u);
                }
            }
            mma_commit(&S.a_empty[sa]);
            mma_commit(&S.b_empty[sb]);
            if ((i % DRAIN) == DRAIN - 1 || i == nk - 1) mma_commit(&S.acc_full[g & 1]);
        }
    }
    if (!ok) atomicOr(err, KERR_MBAR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TCOLS);
}

// ecg[s][l][t] (l < nmove) = sum_c partial[c][s*nmove + l][t]; block per (row, 32 steps)
__global__ void k_reduce_rows(int steps, int rows, int nchunks, int nmove, int nleads, const double *__restrict__ partial,
                              const double *__restrict__ k0w, double *__restrict__ ecg) {
    __shared__ double red[8][33];
    const int tt = blockIdx.x * 32 + (threadIdx.x & 31);
    const int w = threadIdx.x >> 5;
    const int r = blockIdx.y;
    const int s = r / nmove, l = r % nmove;
    double acc = 0.0;
    if (tt < steps)
        for (int c = w; c < nchunks; c += 8) acc += partial[((size_t)c * rows + r) * steps + tt];
    red[w][threadIdx.x & 31] = acc;
    __syncthreads();
    if (w == 0 && tt < steps) {
        double v = k0w ? k0w[(size_t)s * nleads + l] : 0.0;
        for (int i = 0; i < 8; ++i) v += red[i][threadIdx.x];
        ecg[((size_t)s * nleads + l) * steps + tt] = v;
    }
}

template <int NB, int N>
void launch_gemm(cudaStream_t st, const BatchArgs &A) {
    const size_t smem = sizeof(BatchSmem<NB, N>) + 1024;
    static bool attr = false;
    if (!attr) {
        EKG_CUDA(cudaFuncSetAttribute(k_batch_umma<NB, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    dim3 grid((unsigned)((A.steps + BM - 1) / BM), (unsigned)A.ntiles, (unsigned)A.nchunks);
    k_batch_umma<NB, N><<<grid, WS_THREADS, smem, st>>>(A.steps, A.nl, A.nkt, A.rows, A.nmove, A.n_sims, A.t_hilo,
                                                        A.at_hilo, A.ck0, A.ck1, A.cl, A.hconst, A.k3, A.F, A.Bt,
                                                        A.partial, A.err);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace

int batch_tile_rows(int two_bases) { return two_bases ? 128 : 256; }

void launch_taylor_w(cudaStream_t s, const HeartDev &h, const float *W0, int J, const double *centre,
                     const double *scale, float *Wt) {
    dim3 grid((unsigned)((h.apad + 255) / 256), (unsigned)h.nleads);
    k_taylor_w<<<grid, 256, 0, s>>>(h.apad, h.nleads, J, W0, h.at.p, h.a_layer.p, centre, scale, Wt);
    EKG_CUDA(cudaGetLastError());
}

void launch_reduce_layers(cudaStream_t s, int steps, int rows, int nl, const int32_t *lc0, const int32_t *lc1,
                          const double *partial, double *Q) {
    dim3 grid((unsigned)((steps + 31) / 32), (unsigned)rows);
    k_reduce_layers<<<grid, 256, 0, s>>>(steps, rows, nl, lc0, lc1, partial, Q);
    EKG_CUDA(cudaGetLastError());
}

void launch_static_combine(cudaStream_t s, const HeartDev &h, int J, int Jb, int nmove, int n_sims, const double *F,
                           const double *coef, const double *k3, const double *Q1, const double *Q2, double *ecg) {
    if (nmove >= h.nleads) return;
    dim3 grid((unsigned)((h.steps + 127) / 128), (unsigned)(h.nleads - nmove), (unsigned)n_sims);
    k_static_combine<<<grid, 128, 0, s>>>(h.steps, h.nleads, h.nlayers, J, Jb, nmove, n_sims, F, coef, k3, Q1, Q2,
                                          ecg);
    EKG_CUDA(cudaGetLastError());
}

void launch_batch_lead_field(cudaStream_t s, const HeartDev &h, int two_bases, const double *layer_k,
                             const double *leads, int nmove, int n_sims, uint8_t *Bt) {
    const int threads = n_sims < 128 ? ((n_sims + 31) / 32) * 32 : 128;
    dim3 grid((unsigned)(h.apad / 8), (unsigned)((n_sims + threads - 1) / threads));
    const int nkt = (int)(h.apad / BKT);
    const bool diag = h.nhood == EKG_NHOOD_3D4;
#define EKG_LF(NN, DG)                                                                                           \
    k_batch_lead_field<NN, DG><<<grid, threads, 0, s>>>(h.apad, nkt, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p, \
                                                        h.nnb, h.difs.p, h.at.p, h.a_layer.p, layer_k, h.nlayers,  \
                                                        leads, h.centre[0], h.centre[1], h.centre[2], h.nleads,    \
                                                        nmove, n_sims, Bt)
    if (two_bases) {
        if (diag) EKG_LF(128, true);
        else EKG_LF(128, false);
    } else {
        if (diag) EKG_LF(256, true);
        else EKG_LF(256, false);
    }
#undef EKG_LF
    EKG_CUDA(cudaGetLastError());
}

void launch_batch_gemm(cudaStream_t s, const BatchArgs &A) {
    if (A.two_bases) launch_gemm<2, 128>(s, A);
    else launch_gemm<1, 256>(s, A);
}

void launch_reduce_rows(cudaStream_t s, int steps, int rows_used, int rows, int nchunks, int nmove, int nleads,
                        const double *partial, const double *k0w, double *ecg) {
    dim3 grid((unsigned)((steps + 31) / 32), (unsigned)rows_used);
    k_reduce_rows<<<grid, 256, 0, s>>>(steps, rows, nchunks, nmove, nleads, partial, k0w, ecg);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace ekg
