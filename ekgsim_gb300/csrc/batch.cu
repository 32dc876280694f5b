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
// * Moved leads (lead genes): Y_b[(s,l), t] = sum_{a in L} W'_s[l,a] B_b,a(t), W'_s = W_s exp(k5_s at_a).
//   sigma(k1 tau) is 1 to within 2^-30 for tau > T+ = 30 ln2 / k1, and B_b,a(t) is below 2^-30
//   for tau < -T- = -30 ln2 / (k1 - k4).  Outside the band |tau| <~ T the bases are exactly
//       B1 -> exp(-k4 tau),  B2 -> 1   (tau > T+),      B1, B2 -> 0   (tau < -T-),
//   so for a tile of 128 steps starting at t0 the APs split (they are sorted by at within a
//   layer) into a steady prefix (at < t0 - T+), a band, and a suffix that does not contribute:
//       Y_b(t) = band GEMM + [B1: exp(-k4 (t - t0)) U1, B2: U0],
//       U1 = sum_{steady a} W' exp(-k4 (t0 - at_a)),   U0 = sum_{steady a} W'.
//   The band GEMM runs on the tensor cores with M = 128 steps, N = 256 (or 128) rows
//   (simulation, moved lead), K = the band's APs of one layer.  The B operand W' is written per
//   batch in BF16 hi+lo, already tiled in the UMMA canonical layout, and streamed into shared
//   memory with 1-D bulk copies (TMA engine, mbarrier tx counts); the A operand B_b,a(t) is
//   evaluated by 256 producer threads in FP32 per K stage.  The epilogue forms
//   ((1-k3) Y1 + k3 Y2) F_L(t) per row in FP64.  With a batch-uniform k3 the two bases collapse
//   into one (N = 256, three MMAs per K step instead of six).  The steady sums U0, U1 come from
//   per-8-AP partial sums the operand kernel writes in FP32 (k_band_u), and the reduction adds
//   F_L(t) [(1-k3) exp(-k4 (t - t0)) U1 + k3 U0] per layer.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>

#include "ekg_internal.h"
#include "umma_ptx.h"

namespace ekg {

using namespace ptx;

namespace {

constexpr int BM = 128, BKT = 64;
constexpr int LF_THREADS = 128;  // threads of the moved-lead operand kernel

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
// 1/sqrt(x) for normal x (squared distances >= 1 here), one MUFU operation
__device__ __forceinline__ float rsqa(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
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
// contiguous, [lc0[L], lc1[L])), summed in FP64 and stored in FP32; block per (row, 32 steps),
// warps split chunks, fixed order.
__global__ void k_reduce_layers(int steps, int rows, int nl, const int32_t *__restrict__ lc0,
                                const int32_t *__restrict__ lc1, const double *__restrict__ partial,
                                float *__restrict__ Q) {
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
            Q[((size_t)L * rows + row) * steps + tt] = (float)r;
        }
        __syncthreads();
    }
}

// Static leads: ecg[s][l][t] = sum_L F[s][L][t] sum_j coef[s][L][j] ((1-k3) Q1 + k3 Q2)[L][l*J+j][t],
// coef[s][L][j] = exp(k5 c_L) (k5 s_L)^j / j! (k5 of the simulation's layer AP, c_L and s_L the
// centre and half-range of the layer's activation times; from k_layer_factors), the Taylor sum
// per layer in FP32 (the basis is stored in FP32), the sum over layers in float-float; written as
// FP64 and as float-float.  Block = 128 steps of one static lead for SC_SIMS simulations: a
// thread loads the basis rows of its step once per layer and applies them to every simulation of
// the group (coefficients broadcast from shared memory).
constexpr int SC_SIMS = 16;
__global__ void __launch_bounds__(128) k_static_combine(int steps, int nleads, int nl, int J, int Jb, int nmove,
                                                        int n_sims, const float *__restrict__ F,
                                                        const float *__restrict__ coef, const double *__restrict__ k3,
                                                        const float *__restrict__ Q1, const float *__restrict__ Q2,
                                                        double *__restrict__ ecg, float2 *__restrict__ ecg_ff,
                                                        const double *__restrict__ cst) {
    __shared__ float s_c[SC_SIMS][11];  // [simulation][j < J: coefficient, 10: k3] of the current layer
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = nmove + blockIdx.y, s0 = blockIdx.z * SC_SIMS;
    const int ns = min(SC_SIMS, n_sims - s0);
    const bool on = t < steps;
    const int tc = on ? t : steps - 1;
    const int rows = nleads * Jb;  // the basis stores Jb terms per lead
    float2 acc[SC_SIMS];
#pragma unroll
    for (int i = 0; i < SC_SIMS; ++i) acc[i] = make_float2(0.f, 0.f);
    for (int L = 0; L < nl; ++L) {
        __syncthreads();
        for (int k = threadIdx.x; k < ns * 11; k += blockDim.x) {
            const int i = k / 11, j = k % 11;
            const size_t sl = (size_t)(s0 + i) * nl + L;
            s_c[i][j] = j < J ? coef[sl * J + j] : (j == 10 ? (float)k3[sl] : 0.f);
        }
        __syncthreads();
        const size_t q0 = ((size_t)L * rows + (size_t)l * Jb) * steps + tc;
        float q1[10], q2[10];
#pragma unroll
        for (int j = 0; j < 10; ++j) {  // J <= 10 (the basis order)
            q1[j] = j < J ? Q1[q0 + (size_t)j * steps] : 0.f;
            q2[j] = j < J ? Q2[q0 + (size_t)j * steps] : 0.f;
        }
#pragma unroll
        for (int i = 0; i < SC_SIMS; ++i)
            if (i < ns) {
                float v1 = 0.f, v2 = 0.f;
#pragma unroll
                for (int j = 0; j < 10; ++j)
                    if (j < J) {
                        v1 = fmaf(s_c[i][j], q1[j], v1);
                        v2 = fmaf(s_c[i][j], q2[j], v2);
                    }
                acc[i] = ff_add_f(acc[i], F[((size_t)(s0 + i) * nl + L) * steps + tc] * fmaf(s_c[i][10], v2 - v1, v1));
            }
    }
    if (!on) return;
#pragma unroll
    for (int i = 0; i < SC_SIMS; ++i)
        if (i < ns) {
            const size_t o = ((size_t)(s0 + i) * nleads + l) * steps + t;
            if (cst) acc[i] = ff_add(acc[i], ff_from_double(cst[(size_t)(s0 + i) * nleads + l]));
            ecg[o] = ff_to_double(acc[i]);
            ecg_ff[o] = acc[i];
        }
}

// ------------------------------------------------------------------ moved-lead operand
// W'_s[l][a] for the moved leads l < nmove, written as BF16 hi/lo into the tiled B layout:
// [N tile][K tile][part hi/lo][N*128 bytes], element (row n, k) of a tile at byte
// ((k/8) * (N/8) + n/8) * 128 + (n%8) * 16 + (k%8) * 2.
// Block = up to 128 simulations (one per thread) x one segment of 8-AP chunks; per chunk the voxel
// data is a broadcast load for the warp (and every branch on it is warp-uniform) and each thread
// writes one 16-byte row segment per part; a warp's 32 simulations x nmove rows are contiguous
// in the tile.
// The field at p = v + d uses |m - d|^2 = |m|^2 - 2 m.d + |d|^2 with m = r - v, and
// g.d = (m.d - |d|^2) |m - d|^-3: one rsqrt and a few FMAs per neighbour.
//
// Interior voxels (every neighbour present, out-neighbour offsets summing to zero):
// w(v) = sum_n d_n . grad phi(v + d_n)
// with phi(v) = 1/|r - v| harmonic, so by Taylor expansion in d_n
//     w = sum_{k odd} (1/k!) sum_n (d_n . grad)^(k+1) phi(v),
// whose k = 1 term is (sum_n d_x^2) lap phi = 0.  For a neighbour set with the symmetry of the cube
// the k = 3 and k = 5 terms reduce, with lap phi = 0, to
//     f4 sum_i d_i^4 phi + f6 sum_i d_i^6 phi,
//     sum_i d_i^4 phi = rho^5 (105 T4 - 63),   sum_i d_i^6 phi = rho^7 (4050 - 14175 T4 + 10395 T6),
// rho = 1/|m|, T4 = sum_i (m_i rho)^4, T6 = sum_i (m_i rho)^6 (f4, f6 from the set's 4th and 6th
// moments, computed on the host; the 8 body diagonals give 168 - 280 T4 and 4320 - 15120 T4 +
// 11088 T6).  The next term is smaller by about 20/|m|^2; the form is used for |m| >= 20, where it
// is closer to the exact sum than the FP32 evaluation of the eight cancelling neighbour terms.
// Evaluated through the symmetric functions of the squares a, b, c of m's components:
// s = a + b + c, P = ab + bc + ca, Q = abc, so that T4 = 1 - 2 P/s^2 and T6 = 1 - 3 P/s^2 + 3 Q/s^3;
// with u = 1/s = rho^2 the field is
//     w = rho u^2 [(A0 + u B0) + u^2 (P (A1 + u B1) + u^2 B2 Q)],
// A0 = a0 + a1, A1 = -2 a1, B0 = b0 + b1 + b2, B1 = -3 b2 - 2 b1, B2 = 3 b2 for the coefficients
// of rho^5 (a1 T4 + a0) + rho^7 (b2 T6 + b1 T4 + b0) (about 20 FP32 operations and one rsqrt).
struct InteriorField {
    float A0 = 0, A1 = 0, B0 = 0, B1 = 0, B2 = 0;
};
// Flag bits above the neighbour mask in vox_pos.w (the mask uses at most 26 bits).
constexpr uint32_t VOX_INTERIOR = 1u << 31;  // every neighbour present, out-neighbour offsets sum to 0
constexpr uint32_t VOX_AP_END = 1u << 30;    // last voxel of its AP (voxels are grouped by AP)
constexpr uint32_t VOX_FEW = 1u << 29;       // not interior, few neighbours absent (closed form minus them)

// closed form of the interior field for m = r - v, used where |m|^2 >= INTERIOR_S_MIN for every lead
// of the lane (a lead displaced towards the heart takes the exact sum for the voxels near it)
constexpr float INTERIOR_S_MIN = 400.f;
struct MSquares {
    float a, b, c, h, s;  // squares of m's components, h = a + b, s = h + c = |m|^2
};
__device__ __forceinline__ MSquares msq(float4 pos, float4 r) {
    const float mz = r.x - pos.x, my = r.y - pos.y, mx = r.z - pos.z;
    MSquares q;
    q.a = mz * mz;
    q.b = my * my;
    q.c = mx * mx;
    q.h = q.a + q.b;
    q.s = q.h + q.c;
    return q;
}
__device__ __forceinline__ float interior_w(const InteriorField &ic, const MSquares &q, float rho) {
    const float u = rho * rho, u2 = u * u;
    const float ab = q.a * q.b;
    const float P = fmaf(q.c, q.h, ab), Q = ab * q.c;
    const float c1 = fmaf(u, ic.B0, ic.A0), c2 = fmaf(u, ic.B1, ic.A1);
    const float inner = fmaf(P, c2, Q * (ic.B2 * u2));
    return (rho * u2) * fmaf(u2, inner, c1);
}

// w(v) for one lead position r relative to the same centre as the voxel positions, general
// neighbourhood, every term evaluated.
__device__ __forceinline__ float voxel_w_general(float4 pos, uint32_t mi, float4 out, float4 r, int nnb,
                                                 const float *s_d) {
    const float mz = r.x - pos.x, my = r.y - pos.y, mx = r.z - pos.z;
    const float s0 = fmaf(mz, mz, fmaf(my, my, mx * mx));
    float w = 0.f;
    for (int n = 0; n < nnb; ++n) {
        if (!(mi & (1u << n))) continue;
        const float4 d = reinterpret_cast<const float4 *>(s_d)[n];
        const float y = fmaf(mz, d.x, fmaf(my, d.y, mx * d.z)) - d.w;  // m.d - |d|^2
        const float rs = rsqa(fmaf(-2.f, y, s0 - d.w));                // |m - d|^2 = |m|^2 - |d|^2 - 2 y
        w = fmaf(rs * rs * rs, y, w);
    }
    if (out.w != 0.f) {
        const float rs = rsqa(s0);
        w = fmaf(-(rs * rs * rs), fmaf(mz, out.x, fmaf(my, out.y, mx * out.z)), w);
    }
    return w;
}

// Same for the 8 body diagonals ("3D4", creation order (-1,-1,-1) ... (1,1,1), |d|^2 = 3): with
// p = my + mx, q = my - mx, zm = -mz - 3, zp = mz - 3 the eight y = m.d - 3 are
// zm-p, zm-q, zm+q, zm+p, zp-p, zp-q, zp+q, zp+p, and |m - d|^2 = (|m|^2 - 3) - 2 y.  Missing
// neighbours are masked, the out-neighbour term is skipped where there is none (every test on
// the voxel is uniform over the warp).
__device__ __forceinline__ float voxel_w_diag(float4 pos, uint32_t mi, float4 out, float4 r) {
    const float mz = r.x - pos.x, my = r.y - pos.y, mx = r.z - pos.z;
    const float s0 = fmaf(mz, mz, fmaf(my, my, mx * mx));
    const float b = s0 - 3.f;
    const float p = my + mx, q = my - mx;
    const float zm = -mz - 3.f, zp = mz - 3.f;
    const float y[8] = {zm - p, zm - q, zm + q, zm + p, zp - p, zp - q, zp + q, zp + p};
    float w = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float rs = rsqa(fmaf(-2.f, y[n], b));
        if ((mi >> n) & 1u) w = fmaf(rs * rs * rs, y[n], w);
    }
    if (out.w != 0.f) {
        const float rs0 = rsqa(s0);
        w = fmaf(-(rs0 * rs0 * rs0), fmaf(mz, out.x, fmaf(my, out.y, mx * out.z)), w);
    }
    return w;
}

// A voxel flagged VOX_FEW with the lane's leads at least 20 cells away: the field of the full set
// (closed form) minus the terms of the absent neighbours `miss`, minus the out-neighbour term,
//     w = W_full(m) - sum_{n in miss} y_n |m - d_n|^-3 - |m|^-3 m.out,
// one rsqrt per absent neighbour instead of one per present one.  The loop over the absent
// neighbours is uniform over the warp (one voxel per warp), shared by the NP lead positions.
template <int NP>
__device__ __forceinline__ void few_w(const InteriorField &ic, const MSquares (&q)[NP], float4 pos,
                                      const float4 (&r)[NP], uint32_t miss, float4 out, const float *s_d,
                                      float (&acc)[NP]) {
    float mz[NP], my[NP], mx[NP], rho[NP], w[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        mz[k] = r[k].x - pos.x;
        my[k] = r[k].y - pos.y;
        mx[k] = r[k].z - pos.z;
        rho[k] = rsqa(q[k].s);
        w[k] = interior_w(ic, q[k], rho[k]);
    }
    for (; miss; miss &= miss - 1) {
        const float4 d = reinterpret_cast<const float4 *>(s_d)[__ffs(miss) - 1];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const float y = fmaf(mz[k], d.x, fmaf(my[k], d.y, mx[k] * d.z)) - d.w;
            const float rs = rsqa(fmaf(-2.f, y, q[k].s - d.w));
            w[k] = fmaf(-(rs * rs * rs), y, w[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        if (out.w != 0.f)
            w[k] = fmaf(-(rho[k] * rho[k] * rho[k]), fmaf(mz[k], out.x, fmaf(my[k], out.y, mx[k] * out.z)), w[k]);
        acc[k] += w[k];
    }
}

// sum_{v in a} w(v) for the 8 APs of a chunk (voxel records [vb, vend) of vox_pos / vox_out, in
// shared or global memory) and NP lead positions, into s_w[k][j][tid]: one flat loop over the
// chunk's voxels (grouped by AP, the last one of each AP flagged); APs without
// voxels (padding, at the end of a layer) get 0.  Interior voxels use the closed form where the
// lane's leads are at least 20 cells away (lanes normally agree), boundary voxels with few absent
// neighbours the closed form minus those, the rest the exact sum.
// ALLFAR: every voxel of the chunk is known to be far from the lane's leads (the stage's bounding
// box is), so the per-voxel distance test is skipped.
template <bool DIAG, int NP, bool ALLFAR = false>
__device__ __forceinline__ void chunk_w(int vb, int vend, const float4 *vox_pos, const float4 *vox_out,
                                        const float4 (&r)[NP], int nnb, const float *s_d, const InteriorField &ic,
                                        float (*s_w)[8][LF_THREADS], int tid) {
    const uint32_t full = (1u << nnb) - 1u;
    float acc[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = 0.f;
    int j = 0;
    for (int v = vb; v < vend; ++v) {
        const float4 pos = vox_pos[v];
        const uint32_t mi = __float_as_uint(pos.w);
        MSquares q[NP];
        bool far = true;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            q[k] = msq(pos, r[k]);
            if (!ALLFAR) far = far && q[k].s >= INTERIOR_S_MIN;
        }
        if ((mi & VOX_INTERIOR) && far) {
#pragma unroll
            for (int k = 0; k < NP; ++k) acc[k] += interior_w(ic, q[k], rsqa(q[k].s));
        } else if ((mi & VOX_FEW) && far) {
            few_w<NP>(ic, q, pos, r, full & ~mi, vox_out[v], s_d, acc);
        } else {
            const float4 out = vox_out[v];
#pragma unroll
            for (int k = 0; k < NP; ++k)
                acc[k] += DIAG ? voxel_w_diag(pos, mi, out, r[k]) : voxel_w_general(pos, mi, out, r[k], nnb, s_d);
        }
        if (mi & VOX_AP_END) {
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                s_w[k][j][tid] = acc[k];
                acc[k] = 0.f;
            }
            ++j;
        }
    }
    for (; j < 8; ++j)
#pragma unroll
        for (int k = 0; k < NP; ++k) s_w[k][j][tid] = 0.f;
}

// Work items: (32-AP stage st, group of LF_THREADS * LF_ROWS rows), taken from the counter `work`
// (zeroed before the launch) by a grid of one wave of resident blocks, stages in `stage_order`
// (descending voxel count, so that the last items are short); every item writes its own
// outputs, so the results do not depend on the order.  A thread owns LF_ROWS consecutive rows
// (row = s * nmove + l) and evaluates their lead positions together, so the voxel loads and tests
// are shared by LF_ROWS field evaluations.  Per item and row the thread writes the BF16 hi/lo tile
// row segments and, for the steady part, the stage's sums
//     P1[st][row'] = (sum_a W'[a], sum_a W'[a] exp(-k4 (T_st - at_a))) over the stage's APs,
// T_st = tref[st] = the stage's last finite activation time (APs ascend within a layer, so every
// factor is <= 1), row' = l * S + s.  k_band_u scales the second sum by each entry's
// G_e[st] = exp(-k4 (t0_e - T_st)) and adds the stages of a layer in a fixed order.
// lrel: [S][nmove] lead positions relative to the voxel centre (FP32, differences taken in FP64
// on the host); k5l: [S][nl] k5 * log2(e).
constexpr int MAXE = 8;
constexpr int BST = 32;     // APs per stage
constexpr int LF_ROWS = 4;  // rows per thread
constexpr int LF_VCAP = 256;  // voxel records of a stage staged in shared memory
static_assert(LF_THREADS >= BST + BST / 8 + 1, "the stage tables are loaded one entry per thread");
template <bool DIAG, int ROWS, bool SPLIT, bool K0>
__global__ void __launch_bounds__(LF_THREADS, 8) k_batch_lead_field(
    int nlog, int nst, int ngr, int ksplit_arg, int *__restrict__ work, InteriorField ic, const int64_t *__restrict__ a_vox_begin,
    const float4 *__restrict__ vox_pos, const float4 *__restrict__ vox_out, int nnb, const int8_t *__restrict__ difs,
    const float2 *__restrict__ at_hilo, const int32_t *__restrict__ a_layer, const float *__restrict__ k5l, int nl,
    const float4 *__restrict__ hconst, const float4 *__restrict__ lrel, int nmove, int n_sims,
    const float2 *__restrict__ tref, const int32_t *__restrict__ nent, const int32_t *__restrict__ esplit,
    const int32_t *__restrict__ stage_order, const float4 *__restrict__ stage_box, uint8_t *__restrict__ Bt,
    float2 *__restrict__ P1, float *__restrict__ P2) {
    __shared__ float s_d[26 * 4];
    __shared__ float s_w[LF_ROWS][8][LF_THREADS];
    __shared__ float2 s_at[BST];  // the stage's activation times
    __shared__ float s_ez[BST];   // exp(-k4 (T_st - at)), 0 for padding
    __shared__ int s_vb[BST / 8 + 1];  // first voxel of each chunk of the stage, and the end
    __shared__ float4 s_vpos[LF_VCAP], s_vout[LF_VCAP];  // the stage's voxel records, when they fit
    __shared__ int s_item;
    const int tid = threadIdx.x;
    if (tid < nnb) {
        const float dz = difs[3 * tid], dy = difs[3 * tid + 1], dx = difs[3 * tid + 2];
        s_d[4 * tid] = dz;
        s_d[4 * tid + 1] = dy;
        s_d[4 * tid + 2] = dx;
        s_d[4 * tid + 3] = dz * dz + dy * dy + dx * dx;
    }
    const int rows_used = n_sims * nmove;
    const int nkt = nst / 2;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(work, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= nst * ngr) break;
        const int st = stage_order[item / ngr];  // stages with the most voxels first
        const int L = a_layer[(int64_t)st * BST];
        // the stage's voxel records are copied to shared memory once per item (a stage of up to
        // LF_VCAP voxels; larger ones read global memory), so the voxel loop waits on no global load
        const int v0 = (int)a_vox_begin[(int64_t)st * BST], nv = (int)a_vox_begin[(int64_t)(st + 1) * BST] - v0;
        const bool staged = nv <= LF_VCAP;
        if (staged)
            for (int i = tid; i < nv; i += LF_THREADS) {
                s_vpos[i] = vox_pos[v0 + i];
                s_vout[i] = vox_out[v0 + i];
            }
        if (tid < BST) {
            const float2 at = at_hilo[(int64_t)st * BST + tid], T = tref[st];
            s_at[tid] = at;
            s_ez[tid] = isinf(at.x) ? 0.f : ex2a(-hconst[L].y * ((T.x - at.x) + (T.y - at.y)));
        } else if (tid < BST + BST / 8 + 1) {
            s_vb[tid - BST] = (int)a_vox_begin[(int64_t)st * BST + (tid - BST) * 8] - (staged ? v0 : 0);
        }
        __syncthreads();
        const float4 *vp = staged ? s_vpos : vox_pos, *vo = staged ? s_vout : vox_out;
        // with fewer rows than threads x ROWS the warps split the stage's four 8-AP chunks:
        // ksplit groups of LF_THREADS / ksplit threads over the same rows, group g taking chunks
        // g, g + ksplit, ...
        const int ksplit = SPLIT ? ksplit_arg : 1;  // the unsplit instance compiles without the split
        const int gthreads = LF_THREADS / ksplit, kg = tid / gthreads;
        const int rb = (item % ngr) * (gthreads * ROWS) + (tid % gthreads) * ROWS;
        const bool active = rb < rows_used;  // every thread stays for the barriers below
        // whether every voxel of the stage is far from every lead of the warp (squared distance from
        // the lead to the stage's bounding box; a margin of one cell over the closed form's bound)
        bool far_all = true;
        if (active) {
            const float4 lo = stage_box[2 * (size_t)st], hi = stage_box[2 * (size_t)st + 1];
            const int nr0 = min(ROWS, rows_used - rb);
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                if (q >= nr0) break;
                const float4 r = lrel[rb + q];
                const float dz = fmaxf(fmaxf(lo.x - r.x, r.x - hi.x), 0.f);
                const float dy = fmaxf(fmaxf(lo.y - r.y, r.y - hi.y), 0.f);
                const float dx = fmaxf(fmaxf(lo.z - r.z, r.z - hi.z), 0.f);
                far_all = far_all && dz * dz + dy * dy + dx * dx >= INTERIOR_S_MIN + 41.f;
            }
        }
        far_all = __all_sync(0xffffffffu, far_all);
        const int nr = active ? min(ROWS, rows_used - rb) : 0;  // rows of this thread; the rest repeat its last row
        float k5[ROWS], S0[ROWS], S1[ROWS];
#pragma unroll
        for (int q = 0; q < ROWS; ++q) {
            const int row = active ? rb + min(q, nr - 1) : 0;
            k5[q] = k5l[(size_t)(row / nmove) * nl + L];
            S0[q] = S1[q] = 0.f;
        }
        const int kt = st >> 1;
#pragma unroll 1
        for (int kc = active ? kg : BST / 8; kc < BST / 8; kc += ksplit) {
            {
                float4 r[ROWS];
#pragma unroll
                for (int q = 0; q < ROWS; ++q) r[q] = lrel[rb + min(q, nr - 1)];
                if (far_all) chunk_w<DIAG, ROWS, true>(s_vb[kc], s_vb[kc + 1], vp, vo, r, nnb, s_d, ic, s_w, tid);
                else chunk_w<DIAG, ROWS, false>(s_vb[kc], s_vb[kc + 1], vp, vo, r, nnb, s_d, ic, s_w, tid);
            }
            const int col = (st & 1) * (BST / 8) + kc;  // 8-AP column within the 64-AP tile
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                if (q >= nr) break;
                float wv[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float2 at = s_at[kc * 8 + j];
                    wv[j] = isinf(at.x) ? 0.f : s_w[q][j][tid] * ex2a(fmaf(k5[q], at.x, k5[q] * at.y));
                }
                uint4 hv, lv;
                split2(wv[0], wv[1], hv.x, lv.x);
                split2(wv[2], wv[3], hv.y, lv.y);
                split2(wv[4], wv[5], hv.z, lv.z);
                split2(wv[6], wv[7], hv.w, lv.w);
                const int row = rb + q;
                const int nt = row >> nlog, n = row & ((1 << nlog) - 1);
                const size_t tile = ((size_t)nt * nkt + kt) * 2;
                const size_t off = ((size_t)(col << (nlog - 3)) + n / 8) * 128 + (n % 8) * 16;
                *reinterpret_cast<uint4 *>(Bt + (tile << (nlog + 7)) + off) = hv;
                *reinterpret_cast<uint4 *>(Bt + ((tile + 1) << (nlog + 7)) + off) = lv;
                float z0 = 0.f, z1 = 0.f;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    z0 += wv[j];
                    z1 = fmaf(wv[j], s_ez[kc * 8 + j], z1);
                }
                S0[q] += z0;
                S1[q] += z1;
                if (K0 && P2) {
                    // the unscaled field sums of the 8 APs (the resting-potential term, k_k0_moved)
                    float z2 = 0.f;
#pragma unroll
                    for (int j = 0; j < 8; ++j) z2 += s_w[q][j][tid];
                    const int s = row / nmove, l = row % nmove;
                    P2[((size_t)st * 4 + kc) * rows_used + (size_t)l * n_sims + s] = z2;
                }
            }
        }
        const int ne = nent[L];
        const bool steady = ne > 0 && st < esplit[L * MAXE + ne - 1];  // the last entry's steady prefix is the longest
        if (SPLIT && steady && ksplit > 1) {
            // the other groups hand their steady sums to group 0 through the staging area (free once
            // every group is past the voxel loop), added in group order
            float2 *s_p1 = reinterpret_cast<float2 *>(s_vpos);  // [LF_THREADS][ROWS]
            __syncthreads();
            if (kg > 0 && active)
#pragma unroll
                for (int q = 0; q < ROWS; ++q) s_p1[tid * ROWS + q] = make_float2(S0[q], S1[q]);
            __syncthreads();
            if (kg == 0 && active)
                for (int g = 1; g < ksplit; ++g)
#pragma unroll
                    for (int q = 0; q < ROWS; ++q) {
                        const float2 v = s_p1[(g * gthreads + tid) * ROWS + q];
                        S0[q] += v.x;
                        S1[q] += v.y;
                    }
        }
        if (steady && kg == 0 && active)
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                if (q >= nr) break;
                const int row = rb + q, s = row / nmove, l = row % nmove;
                P1[(size_t)st * rows_used + (size_t)l * n_sims + s] = make_float2(S0[q], S1[q]);
            }
    }
}

// Small batches (up to SMALL_SIMS simulations; above that the persistent kernel with one row per
// thread is faster, measured at 160^3: 6 simulations 0.119 against 0.132 ms per pass, 16
// simulations 0.128 against 0.237): one thread per (AP, simulation), so the work spreads
// over the heart instead of over simulations.  A block is four 32-AP stages of one simulation, one
// per warp; eight consecutive lanes are one 8-AP chunk and write its BF16 hi/lo row segment two
// bytes each.  The steady sums of a stage are reduced by a shuffle butterfly within its warp.
// Same outputs as k_batch_lead_field.
constexpr int SMALL_SIMS = 4;
template <int N, bool DIAG>
__global__ void __launch_bounds__(128) k_batch_lead_field_small(
    int nst, InteriorField ic, const int64_t *__restrict__ a_vox_begin, const float4 *__restrict__ vox_pos,
    const float4 *__restrict__ vox_out, int nnb, const int8_t *__restrict__ difs, const float2 *__restrict__ at_hilo,
    const int32_t *__restrict__ a_layer, const float *__restrict__ k5l, int nl, const float4 *__restrict__ hconst,
    const float4 *__restrict__ lrel, int nmove, int n_sims, const float2 *__restrict__ tref,
    const int32_t *__restrict__ nent, const int32_t *__restrict__ esplit, uint8_t *__restrict__ Bt,
    float2 *__restrict__ P1, float *__restrict__ P2) {
    __shared__ float s_d[26 * 4];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < nnb) {
        const float dz = difs[3 * tid], dy = difs[3 * tid + 1], dx = difs[3 * tid + 2];
        s_d[4 * tid] = dz;
        s_d[4 * tid + 1] = dy;
        s_d[4 * tid + 2] = dx;
        s_d[4 * tid + 3] = dz * dz + dy * dy + dx * dx;
    }
    __syncthreads();
    const int64_t apad = (int64_t)nst * BST;
    const int64_t araw = (int64_t)blockIdx.x * 128 + tid;
    const bool valid = araw < apad;  // whole stages are in or out (apad is a multiple of 64)
    const int64_t a = valid ? araw : apad - 1;
    const int s = blockIdx.y;
    const int rows_used = n_sims * nmove;
    const int nkt = nst / 2;
    const int kt = (int)(a / BKT), k = (int)(a % BKT), st = (int)(a / BST);
    const int L = a_layer[a];
    const float k5 = k5l[(size_t)s * nl + L], k4 = hconst[L].y;
    const int ne = nent[L];
    const float2 at = at_hilo[a], T = tref[st];
    const bool pad = isinf(at.x);
    const float e = pad ? 0.f : ex2a(fmaf(k5, at.x, k5 * at.y));
    const float ez = pad ? 0.f : ex2a(-k4 * ((T.x - at.x) + (T.y - at.y)));
    const int vb = (int)a_vox_begin[a], ve = (int)a_vox_begin[a + 1];
    for (int l0 = 0; l0 < nmove; l0 += 2) {
        const int np = l0 + 1 < nmove ? 2 : 1;
        const float4 r0 = lrel[(size_t)s * nmove + l0];
        const float4 r1 = np == 2 ? lrel[(size_t)s * nmove + l0 + 1] : r0;
        float acc0 = 0.f, acc1 = 0.f;
        if (valid)
            for (int v = vb; v < ve; ++v) {
                const float4 pos = vox_pos[v];
                const uint32_t mi = __float_as_uint(pos.w);
                const MSquares q0 = msq(pos, r0), q1 = msq(pos, r1);
                if ((mi & VOX_INTERIOR) && q0.s >= INTERIOR_S_MIN && q1.s >= INTERIOR_S_MIN) {
                    acc0 += interior_w(ic, q0, rsqa(q0.s));
                    if (np == 2) acc1 += interior_w(ic, q1, rsqa(q1.s));
                } else {
                    const float4 out = vox_out[v];
                    acc0 += DIAG ? voxel_w_diag(pos, mi, out, r0) : voxel_w_general(pos, mi, out, r0, nnb, s_d);
                    if (np == 2)
                        acc1 += DIAG ? voxel_w_diag(pos, mi, out, r1) : voxel_w_general(pos, mi, out, r1, nnb, s_d);
                }
            }
        if (P2 && valid) {
            // unscaled field sums per 8-AP part of the stage (the resting-potential term): the warp
            // is one stage, eight lanes one part
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                if (q >= np) break;
                float z = q ? acc1 : acc0;  // every AP, activated or not (padding slots hold no voxels)
                z += __shfl_xor_sync(0xffffffffu, z, 1);
                z += __shfl_xor_sync(0xffffffffu, z, 2);
                z += __shfl_xor_sync(0xffffffffu, z, 4);
                if ((lane & 7) == 0)
                    P2[((size_t)st * 4 + (lane >> 3)) * rows_used + (size_t)(l0 + q) * n_sims + s] = z;
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (q >= np) break;
            const float w = (q ? acc1 : acc0) * e;
            const __nv_bfloat16 hb = __float2bfloat16_rn(w);
            const __nv_bfloat16 lb = __float2bfloat16_rn(w - __bfloat162float(hb));
            const int row = s * nmove + l0 + q;
            if (valid) {
                const int nt = row / N, n = row % N;
                const size_t tile = ((size_t)nt * nkt + kt) * 2;
                const size_t off = (size_t)((k / 8) * (N / 8) + n / 8) * 128 + (n % 8) * 16 + (k % 8) * 2;
                *reinterpret_cast<__nv_bfloat16 *>(Bt + tile * (N * 128) + off) = hb;
                *reinterpret_cast<__nv_bfloat16 *>(Bt + (tile + 1) * (N * 128) + off) = lb;
            }
            // the warp is one stage of one layer: every test below is uniform over it
            if (valid && ne > 0 && st < esplit[L * MAXE + ne - 1]) {
                float x = w, y = w * ez;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    x += __shfl_xor_sync(0xffffffffu, x, o);
                    y += __shfl_xor_sync(0xffffffffu, y, o);
                }
                if (lane == 0) P1[(size_t)st * rows_used + (size_t)(l0 + q) * n_sims + s] = make_float2(x, y);
            }
        }
    }
}

// Steady sums per (row', layer, entry): U[row'][L][e] = sum over the layer's stages [ls0, ls1)
// below the entry's prefix end of (P1[st][row'].x, G_e[st] P1[st][row'].y) (U0, U1),
// G_e[st] = gtab[goff[L][e] + st - ls0[L]].  Two passes in a fixed order: k_band_u sums BU_PARTS
// consecutive parts of the stage range in FP32 (a few stages each), block per (part, 128 rows,
// layer), thread per row, all entries from one read of P1 (small blocks that fit beside the band
// GEMM's CTAs, which they run next to); k_band_u2 adds the parts in FP64, one warp per output.
// Up: [parts][rows][nl][max_ent]; U stored in FP32.  The prefix ends ascend with e.
constexpr int BU_PARTS = 128;
__global__ void __launch_bounds__(128, 8) k_band_u(int rows_used, int nl, int max_ent,
                                                   const int32_t *__restrict__ nent, const int32_t *__restrict__ esplit,
                                                   const int32_t *__restrict__ ls0, const int32_t *__restrict__ ls1,
                                                   const int64_t *__restrict__ goff, const float *__restrict__ gtab,
                                                   const float2 *__restrict__ P1, float2 *__restrict__ Up) {
    const int p = blockIdx.x, L = blockIdx.z;
    const int rr = blockIdx.y * blockDim.x + threadIdx.x;
    if (rr >= rows_used) return;
    const int ne = nent[L], n = ls1[L] - ls0[L];
    const int g0 = ls0[L] + (int)((int64_t)n * p / BU_PARTS), g1 = ls0[L] + (int)((int64_t)n * (p + 1) / BU_PARTS);
    int ge[MAXE];
    const float *gt[MAXE];  // entry e's factor of stage g: gt[e][g - g0]
#pragma unroll
    for (int e = 0; e < MAXE; ++e) {
        ge[e] = e < ne ? min(g1, esplit[L * MAXE + e]) : g0;
        gt[e] = gtab + (e < ne ? goff[L * MAXE + e] + (g0 - ls0[L]) : 0);
    }
    const int gend = ne > 0 ? ge[ne - 1] : g0;
    float a[MAXE], b[MAXE];
#pragma unroll
    for (int e = 0; e < MAXE; ++e) a[e] = b[e] = 0.f;
    for (int g = g0; g < gend; ++g) {
        const float2 v = P1[(size_t)g * rows_used + rr];
#pragma unroll
        for (int e = 0; e < MAXE; ++e)
            if (g < ge[e]) {
                a[e] += v.x;
                b[e] = fmaf(gt[e][g - g0], v.y, b[e]);
            }
    }
#pragma unroll
    for (int e = 0; e < MAXE; ++e)
        if (e < ne) Up[(((size_t)p * rows_used + rr) * nl + L) * max_ent + e] = make_float2(a[e], b[e]);
}

__global__ void __launch_bounds__(256) k_band_u2(int64_t n_out, const float2 *__restrict__ Up, float2 *__restrict__ U) {
    const int lane = threadIdx.x & 31;
    const int64_t i = blockIdx.x * 8 + (threadIdx.x >> 5);  // one warp per output
    if (i >= n_out) return;
    double a = 0.0, b = 0.0;
    for (int p = lane; p < BU_PARTS; p += 32) {
        const float2 v = Up[p * n_out + i];
        a += (double)v.x;
        b += (double)v.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) U[i] = make_float2((float)a, (float)b);
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
static_assert(SA <= SB, "producers read a stage's activation times from its B slot");
constexpr int WS_THREADS = 320;      // 8 producer warps + bulk-copy warp + MMA warp

template <int NB, int N>
struct BatchSmem {
    alignas(1024) uint8_t a[SA][NB][2][BM * WKT * 2];  // [stage][basis][hi/lo]
    alignas(1024) uint8_t b[SB][2][N * WKT * 2];       // [stage][hi/lo]
    alignas(16) float2 at[SB][WKT];                     // activation times of the stage's APs
    alignas(8) uint64_t a_full[SA], a_empty[SA], b_full[SB], b_empty[SB], acc_full[2], acc_empty[2];
    uint32_t tmem_base;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// grid (work items, N tiles).  Item c = (t tile, first stage, end stage, layer): the band of one
// 128-step tile inside one layer, in 32-AP stages.  partial: [items][rows][128] FP32 accumulators
// (float2 of the two bases with NB = 2).
template <int NB, int N>
__global__ void __launch_bounds__(WS_THREADS, (N <= 32 ? 2 : 1)) k_batch_umma(
    int steps, int nl, int nkt, int rows, int nmove, int n_sims, const float2 *__restrict__ t_hilo,
    const float2 *__restrict__ at_hilo, const int4 *__restrict__ items, const float4 *__restrict__ hconst,
    const uint8_t *__restrict__ Bt, float *__restrict__ partial, uint32_t *__restrict__ err) {
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
    const int c = blockIdx.x, nt = blockIdx.y;
    const int4 item = items[c];
    const int t0 = item.x * BM, st0 = item.y, nk = item.z - item.y, L = item.w;
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
            // the stage's activation times arrive with its B operand (the B slot is recycled only
            // after the MMAs of this stage, which wait for this production, and SA <= SB keeps
            // the wait within the slot's current phase)
            const int sb = i % SB;
            if (!mbar_wait(&S.b_full[sb], (uint32_t)((i / SB) & 1))) {
                ok = false;
                break;
            }
            const float2 *atp = S.at[sb] + half * 16;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int kc8 = half * 2 + j;
                float v1[8], v2[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float2 at = atp[j * 8 + e];
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
            // raw accumulators (both bases with NB = 2); the reduction applies F_L(t) and k3
            const int t = t0 + 32 * q + lane;
            if (t < steps) {
#pragma unroll
                for (int jj = 0; jj < HALF; ++jj) {
                    const int r = nt * N + ch * HALF + jj;
                    if (r / nmove >= n_sims) continue;
                    const size_t o = ((size_t)c * rows + r) * BM + (t - t0);
                    if (NB == 2) reinterpret_cast<float2 *>(partial)[o] = make_float2(acc[jj], acc[HALF + jj]);
                    else partial[o] = acc[jj];
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
            mbar_expect_tx(&S.b_full[sb], 2 * BSTAGE + WKT * (uint32_t)sizeof(float2));
            bulk_g2s(S.b[sb][0], src, BSTAGE, &S.b_full[sb]);
            bulk_g2s(S.b[sb][1], src + BTILE, BSTAGE, &S.b_full[sb]);
            bulk_g2s(S.at[sb], at_hilo + (size_t)st * WKT, WKT * (uint32_t)sizeof(float2), &S.b_full[sb]);
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

// ecg[s][l][t] (l < nmove) = sum_L F[s][L][t] [(1 - k3) (Y1_L + E[L][t] U1) + k3 (Y2_L + U0)]
// (with one basis the GEMM already mixed k3: Y_L + (1 - k3) E U1 + k3 U0), Y_L = sum over the band
// items of (t's tile, L) of the raw accumulators, (U0, U1) = U[row'][L][ent[L][j]], row = s * nmove
// + l, row' = l * S + s, j = t / 128.  Block per (row, 32 steps): the 8 warps split each layer's
// items (FP32, combined in a fixed order), the sum over layers is float-float, written as FP64 and
// float-float (few rows, many items); k_reduce_band: one thread per (row, RB_T consecutive steps),
// vector loads of the partials (many rows).
__global__ void __launch_bounds__(256) k_reduce_band_w(int steps, int rows, int nmove, int n_sims, int nleads, int nl,
                                                     int ntt, int max_ent, int nb, const int32_t *__restrict__ ti0,
                                                     const int32_t *__restrict__ ti1, const int32_t *__restrict__ ent,
                                                     const float *__restrict__ partial, const float2 *__restrict__ U,
                                                     const float *__restrict__ E, const float *__restrict__ F,
                                                     const double *__restrict__ k3, double *__restrict__ ecg,
                                                       float2 *__restrict__ ecg_ff, const double *__restrict__ cmov) {
    __shared__ float red[8][2][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tt = blockIdx.x * 32 + lane;
    const int r = blockIdx.y;
    const int s = r / nmove, l = r % nmove;
    const int j = (blockIdx.x * 32) / BM, tl = tt - j * BM;
    const bool on = tt < steps;
    const size_t rp = (size_t)l * n_sims + s;
    float2 v = make_float2(0.f, 0.f);
    for (int L = 0; L < nl; ++L) {
        float y1 = 0.f, y2 = 0.f;
        const int c1 = ti1[j * nl + L];
        if (on) {
            if (nb == 2) {
                for (int c = ti0[j * nl + L] + w; c < c1; c += 8) {
                    const float2 p = reinterpret_cast<const float2 *>(partial)[((size_t)c * rows + r) * BM + tl];
                    y1 += p.x;
                    y2 += p.y;
                }
            } else {
                for (int c = ti0[j * nl + L] + w; c < c1; c += 8) y1 += partial[((size_t)c * rows + r) * BM + tl];
            }
        }
        red[w][0][lane] = y1;
        red[w][1][lane] = y2;
        __syncthreads();
        if (w == 0 && on) {
            y1 = y2 = 0.f;
            for (int i = 0; i < 8; ++i) {
                y1 += red[i][0][lane];
                y2 += red[i][1][lane];
            }
            const float kk = (float)k3[(size_t)s * nl + L];
            const int e = ent[L * ntt + j];
            float st1 = 0.f, st0 = 0.f;
            if (e >= 0) {
                const float2 u = U[(rp * nl + L) * max_ent + e];
                st1 = E[(size_t)L * steps + tt] * u.y;
                st0 = u.x;
            }
            const float x = nb == 2 ? fmaf(kk, (y2 + st0) - (y1 + st1), y1 + st1)
                                    : fmaf(kk, st0 - st1, y1 + st1);
            v = ff_add_f(v, F[((size_t)s * nl + L) * steps + tt] * x);
        }
        __syncthreads();
    }
    if (w == 0 && on) {
        const size_t o = ((size_t)s * nleads + l) * steps + tt;
        if (cmov) v = ff_add(v, ff_from_double(cmov[rp]));
        ecg[o] = ff_to_double(v);
        ecg_ff[o] = v;
    }
}

constexpr int RB_T = 4;  // consecutive steps per thread of k_reduce_band
__global__ void k_reduce_band(int steps, int rows, int nmove, int n_sims, int nleads, int nl, int ntt, int max_ent,
                              int nb, const int32_t *__restrict__ ti0, const int32_t *__restrict__ ti1,
                              const int32_t *__restrict__ ent, const float *__restrict__ partial,
                              const float2 *__restrict__ U, const float *__restrict__ E, const float *__restrict__ F,
                              const double *__restrict__ k3, double *__restrict__ ecg,
                              float2 *__restrict__ ecg_ff, const double *__restrict__ cmov) {
    const int t0 = (blockIdx.x * blockDim.x + threadIdx.x) * RB_T;  // RB_T steps inside one 128-step tile
    if (t0 >= steps) return;
    const int r = blockIdx.y;
    const int s = r / nmove, l = r % nmove;
    const int j = t0 / BM, tl = t0 - j * BM;
    const size_t rp = (size_t)l * n_sims + s;
    float2 v[RB_T];
#pragma unroll
    for (int k = 0; k < RB_T; ++k) v[k] = make_float2(0.f, 0.f);
    for (int L = 0; L < nl; ++L) {
        const float kk = (float)k3[(size_t)s * nl + L];
        float y1[RB_T], y2[RB_T];
#pragma unroll
        for (int k = 0; k < RB_T; ++k) y1[k] = y2[k] = 0.f;
        const int c0 = ti0[j * nl + L], c1 = ti1[j * nl + L];
        if (nb == 2) {
            for (int c = c0; c < c1; ++c) {
                const float4 *p = reinterpret_cast<const float4 *>(partial + (((size_t)c * rows + r) * BM + tl) * 2);
                const float4 a = p[0], b = p[1];
                y1[0] += a.x;
                y2[0] += a.y;
                y1[1] += a.z;
                y2[1] += a.w;
                y1[2] += b.x;
                y2[2] += b.y;
                y1[3] += b.z;
                y2[3] += b.w;
            }
        } else {
            for (int c = c0; c < c1; ++c) {
                const float4 a = *reinterpret_cast<const float4 *>(partial + ((size_t)c * rows + r) * BM + tl);
                y1[0] += a.x;
                y1[1] += a.y;
                y1[2] += a.z;
                y1[3] += a.w;
            }
        }
        const int e = ent[L * ntt + j];
        const float2 u = e >= 0 ? U[(rp * nl + L) * max_ent + e] : make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < RB_T; ++k) {
            const int tt = t0 + k;
            if (tt >= steps) break;
            const float st1 = e >= 0 ? E[(size_t)L * steps + tt] * u.y : 0.f, st0 = u.x;
            const float x = nb == 2 ? fmaf(kk, (y2[k] + st0) - (y1[k] + st1), y1[k] + st1)
                                    : fmaf(kk, st0 - st1, y1[k] + st1);
            v[k] = ff_add_f(v[k], F[((size_t)s * nl + L) * steps + tt] * x);
        }
    }
    const float2 c = cmov ? ff_from_double(cmov[rp]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < RB_T; ++k) {
        const int tt = t0 + k;
        if (tt >= steps) break;
        const size_t o = ((size_t)s * nleads + l) * steps + tt;
        if (cmov) v[k] = ff_add(v[k], c);
        ecg[o] = ff_to_double(v[k]);
        ecg_ff[o] = v[k];
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
    dim3 grid((unsigned)A.nitems, (unsigned)A.ntiles);
    k_batch_umma<NB, N><<<grid, WS_THREADS, smem, st>>>(A.steps, A.nl, A.nkt, A.rows, A.nmove, A.n_sims, A.t_hilo,
                                                        A.at_hilo, A.items, A.hconst, A.Bt, A.partial, A.err);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace

// N of the band GEMM's row tiles: the smallest instance that holds the rows (one simulation's moved
// leads fit 32), else the largest (256 with one basis, 128 with two).
int small_operand_sims() { return SMALL_SIMS; }

int batch_tile_rows(int two_bases, int rows_used) {
    if (rows_used <= 32) return 32;
    if (two_bases || rows_used <= 128) return 128;
    return 256;
}

void launch_taylor_w(cudaStream_t s, const HeartDev &h, const float *W0, int J, const double *centre,
                     const double *scale, float *Wt) {
    dim3 grid((unsigned)((h.apad + 255) / 256), (unsigned)h.nleads);
    k_taylor_w<<<grid, 256, 0, s>>>(h.apad, h.nleads, J, W0, h.at.p, h.a_layer.p, centre, scale, Wt);
    EKG_CUDA(cudaGetLastError());
}

void launch_reduce_layers(cudaStream_t s, int steps, int rows, int nl, const int32_t *lc0, const int32_t *lc1,
                          const double *partial, float *Q) {
    dim3 grid((unsigned)((steps + 31) / 32), (unsigned)rows);
    k_reduce_layers<<<grid, 256, 0, s>>>(steps, rows, nl, lc0, lc1, partial, Q);
    EKG_CUDA(cudaGetLastError());
}

void launch_static_combine(cudaStream_t s, const HeartDev &h, int J, int Jb, int nmove, int n_sims, const float *F,
                           const float *coef, const double *k3, const float *Q1, const float *Q2, double *ecg,
                           float2 *ecg_ff, const double *cst) {
    if (nmove >= h.nleads) return;
    dim3 grid((unsigned)((h.steps + 127) / 128), (unsigned)(h.nleads - nmove), (unsigned)((n_sims + SC_SIMS - 1) / SC_SIMS));
    k_static_combine<<<grid, 128, 0, s>>>(h.steps, h.nleads, h.nlayers, J, Jb, nmove, n_sims, F, coef, k3, Q1, Q2,
                                          ecg, ecg_ff, cst);
    EKG_CUDA(cudaGetLastError());
}

// Lead field of the per-simulation form: one thread per (AP, simulation).  The moved leads (rows
// [0, nmove)) are evaluated in pairs that share the voxel loads, with the same field evaluation as
// the batched form's operand kernel (closed form for interior voxels and for boundary voxels with
// few absent neighbours where the leads are at least 20 cells away, exact sums otherwise); their
// W is written for the k0 term and W' = W exp(k5_L at_a) for the contraction.  With static_rows the
// leads at their loaded position take the resident field W0, scaled the same way (for the dense
// contractions; the band contraction scales W0 itself).  Lead positions are FP64
// [S][lead_stride][3] (z, y, x), made relative to the voxel centre in FP64 before the FP32 cast.
template <bool DIAG>
__global__ void __launch_bounds__(128) k_sim_lead_field(
    int64_t apad, InteriorField ic, const int64_t *__restrict__ a_vox_begin, const float4 *__restrict__ vox_pos,
    const float4 *__restrict__ vox_out, int nnb, const int8_t *__restrict__ difs, const double *__restrict__ at,
    const int32_t *__restrict__ a_layer, const double *__restrict__ layer_k, int nl, const double *__restrict__ leads,
    int lead_stride, double cz, double cy, double cx, int nmove, int nleads, const float *__restrict__ W0,
    float *__restrict__ W, float *__restrict__ Wp, int static_rows) {
    __shared__ float s_d[26 * 4];
    const int tid = threadIdx.x;
    if (tid < nnb) {
        const float dz = difs[3 * tid], dy = difs[3 * tid + 1], dx = difs[3 * tid + 2];
        s_d[4 * tid] = dz;
        s_d[4 * tid + 1] = dy;
        s_d[4 * tid + 2] = dx;
        s_d[4 * tid + 3] = dz * dz + dy * dy + dx * dx;
    }
    __syncthreads();
    const int64_t a = (int64_t)blockIdx.x * 128 + tid;
    const int s = blockIdx.y;
    if (a >= apad) return;
    const double aa = at[a];
    const float f = isinf(aa) ? 0.f : expf((float)(layer_k[((size_t)s * nl + a_layer[a]) * 9 + 5] * aa));
    const int vb = (int)a_vox_begin[a], ve = (int)a_vox_begin[a + 1];
    const uint32_t full = (1u << nnb) - 1u;
    for (int l0 = 0; l0 < nmove; l0 += 2) {
        const int np = l0 + 1 < nmove ? 2 : 1;
        float4 r[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const double *p = leads + ((size_t)s * lead_stride + l0 + min(q, np - 1)) * 3;
            r[q] = make_float4((float)(p[0] - cz), (float)(p[1] - cy), (float)(p[2] - cx), 0.f);
        }
        float acc[2] = {0.f, 0.f};
        for (int v = vb; v < ve; ++v) {
            const float4 pos = vox_pos[v];
            const uint32_t mi = __float_as_uint(pos.w);
            MSquares q[2];
            q[0] = msq(pos, r[0]);
            q[1] = msq(pos, r[1]);
            const bool far = q[0].s >= INTERIOR_S_MIN && q[1].s >= INTERIOR_S_MIN;
            if ((mi & VOX_INTERIOR) && far) {
                acc[0] += interior_w(ic, q[0], rsqa(q[0].s));
                acc[1] += interior_w(ic, q[1], rsqa(q[1].s));
            } else if ((mi & VOX_FEW) && far) {
                few_w<2>(ic, q, pos, r, full & ~mi, vox_out[v], s_d, acc);
            } else {
                const float4 out = vox_out[v];
#pragma unroll
                for (int k = 0; k < 2; ++k)
                    acc[k] += DIAG ? voxel_w_diag(pos, mi, out, r[k]) : voxel_w_general(pos, mi, out, r[k], nnb, s_d);
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (q >= np) break;
            const size_t o = ((size_t)s * nleads + l0 + q) * apad + a;
            W[o] = acc[q];
            if (Wp) Wp[o] = acc[q] * f;
        }
    }
    if (static_rows)
        for (int l = nmove; l < nleads; ++l) Wp[((size_t)s * nleads + l) * apad + a] = W0[(size_t)l * apad + a] * f;
}

// Per-simulation form with many simulations: the moved rows' unscaled field W[s][l][a] (FP32) with
// the batched operand kernel's work split -- items (32-AP stage, group of LF_THREADS * LF_ROWS
// rows) taken from a counter, stages with the most voxels first, a stage's voxel records staged in
// shared memory, LF_ROWS rows per thread sharing each voxel's loads and tests, the stage bounding-box
// test -- instead of one thread per (AP, simulation), whose warps diverge over the APs' voxel
// counts.  Row = s * nmove + l; lead positions FP64 [S][lead_stride][3] made relative to the voxel
// centre in FP64 before the FP32 cast.  The band contraction scales W by exp(k5 at).  With fewer
// rows the block's warps split the stage's four 8-AP chunks: ksplit groups of LF_THREADS / ksplit
// threads, group g taking chunks g, g + ksplit, ... of the item's stage.
template <bool DIAG, int ROWS>
__global__ void __launch_bounds__(LF_THREADS, 8) k_sim_lead_field_rows(
    int nst, int ngr, int ksplit, int *__restrict__ work, InteriorField ic, const int64_t *__restrict__ a_vox_begin,
    const float4 *__restrict__ vox_pos, const float4 *__restrict__ vox_out, int nnb, const int8_t *__restrict__ difs,
    const double *__restrict__ leads, int lead_stride, double cz, double cy, double cx, int nmove, int n_sims,
    int nleads, int64_t apad, const int32_t *__restrict__ stage_order, const float4 *__restrict__ stage_box,
    float *__restrict__ W) {
    __shared__ float s_d[26 * 4];
    __shared__ float s_w[LF_ROWS][8][LF_THREADS];  // rows [0, ROWS) used
    __shared__ int s_vb[BST / 8 + 1];
    __shared__ float4 s_vpos[LF_VCAP], s_vout[LF_VCAP];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    if (tid < nnb) {
        const float dz = difs[3 * tid], dy = difs[3 * tid + 1], dx = difs[3 * tid + 2];
        s_d[4 * tid] = dz;
        s_d[4 * tid + 1] = dy;
        s_d[4 * tid + 2] = dx;
        s_d[4 * tid + 3] = dz * dz + dy * dy + dx * dx;
    }
    const int rows_used = n_sims * nmove;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(work, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= nst * ngr) break;
        const int st = stage_order[item / ngr];
        const int v0 = (int)a_vox_begin[(int64_t)st * BST], nv = (int)a_vox_begin[(int64_t)(st + 1) * BST] - v0;
        const bool staged = nv <= LF_VCAP;
        if (staged)
            for (int i = tid; i < nv; i += LF_THREADS) {
                s_vpos[i] = vox_pos[v0 + i];
                s_vout[i] = vox_out[v0 + i];
            }
        if (tid < BST / 8 + 1) s_vb[tid] = (int)a_vox_begin[(int64_t)st * BST + tid * 8] - (staged ? v0 : 0);
        __syncthreads();
        const float4 *vp = staged ? s_vpos : vox_pos, *vo = staged ? s_vout : vox_out;
        const int gthreads = LF_THREADS / ksplit, kg = tid / gthreads;
        const int rb = (item % ngr) * (gthreads * ROWS) + (tid % gthreads) * ROWS;
        const int nr = rb < rows_used ? min(ROWS, rows_used - rb) : 0;  // the rest repeat the last row
        float4 r[ROWS];
        bool far_all = true;
        if (nr > 0) {
            const float4 lo = stage_box[2 * (size_t)st], hi = stage_box[2 * (size_t)st + 1];
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                const int row = rb + min(q, nr - 1);
                const double *p = leads + ((size_t)(row / nmove) * lead_stride + row % nmove) * 3;
                r[q] = make_float4((float)(p[0] - cz), (float)(p[1] - cy), (float)(p[2] - cx), 0.f);
                const float dz = fmaxf(fmaxf(lo.x - r[q].x, r[q].x - hi.x), 0.f);
                const float dy = fmaxf(fmaxf(lo.y - r[q].y, r[q].y - hi.y), 0.f);
                const float dx = fmaxf(fmaxf(lo.z - r[q].z, r[q].z - hi.z), 0.f);
                far_all = far_all && dz * dz + dy * dy + dx * dx >= INTERIOR_S_MIN + 41.f;
            }
        }
        far_all = __all_sync(0xffffffffu, far_all);
        if (nr == 0) continue;
#pragma unroll 1
        for (int kc = kg; kc < BST / 8; kc += ksplit) {
            if (far_all) chunk_w<DIAG, ROWS, true>(s_vb[kc], s_vb[kc + 1], vp, vo, r, nnb, s_d, ic, s_w, tid);
            else chunk_w<DIAG, ROWS, false>(s_vb[kc], s_vb[kc + 1], vp, vo, r, nnb, s_d, ic, s_w, tid);
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                if (q >= nr) break;
                const int row = rb + q;
                float4 *dst = reinterpret_cast<float4 *>(W + ((size_t)(row / nmove) * nleads + row % nmove) * apad +
                                                         (size_t)st * BST + kc * 8);
                dst[0] = make_float4(s_w[q][0][tid], s_w[q][1][tid], s_w[q][2][tid], s_w[q][3][tid]);
                dst[1] = make_float4(s_w[q][4][tid], s_w[q][5][tid], s_w[q][6][tid], s_w[q][7][tid]);
            }
        }
    }
}

void launch_sim_lead_field_rows(cudaStream_t s, const HeartDev &h, const double *d_leads, int nmove, int lead_stride,
                                int n_sims, float *W, int *work, int sm_count) {
    InteriorField ic;
    ic.A0 = h.interior_c[0];
    ic.A1 = h.interior_c[1];
    ic.B0 = h.interior_c[2];
    ic.B1 = h.interior_c[3];
    ic.B2 = h.interior_c[4];
    const int rows_used = n_sims * nmove;
    int rows_t = 4, ksplit = 1;  // the operand kernel's layouts (rows per thread, chunk split)
    if (rows_used <= 32) rows_t = 1, ksplit = 4;
    else if (rows_used <= 64) rows_t = 1, ksplit = 2;
    else if (rows_used <= 128) rows_t = 1, ksplit = 1;
    else if (rows_used <= 256) rows_t = 4, ksplit = 2;
    const int grows = LF_THREADS / ksplit * rows_t;
    const int ngr = (rows_used + grows - 1) / grows;
    const int nst = (int)(h.apad / BST);
    const int items = nst * ngr;
    const int grid = std::max(1, std::min(items, sm_count * 8));
    EKG_CUDA(cudaMemsetAsync(work, 0, sizeof(int), s));
    auto go = [&](auto kern) {
        kern<<<grid, LF_THREADS, 0, s>>>(nst, ngr, ksplit, work, ic, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p, h.nnb,
                                         h.difs.p, d_leads, lead_stride, h.centre[0], h.centre[1], h.centre[2], nmove,
                                         n_sims, h.nleads, h.apad, h.stage_order.p, h.stage_box.p, W);
    };
    const bool diag = h.nhood == EKG_NHOOD_3D4;
    if (rows_t == 1) {
        if (diag) go(k_sim_lead_field_rows<true, 1>);
        else go(k_sim_lead_field_rows<false, 1>);
    } else {
        if (diag) go(k_sim_lead_field_rows<true, 4>);
        else go(k_sim_lead_field_rows<false, 4>);
    }
    EKG_CUDA(cudaGetLastError());
}

void launch_sim_lead_field(cudaStream_t s, const HeartDev &h, const double *d_leads, int nmove, int lead_stride,
                           int n_sims, const double *d_layer_k, const float *W0, float *W, float *Wp,
                           bool static_rows) {
    if (nmove == 0 && !static_rows) return;
    InteriorField ic;
    ic.A0 = h.interior_c[0];
    ic.A1 = h.interior_c[1];
    ic.B0 = h.interior_c[2];
    ic.B1 = h.interior_c[3];
    ic.B2 = h.interior_c[4];
    const dim3 g((unsigned)((h.apad + 127) / 128), (unsigned)n_sims);
    if (h.nhood == EKG_NHOOD_3D4)
        k_sim_lead_field<true><<<g, 128, 0, s>>>(h.apad, ic, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p, h.nnb, h.difs.p,
                                                 h.at.p, h.a_layer.p, d_layer_k, h.nlayers, d_leads, lead_stride,
                                                 h.centre[0], h.centre[1], h.centre[2], nmove, h.nleads, W0, W, Wp,
                                                 static_rows ? 1 : 0);
    else
        k_sim_lead_field<false><<<g, 128, 0, s>>>(h.apad, ic, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p, h.nnb, h.difs.p,
                                                  h.at.p, h.a_layer.p, d_layer_k, h.nlayers, d_leads, lead_stride,
                                                  h.centre[0], h.centre[1], h.centre[2], nmove, h.nleads, W0, W, Wp,
                                                 static_rows ? 1 : 0);
    EKG_CUDA(cudaGetLastError());
}

void launch_batch_lead_field(cudaStream_t s, const HeartDev &h, int tile_rows, bool small, int blocks_per_sm,
                             const float *k5l,
                             const float4 *hconst, const float4 *lrel, int nmove, int n_sims, const BandArgs &B,
                             uint8_t *Bt, int *work, int sm_count) {
    const int rows_used = n_sims * nmove;
    const int nst = (int)(h.apad / BST);
    const bool diag = h.nhood == EKG_NHOOD_3D4;
    InteriorField ic;
    ic.A0 = h.interior_c[0];
    ic.A1 = h.interior_c[1];
    ic.B0 = h.interior_c[2];
    ic.B1 = h.interior_c[3];
    ic.B2 = h.interior_c[4];
    const int nlog = tile_rows == 32 ? 5 : (tile_rows == 128 ? 7 : 8);
    if (small) {
        dim3 g((unsigned)((nst * BST + 127) / 128), (unsigned)n_sims);
#define EKG_LFS(NN, DG)                                                                                            \
    k_batch_lead_field_small<NN, DG><<<g, 128, 0, s>>>(nst, ic, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p, h.nnb,  \
                                                       h.difs.p, h.at_hilo.p, h.a_layer.p, k5l, h.nlayers, hconst,  \
                                                       lrel, nmove, n_sims, B.tref, B.nent, B.esplit, Bt, B.P1, B.P2)
        if (tile_rows == 32) {
            if (diag) EKG_LFS(32, true);
            else EKG_LFS(32, false);
        } else if (tile_rows == 128) {
            if (diag) EKG_LFS(128, true);
            else EKG_LFS(128, false);
        } else {
            if (diag) EKG_LFS(256, true);
            else EKG_LFS(256, false);
        }
#undef EKG_LFS
        EKG_CUDA(cudaGetLastError());
        return;
    }
    // rows per thread and chunk split by the rows: a warp covers 32 lanes x rows, so few rows take
    // one row per thread, and the block's warps split a stage's four 8-AP chunks when the rows fill
    // fewer than all of them (measured at 160^3 against four rows per thread and four groups: 32
    // simulations x 2 moved leads 0.208 against 0.288 ms per pass, 128 simulations 0.457 against 0.508)
    int rows_t = 4, ksplit = 1;
    if (rows_used <= 32) rows_t = 1, ksplit = 4;
    else if (rows_used <= 64) rows_t = 1, ksplit = 2;
    else if (rows_used <= 128) rows_t = 1, ksplit = 1;
    else if (rows_used <= 256) rows_t = 4, ksplit = 2;
    const int grows = LF_THREADS / ksplit * rows_t;
    const int ngr = (rows_used + grows - 1) / grows;
    EKG_CUDA(cudaMemsetAsync(work, 0, sizeof(int), s));
    auto go = [&](auto kern) {
        static int per_sm = 0;
        if (!per_sm) EKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, LF_THREADS, 0));
        const int bps = blocks_per_sm > 0 ? std::min(blocks_per_sm, std::max(1, per_sm)) : std::max(1, per_sm);
        const int grid = std::max(1, std::min(nst * ngr, bps * sm_count));
        kern<<<grid, LF_THREADS, 0, s>>>(nlog, nst, ngr, ksplit, work, ic, h.a_vox_begin.p, h.vox_pos.p, h.vox_out.p,
                                         h.nnb, h.difs.p, h.at_hilo.p, h.a_layer.p, k5l, h.nlayers, hconst, lrel, nmove,
                                         n_sims, B.tref, B.nent, B.esplit, h.stage_order.p, h.stage_box.p, Bt, B.P1,
                                         B.P2);
    };
    // the resting-potential sums (P2) only where a pass needs them: the unsplit instance is compiled
    // with and without them
    const bool k0 = B.P2 != nullptr;
    if (diag) {
        if (rows_t == 1) go(k_batch_lead_field<true, 1, true, true>);
        else if (ksplit > 1) go(k_batch_lead_field<true, 4, true, true>);
        else if (k0) go(k_batch_lead_field<true, 4, false, true>);
        else go(k_batch_lead_field<true, 4, false, false>);
    } else {
        if (rows_t == 1) go(k_batch_lead_field<false, 1, true, true>);
        else if (ksplit > 1) go(k_batch_lead_field<false, 4, true, true>);
        else if (k0) go(k_batch_lead_field<false, 4, false, true>);
        else go(k_batch_lead_field<false, 4, false, false>);
    }
    EKG_CUDA(cudaGetLastError());
}

void launch_batch_gemm(cudaStream_t s, const BatchArgs &A) {
    if (A.nitems == 0) return;
    const int N = A.tile_rows > 0 ? A.tile_rows : batch_tile_rows(A.two_bases, A.rows_used);
    if (A.two_bases) {
        if (N == 32) launch_gemm<2, 32>(s, A);
        else launch_gemm<2, 128>(s, A);
    } else {
        if (N == 32) launch_gemm<1, 32>(s, A);
        else if (N == 128) launch_gemm<1, 128>(s, A);
        else launch_gemm<1, 256>(s, A);
    }
}

// ------------------------------------------------------------------ resting-potential term
// A layer's resting potential k0 adds k0_L sum_{a in L} W[l][a] to every sample of lead l (the AP
// differences of the dipoles cancel it within a layer, simlib/simulator.cpp:509-525); the sum over
// layers of sum_a W vanishes, so the term is taken relative to the first layer's k0.
// Moved rows: thread per row' = l * S + s, the per-part unscaled sums P2 of each layer's stages
// added in FP64 in a fixed order.
__global__ void k_k0_moved(int rows_used, int n_sims, int nl, const int32_t *__restrict__ ls0,
                           const int32_t *__restrict__ ls1, const float *__restrict__ P2,
                           const double *__restrict__ layer_k, double *__restrict__ cmov) {
    const int rp = blockIdx.x * blockDim.x + threadIdx.x;
    if (rp >= rows_used) return;
    const int s = rp % n_sims;
    const double k00 = layer_k[(size_t)s * nl * 9];
    double c = 0.0;
    for (int L = 0; L < nl; ++L) {
        double sw = 0.0;
        for (int p = ls0[L] * 4; p < ls1[L] * 4; ++p) sw += (double)P2[(size_t)p * rows_used + rp];
        c += (layer_k[((size_t)s * nl + L) * 9] - k00) * sw;
    }
    cmov[rp] = c;
}

// Static leads: K0s[L][l] = sum_{a in L} W0[l][a] in FP64, block per (lead, layer).
__global__ void k_k0_static_sums(int nleads, int64_t apad, const int32_t *__restrict__ ls0,
                                 const int32_t *__restrict__ ls1, const float *__restrict__ W0,
                                 double *__restrict__ K0s) {
    __shared__ double red[8];
    const int l = blockIdx.x, L = blockIdx.y;
    double v = 0.0;
    for (int64_t a = (int64_t)ls0[L] * 32 + threadIdx.x; a < (int64_t)ls1[L] * 32; a += blockDim.x)
        v += (double)W0[(size_t)l * apad + a];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        K0s[(size_t)L * nleads + l] = t;
    }
}

// cst[s][l] = sum_L (k0_L - k0_0) K0s[L][l] for the static leads l >= nmove (relative: the batched
// form, whose other terms carry no k0), or sum_L k0_L K0s[L][l] (the per-simulation form's k0w).
__global__ void k_k0_static(int n_sims, int nleads, int nmove, int nl, const double *__restrict__ K0s,
                            const double *__restrict__ layer_k, double *__restrict__ cst, int relative) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_sims * nleads) return;
    const int s = i / nleads, l = i % nleads;
    if (l < nmove) return;
    const double k00 = relative ? layer_k[(size_t)s * nl * 9] : 0.0;
    double c = 0.0;
    for (int L = 0; L < nl; ++L) c += (layer_k[((size_t)s * nl + L) * 9] - k00) * K0s[(size_t)L * nleads + l];
    cst[i] = c;
}

void launch_k0_moved(cudaStream_t s, const BandArgs &A, const int32_t *ls0, const int32_t *ls1,
                     const double *layer_k, double *cmov) {
    k_k0_moved<<<(unsigned)((A.rows_used + 127) / 128), 128, 0, s>>>(A.rows_used, A.n_sims, A.nl, ls0, ls1, A.P2,
                                                                     layer_k, cmov);
    EKG_CUDA(cudaGetLastError());
}

void launch_k0_static_sums(cudaStream_t s, int nleads, int64_t apad, int nl, const int32_t *ls0, const int32_t *ls1,
                           const float *W0, double *K0s) {
    k_k0_static_sums<<<dim3((unsigned)nleads, (unsigned)nl), 256, 0, s>>>(nleads, apad, ls0, ls1, W0, K0s);
    EKG_CUDA(cudaGetLastError());
}

void launch_k0_static(cudaStream_t s, int n_sims, int nleads, int nmove, int nl, const double *K0s,
                      const double *layer_k, double *cst, bool relative) {
    const int n = n_sims * nleads;
    k_k0_static<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n_sims, nleads, nmove, nl, K0s, layer_k, cst,
                                                            relative ? 1 : 0);
    EKG_CUDA(cudaGetLastError());
}

// out[L][l] = sum_{a: a_layer[a] == L} W0[l][a] in FP64, block per (lead, layer); padding APs hold
// no voxels (W0 = 0).
__global__ void k_w0_layer_sums(int64_t apad, int nleads, const float *__restrict__ W0,
                                const int32_t *__restrict__ a_layer, double *__restrict__ out) {
    __shared__ double red[8];
    const int l = blockIdx.x, L = blockIdx.y;
    double v = 0.0;
    for (int64_t a = threadIdx.x; a < apad; a += blockDim.x)
        if (a_layer[a] == L) v += (double)W0[(size_t)l * apad + a];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        out[(size_t)L * nleads + l] = t;
    }
}

void launch_w0_layer_sums(cudaStream_t s, const HeartDev &h, const float *W0, double *out) {
    k_w0_layer_sums<<<dim3((unsigned)h.nleads, (unsigned)h.nlayers), 256, 0, s>>>(h.apad, h.nleads, W0, h.a_layer.p,
                                                                                  out);
    EKG_CUDA(cudaGetLastError());
}

int band_u_parts() { return BU_PARTS; }

void launch_band_u(cudaStream_t s, const BandArgs &A) {
    k_band_u<<<dim3(BU_PARTS, (unsigned)((A.rows_used + 127) / 128), (unsigned)A.nl), 128, 0, s>>>(
        A.rows_used, A.nl, A.max_ent, A.nent, A.esplit, A.ls0, A.ls1, A.goff, A.gtab, A.P1, A.Up);
    const int64_t n = (int64_t)A.rows_used * A.nl * A.max_ent;
    k_band_u2<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, A.Up, A.U);
    EKG_CUDA(cudaGetLastError());
}

void launch_reduce_band(cudaStream_t s, const BandArgs &A) {
    if (A.rows_used < 64) {
        dim3 grid((unsigned)((A.steps + 31) / 32), (unsigned)A.rows_used);
        k_reduce_band_w<<<grid, 256, 0, s>>>(A.steps, A.rows, A.nmove, A.n_sims, A.nleads, A.nl, A.ntt, A.max_ent,
                                             A.nb, A.ti0, A.ti1, A.ent, A.partial, A.U, A.E, A.F, A.k3, A.ecg,
                                             A.ecg_ff, A.cmov);
    } else {
        dim3 grid((unsigned)((A.steps + 128 * RB_T - 1) / (128 * RB_T)), (unsigned)A.rows_used);
        k_reduce_band<<<grid, 128, 0, s>>>(A.steps, A.rows, A.nmove, A.n_sims, A.nleads, A.nl, A.ntt, A.max_ent,
                                           A.nb, A.ti0, A.ti1, A.ent, A.partial, A.U, A.E, A.F, A.k3, A.ecg,
                                           A.ecg_ff, A.cmov);
    }
    EKG_CUDA(cudaGetLastError());
}

}  // namespace ekg
