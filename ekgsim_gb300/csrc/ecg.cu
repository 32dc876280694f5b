// ecg.cu -- simulated ECG of one heart: lead field, AP factors, contraction, FP64 reduction,
// criteria.
//
// The reference forms, per non-empty voxel x, the dipole D_x(t) = sum_n d_n (AP(x-d_n,t) - AP(x,t))
// and adds g_l(x) . D_x(t) to lead l, g_l(x) = (r_l - x)/|r_l - x|^3 (simlib/simulator.cpp:489-537).
// The same sum regrouped by cell AP (the reference's apIndex, simlib/simulator.cpp:561-621) is a
// contraction over the de-duplicated APs:
//     ECG_l(t) = sum_a W[l,a] AP_a(t),   W[l,a] = sum_{voxels y of AP a} w_l(y),
//     w_l(y)   = sum_{n: y+d_n non-empty} g_l(y+d_n).d_n  -  g_l(y) . sum_{n: y-d_n non-empty} d_n.
// The Wohlfart AP (simlib/Wohlfart.h:195-203) with k8 shifted by the activation time
// (simlib/simulator.cpp:154-170) factors, with tau = t - at, as
//     AP_a(t) - k0 = H_a(t) * F_L(t) * exp(k5 at),
//     H_a(t) = sigma(k1 tau) ((1-k3) exp(-k4 tau) + k3)                (per AP and step, FP32)
//     F_L(t) = k2 exp(-k5 t) (1 - (1 + exp(-k7 (t-k8)) (2^(k7/k6) - 1))^(-k6/k7))   (per layer, FP64)
// so the device evaluates H on the fly, folds exp(k5 at) into the lead field (W' = W exp(k5 at)),
// and applies F_L in FP64 to each layer's partial sums.  k0 cancels inside every AP difference of
// one layer; across layers it leaves the constant sum_L k0_L sum_{a in L} W[l,a].
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ekg_internal.h"

namespace ekg {

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// H_a(t) in FP32; c = {k1*log2(e), k4*log2(e), 1-k3, k3}
__device__ __forceinline__ float h_value(float tau, float4 c) {
    const float e1 = ex2_approx(-c.x * tau);
    const float s = rcp_approx(1.0f + e1);
    const float e4 = ex2_approx(-c.y * tau);
    const float h = s * fmaf(c.z, e4, c.w);
    return s == 0.0f ? 0.0f : h;
}

// ------------------------------------------------------------------ lead field
// One thread per (AP a, lead l, sim s).  Lead positions FP64 [S][lead_stride][3] (z,y,x);
// W [S][w_lead_stride][apad].
__global__ void k_lead_field(int64_t apad, const int64_t *__restrict__ a_vox_begin,
                             const int32_t *__restrict__ vox_zyx, const uint32_t *__restrict__ nb_in,
                             const uint32_t *__restrict__ nb_out, int nnb, const int8_t *__restrict__ difs,
                             const double *__restrict__ leads, int nleads, int lead_stride,
                             float *__restrict__ W, int w_lead_stride) {
    __shared__ int8_t s_dif[26 * 3];
    if (threadIdx.x < nnb * 3) s_dif[threadIdx.x] = difs[threadIdx.x];
    __syncthreads();
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y, s = blockIdx.z;
    if (a >= apad || l >= nleads) return;
    const double *r = leads + ((size_t)s * lead_stride + l) * 3;
    const float rz = (float)r[0], ry = (float)r[1], rx = (float)r[2];
    const float rzl = (float)(r[0] - (double)rz), ryl = (float)(r[1] - (double)ry), rxl = (float)(r[2] - (double)rx);
    double acc = 0.0;
    const int64_t v0 = a_vox_begin[a], v1 = a_vox_begin[a + 1];
    for (int64_t v = v0; v < v1; ++v) {
        const int32_t p = vox_zyx[v];
        // bordered coordinates (simlib/simulator.cpp:458-463, 487)
        const float pz = (float)((p >> 20) + 1), py = (float)(((p >> 10) & 1023) + 1), px = (float)((p & 1023) + 1);
        const uint32_t mi = nb_in[v], mo = nb_out[v];
        float w = 0.f;
        float sz = 0.f, sy = 0.f, sx = 0.f;
        for (int n = 0; n < nnb; ++n) {
            const float dz = s_dif[3 * n], dy = s_dif[3 * n + 1], dx = s_dif[3 * n + 2];
            if (mi & (1u << n)) {
                const float mz = (rz - (pz + dz)) + rzl, my = (ry - (py + dy)) + ryl, mx = (rx - (px + dx)) + rxl;
                const float ss = fmaf(mz, mz, fmaf(my, my, mx * mx));
                const float rs = rsqrtf(ss);
                const float f = rs * rs * rs;
                w = fmaf(f, fmaf(mz, dz, fmaf(my, dy, mx * dx)), w);
            }
            if (mo & (1u << n)) {
                sz += dz;
                sy += dy;
                sx += dx;
            }
        }
        if (mo) {
            const float mz = (rz - pz) + rzl, my = (ry - py) + ryl, mx = (rx - px) + rxl;
            const float ss = fmaf(mz, mz, fmaf(my, my, mx * mx));
            const float rs = rsqrtf(ss);
            const float f = rs * rs * rs;
            w = fmaf(-f, fmaf(mz, sz, fmaf(my, sy, mx * sx)), w);
        }
        acc += (double)w;
    }
    W[((size_t)s * w_lead_stride + l) * apad + a] = (float)acc;
}

// ------------------------------------------------------------------ per-layer factors
// F[s][L][t] = k2 exp(-k5 t) R(t), R(t) = 1 - (1 + exp(-k7 (t - k8) + ln(2^(k7/k6) - 1)))^(-k6/k7)
// (the repolarisation factor of WohlfartPlus, sim.cpp).  Block per (sim, layer): the constant
// ln(2^(k7/k6) - 1) and the exponent u = -k7 (t - k8) + ln(...) in FP64, the transcendentals in
// FP32 in a form that keeps relative precision at both ends:
//     ln(1 + e^u) = log1p(exp(u)) (u + log1p(exp(-u)) for u > 0),  R = -expm1(-(k6/k7) ln(1 + e^u)).
// layer_k: [S][nl][9].
// cpre: the constants ln(2^(k7/k6) - 1) per (sim, layer) when the host computed them (small
// passes, where the FP64 pow/log would be one block's latency), else NULL.
__global__ void k_layer_factors(int nl, int steps, const double *__restrict__ t, const double *__restrict__ layer_k,
                                const double *__restrict__ cpre, int n_sims, double *__restrict__ F,
                                float *__restrict__ Ff, float *__restrict__ layer_c, const double *__restrict__ centre,
                                const double *__restrict__ scale, int J, float *__restrict__ coef) {
    const int64_t sl = blockIdx.x;  // sim * nl + layer
    const double *k = layer_k + sl * 9;
    __shared__ double c;
    if (threadIdx.x == 0) {
        c = cpre ? cpre[sl] : log(pow(2.0, k[7] / k[6]) - 1);
        const double L2E = 1.4426950408889634;
        reinterpret_cast<float4 *>(layer_c)[sl] =
            make_float4((float)(k[1] * L2E), (float)(k[4] * L2E), (float)(1.0 - k[3]), (float)k[3]);
    } else if (threadIdx.x == 32 && coef) {
        // Taylor coefficients of the static-lead basis: coef[sl][j] = exp(k5 c_L) (k5 s_L)^j / j!
        const int L = (int)(sl % nl);
        const double x = k[5] * scale[L];
        double e = exp(k[5] * centre[L]);
        for (int j = 0; j < J; ++j) {
            coef[sl * J + j] = (float)e;
            e *= x / (j + 1);
        }
    }
    __syncthreads();
    const float r = (float)(k[6] / k[7]);
    for (int step = threadIdx.x; step < steps; step += blockDim.x) {
        const double tt = t[step];
        const float u = (float)fma(-k[7], tt - k[8], c);
        const float sp = u > 0.f ? u + log1pf(expf(-u)) : log1pf(expf(u));
        const float R = -expm1f(-r * sp);
        const float e5 = expf((float)(-k[5] * tt));
        const double f = k[2] * (double)e5 * (double)R;
        F[sl * steps + step] = f;
        Ff[sl * steps + step] = (float)f;
    }
}

// k0 term: k0w[s][l] = sum_L k0_L sum_{a in L} W[s][l][a]; one block per (l, s).
__global__ void k_k0_term(int64_t apad, int nleads, const float *__restrict__ W, const int32_t *__restrict__ a_layer,
                          const double *__restrict__ layer_k, int nl, double *__restrict__ k0w) {
    const int l = blockIdx.x, s = blockIdx.y;
    __shared__ double red[256];
    double acc = 0.0;
    const float *w = W + ((size_t)s * nleads + l) * apad;
    for (int64_t a = threadIdx.x; a < apad; a += blockDim.x)
        acc += layer_k[((size_t)s * nl + a_layer[a]) * 9 + 0] * (double)w[a];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) k0w[(size_t)s * nleads + l] = red[0];
}

// ------------------------------------------------------------------ contraction (CUDA cores)
// grid (t tiles of 128, K chunks, sims * lead blocks of 16); block 128 threads, one step each.
constexpr int CC_T = 128, CC_LB = 16, CC_STAGE = 256;
__global__ void __launch_bounds__(CC_T) k_contract_cuda(int steps, int nleads, int64_t apad, int nl,
                                                        const float2 *__restrict__ t_hilo,
                                                        const float2 *__restrict__ at_hilo,
                                                        const int32_t *__restrict__ chunk_a0,
                                                        const int32_t *__restrict__ chunk_a1,
                                                        const int32_t *__restrict__ chunk_layer,
                                                        const float *__restrict__ Wp, const float *__restrict__ layer_c,
                                                        const double *__restrict__ F, int nchunks, int nlb,
                                                        double *__restrict__ partial) {
    __shared__ float s_w[CC_LB][CC_STAGE];
    __shared__ float2 s_at[CC_STAGE];
    const int c = blockIdx.y;
    const int s = blockIdx.z / nlb, lb = blockIdx.z % nlb;
    const int t = blockIdx.x * CC_T + threadIdx.x;
    const int a0 = chunk_a0[c], a1 = chunk_a1[c], L = chunk_layer[c];
    const float4 kc = reinterpret_cast<const float4 *>(layer_c)[(size_t)s * nl + L];
    const float2 th = t_hilo[t < steps ? t : steps - 1];
    const int l0 = lb * CC_LB;
    const int nlh = min(CC_LB, nleads - l0);
    float acc[CC_LB];
#pragma unroll
    for (int j = 0; j < CC_LB; ++j) acc[j] = 0.f;
    for (int b = a0; b < a1; b += CC_STAGE) {
        const int nb = min(CC_STAGE, a1 - b);
        __syncthreads();
        for (int i = threadIdx.x; i < CC_STAGE; i += CC_T) {
            s_at[i] = i < nb ? at_hilo[b + i] : make_float2(INFINITY, 0.f);
            for (int j = 0; j < CC_LB; ++j)
                s_w[j][i] = (i < nb && j < nlh) ? Wp[((size_t)s * nleads + l0 + j) * apad + b + i] : 0.f;
        }
        __syncthreads();
        for (int i = 0; i < nb; ++i) {
            const float2 at = s_at[i];
            const float tau = (th.x - at.x) + (th.y - at.y);
            const float h = h_value(tau, kc);
#pragma unroll
            for (int j = 0; j < CC_LB; ++j) acc[j] = fmaf(s_w[j][i], h, acc[j]);
        }
    }
    if (t < steps) {
        const double f = F[((size_t)s * nl + L) * steps + t];
        for (int j = 0; j < nlh; ++j)
            partial[(((size_t)s * nchunks + c) * nleads + l0 + j) * steps + t] = (double)acc[j] * f;
    }
}

// ------------------------------------------------------------------ contraction, band form
// Block per (simulation, K chunk, 16 leads).  With amin, amax the chunk's earliest and latest
// finite activation times and x = k1 log2(e) tau, the steps of the chunk fall into three runs:
//   zero    every AP has k1 (amin - t) log2 e >= 30.5 and (k1 - k4)(amin - t) log2 e >= 30.5:
//           H < 2^-30 of its amplitude (the batched form's truncation), P = 0;
//   steady  k1 (t - amax) log2 e >= 26.5 for every AP: the sigmoid is 1 in FP32 and
//           P[t,l] = (1 - k3) 2^(-k4' (t - amax)) S0[l] + k3 S1[l],
//           S0[l] = sum_a W'[l,a] 2^(-k4' (amax - at_a)), S1[l] = sum_a W'[l,a]  (k4' = k4 log2 e);
//   band    the steps in between (the chunk's upstrokes, some 10 to 30 steps of 1 ms):
//           P[t,l] = sum_a W'[l,a] H_a(t) evaluated directly in FP32, 32 (or 16) steps per pass.
// APs with an infinite activation time (unreached cells, padding) contribute nothing.  The block
// writes only what the runs need: band[s][c][l][t] = P[t,l] (FP32) for the band steps,
// csum[s][c][l] = (S0, S1) when the steady run is not empty, and cinfo[s][c] = (tb0, tb1, amax)
// (first band step, first steady step, the FP32 bits of amax); k_reduce_chunks rebuilds the runs.
// W'[l][a] = W[l][a] exp(k5 at_a) is formed here (the FP32 operations of the lead-field kernel's
// W'), with W the moved rows' field Wm [S][L][apad] for l < wrows and the resident field
// W0 [L][apad] for the others.
constexpr int CB_THREADS = 256, CB_LB = 16, CB_CAP = CONTRACT_BAND_CAP;
// dynamic shared memory of a block with NLB leads: W' [CB_CAP][NLB], the activation times, the
// band passes' partial sums [CB_THREADS][NLB + 1]; five blocks per SM fit up to 12 leads
constexpr size_t cb_smem_bytes(int nlb) {
    return (size_t)CB_CAP * nlb * 4 + (size_t)CB_CAP * 8 + (size_t)CB_THREADS * (nlb + 1) * 4;
}
template <int NLB>
__global__ void __launch_bounds__(CB_THREADS, NLB <= 12 ? 5 : 4) k_contract_band(
    int steps, int nleads, int64_t apad, int nl, const float2 *__restrict__ t_hilo, const float2 *__restrict__ at_hilo,
    const double *__restrict__ at, const int32_t *__restrict__ chunk_a0, const int32_t *__restrict__ chunk_a1,
    const int32_t *__restrict__ chunk_layer, const float *__restrict__ Wm, int wrows, const float *__restrict__ W0,
    const double *__restrict__ layer_k, const float *__restrict__ layer_c, int nchunks, int nlb,
    float *__restrict__ band, float2 *__restrict__ csum, int4 *__restrict__ cinfo) {
    extern __shared__ __align__(16) uint8_t cb_smem[];
    float(*s_w)[NLB] = reinterpret_cast<float(*)[NLB]>(cb_smem);  // W'[a][l] of the chunk
    float2 *s_at = reinterpret_cast<float2 *>(cb_smem + (size_t)CB_CAP * NLB * 4);
    float(*s_red)[NLB + 1] = reinterpret_cast<float(*)[NLB + 1]>(s_at + CB_CAP);  // [slice * rows + step]
    __shared__ float s_ext[2][CB_THREADS / 32];
    __shared__ float s_part[2][CB_THREADS / 32][(NLB + 7) / 8 * 8];
    __shared__ float s_sum[2][NLB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c = blockIdx.x;
    const int s = blockIdx.y / nlb, lb = blockIdx.y % nlb;
    const int a0 = chunk_a0[c], na = chunk_a1[c] - a0, L = chunk_layer[c];
    const int l0 = lb * NLB, nlh = min(NLB, nleads - l0);
    const float4 kc = reinterpret_cast<const float4 *>(layer_c)[(size_t)s * nl + L];
    float *out = band + ((size_t)s * nchunks + c) * nleads * (size_t)steps + (size_t)l0 * steps;
    const double k5 = layer_k[((size_t)s * nl + L) * 9 + 5];

    // the chunk: activation times, W' transposed to [a][l], the extreme finite activation times
    float amin = INFINITY, amax = -INFINITY;
    for (int i = tid; i < na; i += CB_THREADS) {
        const float2 a2 = at_hilo[a0 + i];
        s_at[i] = a2;
        if (isfinite(a2.x)) {
            amin = fminf(amin, a2.x);
            amax = fmaxf(amax, a2.x);
        }
        const double ad = at[a0 + i];
        const float f = isinf(ad) ? 0.f : expf((float)(k5 * ad));
        float w[NLB];
#pragma unroll
        for (int l = 0; l < NLB; ++l) {
            const int lg = l0 + l;
            w[l] = l >= nlh ? 0.f
                            : (lg < wrows ? Wm[((size_t)s * nleads + lg) * apad + a0 + i] : W0[(size_t)lg * apad + a0 + i]) * f;
        }
#pragma unroll
        for (int l = 0; l < NLB; l += 4)
            *reinterpret_cast<float4 *>(&s_w[i][l]) = make_float4(w[l], w[l + 1], w[l + 2], w[l + 3]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    }
    if (lane == 0) {
        s_ext[0][warp] = amin;
        s_ext[1][warp] = amax;
    }
    __syncthreads();
#pragma unroll
    for (int w = 0; w < CB_THREADS / 32; ++w) {
        amin = fminf(amin, s_ext[0][w]);
        amax = fmaxf(amax, s_ext[1][w]);
    }
    const bool any_finite = amin <= amax;
    const bool classify = any_finite && kc.x > 0.f && kc.y >= 0.f;
    int nzero = 0, nsteady = 0;
    for (int tb = 0; tb < steps; tb += CB_THREADS) {
        const int t = tb + tid;
        bool z = false, st = false;
        if (t < steps && classify) {
            const float tt = t_hilo[t].x;
            z = kc.x * (amin - tt) >= 30.5f && (kc.x - kc.y) * (amin - tt) >= 30.5f;
            st = kc.x * (tt - amax) >= 26.5f;
        }
        nzero += __syncthreads_count(z);
        nsteady += __syncthreads_count(st);
    }
    if (!any_finite) nzero = steps;
    const int tb0 = nzero, tb1 = steps - nsteady;  // band steps [tb0, tb1)
    if (lb == 0 && tid == 0) cinfo[(size_t)s * nchunks + c] = make_int4(tb0, tb1, __float_as_int(amax), 0);

    if (nsteady > 0) {
        // S0, S1 per lead: each thread its APs, then a shuffle and a shared-memory reduction (eight
        // leads at a time, which keeps the accumulators in registers)
#pragma unroll 1
        for (int lh = 0; lh < NLB; lh += 8) {
            float u0[8], u1[8];
#pragma unroll
            for (int l = 0; l < 8; ++l) u0[l] = u1[l] = 0.f;
            for (int i = tid; i < na; i += CB_THREADS) {
                const float2 a2 = s_at[i];
                if (!isfinite(a2.x)) continue;
                const float g = ex2_approx(-kc.y * ((amax - a2.x) - a2.y));
#pragma unroll
                for (int l = 0; l < 8; ++l) {
                    const float w = lh + l < NLB ? s_w[i][lh + l] : 0.f;
                    u0[l] = fmaf(w, g, u0[l]);
                    u1[l] += w;
                }
            }
            // the 16 warp sums by recursive halving: at each level a lane keeps half of its values
            // (chosen by one lane bit) and adds its partner's copy of them; 16 shuffles instead of 80
            float v[16];
#pragma unroll
            for (int l = 0; l < 8; ++l) {
                v[l] = u0[l];
                v[8 + l] = u1[l];
            }
#pragma unroll
            for (int o = 16, n = 8; o > 1; o >>= 1, n >>= 1) {
                const bool up = lane & o;
#pragma unroll
                for (int j = 0; j < n; ++j) {
                    const float keep = up ? v[j + n] : v[j], give = up ? v[j] : v[j + n];
                    v[j] = keep + __shfl_xor_sync(0xffffffffu, give, o);
                }
            }
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
            // lane holds value 8 b4 + 4 b3 + 2 b2 + b1 (b_i its lane bits): (S0 or S1, lead)
            const int idx = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
            if (!(lane & 1)) s_part[idx >> 3][warp][lh + (idx & 7)] = v[0];
        }
        __syncthreads();
        if (tid < 2 * NLB) {
            const int k = tid / NLB, l = tid % NLB;
            float v = 0.f;
            for (int w = 0; w < CB_THREADS / 32; ++w) v += s_part[k][w][l];
            s_sum[k][l] = v;
        }
        __syncthreads();
        if (tid < nlh) csum[((size_t)s * nchunks + c) * nleads + l0 + tid] = make_float2(s_sum[0][tid], s_sum[1][tid]);
    }

    // band: passes of 32, 16 or 8 steps (the fewest steps that cover the run), lane = step.  The
    // chunk's APs are dealt round-robin to 256 / rows slices (slice j takes APs j, j + nsl, ...);
    // the 8 lanes of a quarter warp share one slice, so the W' reads are broadcasts.
    // With T the chunk's first (smallest) activation time the two exponentials separate,
    //     2^(-k' (t - at)) = 2^(-k' (t - T)) 2^(k' (at - T)),
    // one factor per step and one per AP (replacing the AP time in shared memory), which leaves one
    // SFU operation (the sigmoid's reciprocal) per (AP, step).  Taken while the per-AP factors stay
    // below 2^64: the band steps end within 26.5 / k1' of amax, so the per-step factors stay above
    // 2^-100 (no underflow) and the exponents' rounding stays that of the direct form's.
    if (tb0 >= tb1) return;
    const float2 T = s_at[0];
    const bool sep = classify && kc.x * (amax - T.x) < 64.f && kc.y * (amax - T.x) < 64.f;
    float2 *s_g = s_at;
    if (sep) {
        __syncthreads();  // every read of s_at above is done
        for (int i = tid; i < na; i += CB_THREADS) {
            const float2 a2 = s_at[i];
            float2 g = make_float2(INFINITY, 0.f);  // H = 0 (no activation)
            if (isfinite(a2.x)) {
                const float d = (a2.x - T.x) + (a2.y - T.y);
                g = make_float2(ex2_approx(kc.x * d), ex2_approx(kc.y * d));
            }
            s_g[i] = g;
        }
        __syncthreads();
    }
    for (int tb = tb0; tb < tb1;) {
        const int rem = tb1 - tb;
        const int rows = rem > 24 ? 32 : (rem > 8 ? 16 : 8);
        const int nsl = CB_THREADS / rows, r = lane & (rows - 1), sl = warp * (32 / rows) + lane / rows;
        const float2 th = t_hilo[min(tb + r, steps - 1)];
        float acc[NLB];
#pragma unroll
        for (int l = 0; l < NLB; ++l) acc[l] = 0.f;
        if (sep) {
            const float d = (th.x - T.x) + (th.y - T.y);
            const float E1 = ex2_approx(-kc.x * d), E4 = ex2_approx(-kc.y * d);
            for (int i = sl; i < na; i += nsl) {
                const float2 g = s_g[i];
                const float sg = rcp_approx(fmaf(E1, g.x, 1.0f));
                const float hv = sg * fmaf(kc.z, E4 * g.y, kc.w);
                const float h = sg == 0.f ? 0.f : hv;
#pragma unroll
                for (int l = 0; l < NLB; l += 4) {
                    const float4 w = *reinterpret_cast<const float4 *>(&s_w[i][l]);
                    acc[l] = fmaf(w.x, h, acc[l]);
                    acc[l + 1] = fmaf(w.y, h, acc[l + 1]);
                    acc[l + 2] = fmaf(w.z, h, acc[l + 2]);
                    acc[l + 3] = fmaf(w.w, h, acc[l + 3]);
                }
            }
        } else {
            for (int i = sl; i < na; i += nsl) {
                const float2 a2 = s_at[i];
                const float h = h_value(((th.x - a2.x) + (th.y - a2.y)), kc);
#pragma unroll
                for (int l = 0; l < NLB; l += 4) {
                    const float4 w = *reinterpret_cast<const float4 *>(&s_w[i][l]);
                    acc[l] = fmaf(w.x, h, acc[l]);
                    acc[l + 1] = fmaf(w.y, h, acc[l + 1]);
                    acc[l + 2] = fmaf(w.z, h, acc[l + 2]);
                    acc[l + 3] = fmaf(w.w, h, acc[l + 3]);
                }
            }
        }
#pragma unroll
        for (int l = 0; l < NLB; ++l) s_red[sl * rows + r][l] = acc[l];
        __syncthreads();
        for (int i = tid; i < rows * NLB; i += CB_THREADS) {
            const int l = i / rows, rr = i % rows, t = tb + rr;
            float v = 0.f;
            for (int w = 0; w < nsl; ++w) v += s_red[w * rows + rr][l];
            if (t < tb1 && l < nlh) out[(size_t)l * steps + t] = v;
        }
        __syncthreads();
        tb += rows;
    }
}

// ecg[s][l][t] = k0w[s][l] + sum_L F_L(t) sum_{c in L} P_c[l][t] from the band contraction's
// compact outputs: warp per (simulation, lead, 32 steps), lane = step.  Within a layer the APs
// ascend in activation time, so the chunks' tb0 and tb1 ascend with the chunk index.  Per layer:
//   - the chunks steady over the whole tile (tb1 <= t0, a prefix of the layer's chunks) are
//     summed once for the tile, lanes over chunks then a fixed-order tree,
//         A = sum_c 2^(-k4'(t0 - amax_c)) S0_c,   B = sum_c S1_c,
//     and enter step t as (1 - k3) 2^(-k4'(t - t0)) A + k3 B;
//   - the following chunks are taken per step (band value, steady formula or zero) up to the
//     first one whose zero run covers the tile (every later chunk's does too).
// The layer's sum is float-float, times F_L(t) in FP64; the chunk order is fixed, so the result
// does not depend on scheduling.  Also writes the float-float copy.
__global__ void __launch_bounds__(512) k_reduce_chunks(
    int steps, int nleads, int nl, int nchunks, const int32_t *__restrict__ layer_c0, const int32_t *__restrict__ layer_c1,
    const float2 *__restrict__ t_hilo, const float *__restrict__ layer_c, const double *__restrict__ F,
    const float *__restrict__ band, const float2 *__restrict__ csum, const int4 *__restrict__ cinfo,
    const double *__restrict__ k0w, double *__restrict__ ecg, float2 *__restrict__ ecg_ff) {
    const int lane = threadIdx.x & 31;
    const int l = blockIdx.z * 16 + (threadIdx.x >> 5), s = blockIdx.y;
    const int t0 = blockIdx.x * 32, t = t0 + lane;
    if (l >= nleads) return;  // warps are independent: no block-wide barrier below
    const bool valid = t < steps;
    const float2 th0 = t_hilo[t0], th = t_hilo[valid ? t : steps - 1];
    const int4 *ci = cinfo + (size_t)s * nchunks;
    const float2 *cs = csum + (size_t)s * nchunks * nleads;
    const float *bd = band + (size_t)s * nchunks * nleads * (size_t)steps + (size_t)l * steps;
    double acc = 0.0;
    for (int L = 0; L < nl; ++L) {
        const int c0 = layer_c0[L], c1 = layer_c1[L];
        if (c0 >= c1) continue;
        const float4 kc = reinterpret_cast<const float4 *>(layer_c)[(size_t)s * nl + L];
        // the steady prefix [c0, clo): clo = the first chunk with tb1 > t0
        int clo = c1;
        for (int cb = c0; cb < c1; cb += 32) {
            const unsigned m = __ballot_sync(0xffffffffu, cb + lane < c1 && ci[cb + lane].y > t0);
            if (m) {
                clo = cb + __ffs(m) - 1;
                break;
            }
        }
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
        for (int c = c0 + lane; c < clo; c += 32) {
            const float2 sv = cs[(size_t)c * nleads + l];
            const float g = ex2_approx(-kc.y * ((th0.x - __int_as_float(ci[c].z)) + th0.y));
            A = ff_add_f(A, g * sv.x);
            B = ff_add_f(B, sv.y);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float2 a2 = make_float2(__shfl_down_sync(0xffffffffu, A.x, o), __shfl_down_sync(0xffffffffu, A.y, o));
            const float2 b2 = make_float2(__shfl_down_sync(0xffffffffu, B.x, o), __shfl_down_sync(0xffffffffu, B.y, o));
            A = ff_add(A, a2);
            B = ff_add(B, b2);
        }
        A = make_float2(__shfl_sync(0xffffffffu, A.x, 0), __shfl_sync(0xffffffffu, A.y, 0));
        B = make_float2(__shfl_sync(0xffffffffu, B.x, 0), __shfl_sync(0xffffffffu, B.y, 0));
        const float e0 = kc.z * ex2_approx(-kc.y * ((th.x - th0.x) + (th.y - th0.y)));
        float2 sum = ff_add(ff_mul(make_float2(e0, 0.f), A), ff_mul(make_float2(kc.w, 0.f), B));
        // the chunks after the prefix, per step; the lanes load 32 chunks' run limits and steady sums
        // at once (one coalesced load each) and pass them round by shuffles
        bool done = false;
        for (int cb = clo; cb < c1 && !done; cb += 32) {
            const int cc = cb + lane;
            const int4 mine = cc < c1 ? ci[cc] : make_int4(steps, steps, 0, 0);
            const float2 smine = cc < c1 ? cs[(size_t)cc * nleads + l] : make_float2(0.f, 0.f);
            const int nj = min(32, c1 - cb);
#pragma unroll 4
            for (int j = 0; j < nj; ++j) {
                const int tb0 = __shfl_sync(0xffffffffu, mine.x, j), tb1 = __shfl_sync(0xffffffffu, mine.y, j);
                const float am = __int_as_float(__shfl_sync(0xffffffffu, mine.z, j));
                const float s0 = __shfl_sync(0xffffffffu, smine.x, j), s1 = __shfl_sync(0xffffffffu, smine.y, j);
                if (tb0 >= t0 + 32) {  // this chunk and every later one are zero over the tile
                    done = true;
                    break;
                }
                if (valid && t >= tb0) {
                    float v;
                    if (t < tb1) {
                        v = bd[(size_t)(cb + j) * nleads * steps + t];
                    } else {
                        const float e = kc.z * ex2_approx(-kc.y * ((th.x - am) + th.y));
                        v = fmaf(e, s0, kc.w * s1);
                    }
                    sum = ff_add_f(sum, v);
                }
            }
        }
        if (valid) acc = fma(ff_to_double(sum), F[((size_t)s * nl + L) * steps + t], acc);
    }
    if (valid) {
        const double r = k0w[(size_t)s * nleads + l] + acc;
        const size_t o = ((size_t)s * nleads + l) * steps + t;
        ecg[o] = r;
        ecg_ff[o] = ff_from_double(r);
    }
}

// ecg[s][l][t] = k0w[s][l] + sum_c partial[s][c][l][t]: one block per (s, l, 32 steps); warp w
// sums chunks c = w, w+8, ... for 32 consecutive steps (coalesced), then the 8 warp sums are added
// in warp order, so the result does not depend on scheduling.  Also writes the float-float copy.
__global__ void __launch_bounds__(256) k_reduce_ecg(int steps, int nleads, int nchunks,
                                                    const double *__restrict__ partial,
                                                    const double *__restrict__ k0w, double *__restrict__ ecg,
                                                    float2 *__restrict__ ecg_ff) {
    __shared__ double red[8][33];
    const int tt = blockIdx.x * 32 + (threadIdx.x & 31);
    const int w = threadIdx.x >> 5;
    const int l = blockIdx.y, s = blockIdx.z;
    double acc = 0.0;
    // the additions stay in chunk order; unrolling lets four loads be in flight at once
    if (tt < steps)
#pragma unroll 4
        for (int c = w; c < nchunks; c += 8) acc += partial[(((size_t)s * nchunks + c) * nleads + l) * steps + tt];
    red[w][threadIdx.x & 31] = acc;
    __syncthreads();
    if (w == 0 && tt < steps) {
        double r = k0w[(size_t)s * nleads + l];
        for (int i = 0; i < 8; ++i) r += red[i][threadIdx.x];
        const size_t o = ((size_t)s * nleads + l) * steps + tt;
        ecg[o] = r;
        ecg_ff[o] = ff_from_double(r);
    }
}

// ------------------------------------------------------------------ criteria
// Output per (s, i): value and argmax.
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// Block-wide reductions for the criteria (NT threads): a warp butterfly, then lane 0 of each warp
// in warp order, so every thread gets the same value in a fixed order.  `red` is shared scratch of
// NT / 32 entries.
template <int NT>
__device__ __forceinline__ double block_sum_ff(float2 v, float2 *red) {
    constexpr int CR_WARPS = NT / 32;
    for (int o = 16; o > 0; o >>= 1) {
        const float2 w = make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
        v = ff_add(v, w);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float2 t = red[0];
    for (int k = 1; k < CR_WARPS; ++k) t = ff_add(t, red[k]);
    return ff_to_double(t);
}
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *red) {
    constexpr int CR_WARPS = NT / 32;
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = red[0];
    for (int k = 1; k < CR_WARPS; ++k) t += red[k];
    return t;
}
template <int NT>
__device__ __forceinline__ double block_minmax(double v, bool is_max, double *red) {
    constexpr int CR_WARPS = NT / 32;
    v = is_max ? warp_max(v) : warp_min(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = red[0];
    for (int k = 1; k < CR_WARPS; ++k) t = is_max ? fmax(t, red[k]) : fmin(t, red[k]);
    return t;
}
__device__ __forceinline__ bool ff_greater(float2 a, float2 b) { return a.x > b.x || (a.x == b.x && a.y > b.y); }

// One block of NT threads per (simulation, criterion lead): threads stride over the steps, sums
// combined in a fixed order (one warp per pair when there are many pairs, four for few).  Pearson, vector correlation and RMS accumulate in float-float (about
// 48 significant bits) on the FP32 pipe, reading the float-float copies of the ECG and targets;
// the few closing operations (means, square roots, quotients) are FP64.  devFromLinear stays FP64
// throughout.  Writes the criterion value and the argmax (first maximum) of the lead.
template <int NT>
__global__ void __launch_bounds__(NT) k_criteria(int steps, int nleads, int i0, int i1, int n_sims, int mode,
                                                         const double *__restrict__ ecg,
                                                         const float2 *__restrict__ ecg_ff,
                                                         const double *__restrict__ targets,
                                                         const float2 *__restrict__ targets_ff,
                                                         const int64_t *__restrict__ tlen,
                                                         const double *__restrict__ toff, int crit_stride,
                                                         double *__restrict__ crit) {
    constexpr int CR_THREADS = NT, CR_WARPS = NT / 32;
    __shared__ float2 redf[CR_WARPS];
    __shared__ double redd[CR_WARPS];
    __shared__ int redi[CR_WARPS];
    const int tid = threadIdx.x;
    const int ni = i1 - i0;  // criterion leads [i0, i1) of this launch
    const int i = i0 + (int)(blockIdx.x % ni), s = (int)(blockIdx.x / ni);
    const size_t row = ((size_t)s * nleads + i) * steps;
    const float2 *af = ecg_ff + row;
    int64_t off = 0;
    for (int j = 0; j < i; ++j) off += tlen[j];
    const float2 *bf = targets_ff + off;
    const int64_t nb = tlen[i];
    const int64_t len = steps < nb ? steps : nb;
    const double inv = 1.0 / (double)len;
    double value = 0.0;
    if (mode == 2) {
        float2 sa = make_float2(0.f, 0.f), sb = sa;
        for (int64_t j = tid; j < len; j += CR_THREADS) {
            sa = ff_add(sa, af[j]);
            sb = ff_add(sb, bf[j]);
        }
        const float2 ma = ff_neg(ff_from_double(block_sum_ff<NT>(sa, redf) * inv));
        const float2 mb = ff_neg(ff_from_double(block_sum_ff<NT>(sb, redf) * inv));
        float2 va = make_float2(0.f, 0.f), vb = va, cv = va;
        for (int64_t j = tid; j < len; j += CR_THREADS) {
            const float2 x = ff_add(af[j], ma), y = ff_add(bf[j], mb);
            va = ff_add(va, ff_mul(x, x));
            vb = ff_add(vb, ff_mul(y, y));
            cv = ff_add(cv, ff_mul(x, y));
        }
        const double dva = block_sum_ff<NT>(va, redf) * inv, dvb = block_sum_ff<NT>(vb, redf) * inv;
        const double dcv = block_sum_ff<NT>(cv, redf) / (double)len;
        value = 1.0 - dcv / (sqrt(dva) * sqrt(dvb));
    } else if (mode == 4) {
        float2 ab = make_float2(0.f, 0.f), aa = ab, bb = ab;
        for (int64_t j = tid; j < len; j += CR_THREADS) {
            const float2 x = af[j], y = bf[j];
            ab = ff_add(ab, ff_mul(x, y));
            aa = ff_add(aa, ff_mul(x, x));
            bb = ff_add(bb, ff_mul(y, y));
        }
        const double dab = block_sum_ff<NT>(ab, redf), daa = block_sum_ff<NT>(aa, redf), dbb = block_sum_ff<NT>(bb, redf);
        value = 1.0 - dab / (sqrt(daa) * sqrt(dbb));
    } else if (mode == 1) {
        float2 q = make_float2(0.f, 0.f);
        for (int64_t j = tid; j < len; j += CR_THREADS) {
            const float2 x = ff_add(af[j], ff_neg(bf[j]));
            q = ff_add(q, ff_mul(x, x));
        }
        value = sqrt(block_sum_ff<NT>(q, redf) / (double)len);
    } else {
        // devFromLinear (vectorMath.h:373-404): min/max over the whole simulated lead
        const double *a = ecg + row;
        const double *b = targets + off;
        double mn = INFINITY, mx = -INFINITY;
        for (int64_t j = tid; j < steps; j += CR_THREADS) {
            mn = fmin(mn, a[j]);
            mx = fmax(mx, a[j]);
        }
        const double amax = block_minmax<NT>(mx, true, redd);
        const double amin = block_minmax<NT>(mn, false, redd);
        const double amult = 1.0 / (amax - amin);
        const double bofs = toff[i];
        double sd = 0;
        for (int64_t j = tid; j < len; j += CR_THREADS) sd += (a[j] * amult + bofs) / (b[j] + bofs);
        const double mean = block_sum<NT>(sd, redd) * inv;
        double var = 0;
        for (int64_t j = tid; j < len; j += CR_THREADS) {
            const double d = (a[j] * amult + bofs) / (b[j] + bofs) - mean;
            var += d * d;
        }
        var = block_sum<NT>(var, redd) * inv;
        value = (var == 0) ? 1.0 / 1e-30 : sqrt(var);
    }
    // argmax of the simulated lead (first maximum), for the peak-position criterion; float-float
    // values are normalised, so comparing (hi, lo) in order compares the values
    float2 best = make_float2(-INFINITY, 0.f);
    int arg = 0x7fffffff;
    for (int j = tid; j < steps; j += CR_THREADS) {
        const float2 v = af[j];
        if (ff_greater(v, best)) {
            best = v;
            arg = j;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float2 v2 = make_float2(__shfl_xor_sync(0xffffffffu, best.x, o), __shfl_xor_sync(0xffffffffu, best.y, o));
        const int a2 = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ff_greater(v2, best) || (v2.x == best.x && v2.y == best.y && a2 < arg)) {
            best = v2;
            arg = a2;
        }
    }
    __syncthreads();
    if ((tid & 31) == 0) {
        redf[tid >> 5] = best;
        redi[tid >> 5] = arg;
    }
    __syncthreads();
    if (tid == 0) {
        for (int k = 1; k < CR_WARPS; ++k)
            if (ff_greater(redf[k], best) || (redf[k].x == best.x && redf[k].y == best.y && redi[k] < arg)) {
                best = redf[k];
                arg = redi[k];
            }
        crit[((size_t)s * crit_stride + i) * 2 + 0] = value;
        crit[((size_t)s * crit_stride + i) * 2 + 1] = (double)arg;
    }
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launch_lead_field(cudaStream_t s, const HeartDev &h, const double *d_leads, int nleads_in, int lead_stride,
                       int n_sims, float *d_W, int w_lead_stride) {
    dim3 grid((unsigned)((h.apad + 127) / 128), (unsigned)nleads_in, (unsigned)n_sims);
    k_lead_field<<<grid, 128, 0, s>>>(h.apad, h.a_vox_begin.p, h.vox_zyx.p, h.vox_nb.p, h.vox_nbo.p, h.nnb,
                                      h.difs.p, d_leads, nleads_in, lead_stride, d_W, w_lead_stride);
    EKG_CUDA(cudaGetLastError());
}

void launch_layer_factors(cudaStream_t s, const HeartDev &h, const double *d_layer_k, const double *d_cpre,
                          int n_sims, double *d_F, float *d_Ff, float *d_layer_c, const double *d_centre,
                          const double *d_scale, int J, float *d_coef) {
    k_layer_factors<<<(unsigned)((int64_t)n_sims * h.nlayers), 128, 0, s>>>(
        h.nlayers, h.steps, h.t.p, d_layer_k, d_cpre, n_sims, d_F, d_Ff, d_layer_c, d_centre, d_scale, J, d_coef);
    EKG_CUDA(cudaGetLastError());
}

void launch_k0_term(cudaStream_t s, const HeartDev &h, const float *d_W, const double *d_layer_k, int n_sims,
                    double *d_k0w, int rows) {
    dim3 grid((unsigned)rows, (unsigned)n_sims);
    k_k0_term<<<grid, 256, 0, s>>>(h.apad, h.nleads, d_W, h.a_layer.p, d_layer_k, h.nlayers, d_k0w);
    EKG_CUDA(cudaGetLastError());
}

void launch_contract_cuda(cudaStream_t s, const HeartDev &h, const float *d_Wp, const float *d_layer_c,
                          const double *d_F, int n_sims, double *d_partial) {
    const int nlb = (h.nleads + CC_LB - 1) / CC_LB;
    dim3 grid((unsigned)((h.steps + CC_T - 1) / CC_T), (unsigned)h.nchunks, (unsigned)(n_sims * nlb));
    k_contract_cuda<<<grid, CC_T, 0, s>>>(h.steps, h.nleads, h.apad, h.nlayers, h.t_hilo.p, h.at_hilo.p,
                                          h.chunk_a0.p, h.chunk_a1.p, h.chunk_layer.p, d_Wp, d_layer_c, d_F,
                                          h.nchunks, nlb, d_partial);
    EKG_CUDA(cudaGetLastError());
}

void launch_contract_band(cudaStream_t s, const HeartDev &h, const float *d_Wm, int wrows, const float *d_W0,
                          const double *d_layer_k, const float *d_layer_c, int n_sims, float *d_band, float2 *d_csum,
                          int4 *d_cinfo) {
    static bool attr = false;
    if (!attr) {
        EKG_CUDA(cudaFuncSetAttribute(k_contract_band<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cb_smem_bytes(4)));
        EKG_CUDA(cudaFuncSetAttribute(k_contract_band<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cb_smem_bytes(8)));
        EKG_CUDA(cudaFuncSetAttribute(k_contract_band<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cb_smem_bytes(12)));
        EKG_CUDA(cudaFuncSetAttribute(k_contract_band<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cb_smem_bytes(16)));
        attr = true;
    }
    // leads per block: all of them rounded up to a multiple of 4 when there are at most 16, else
    // blocks of 16
    const int nlr = h.nleads > CB_LB ? CB_LB : (h.nleads + 3) / 4 * 4;
    const int nlb = (h.nleads + nlr - 1) / nlr;
    dim3 grid((unsigned)h.nchunks, (unsigned)(n_sims * nlb));
    auto go = [&](auto kern, int nl_block) {
        kern<<<grid, CB_THREADS, cb_smem_bytes(nl_block), s>>>(h.steps, h.nleads, h.apad, h.nlayers, h.t_hilo.p, h.at_hilo.p, h.at.p,
                                              h.chunk_a0.p, h.chunk_a1.p, h.chunk_layer.p, d_Wm, wrows, d_W0,
                                              d_layer_k, d_layer_c, h.nchunks, nlb, d_band, d_csum, d_cinfo);
    };
    if (nlr == 4) go(k_contract_band<4>, 4);
    else if (nlr == 8) go(k_contract_band<8>, 8);
    else if (nlr == 12) go(k_contract_band<12>, 12);
    else go(k_contract_band<16>, 16);
    EKG_CUDA(cudaGetLastError());
}

void launch_reduce_chunks(cudaStream_t s, const HeartDev &h, const float *d_layer_c, const double *d_F,
                          const float *d_band, const float2 *d_csum, const int4 *d_cinfo, const double *d_k0w,
                          int n_sims, double *d_ecg, float2 *d_ecg_ff) {
    const int nlb = (h.nleads + 15) / 16;
    dim3 grid((unsigned)((h.steps + 31) / 32), (unsigned)n_sims, (unsigned)nlb);
    k_reduce_chunks<<<grid, 32 * std::min(16, h.nleads), 0, s>>>(h.steps, h.nleads, h.nlayers, h.nchunks,
                                                                 h.layer_c0.p, h.layer_c1.p, h.t_hilo.p, d_layer_c, d_F,
                                                                 d_band, d_csum, d_cinfo, d_k0w, d_ecg, d_ecg_ff);
    EKG_CUDA(cudaGetLastError());
}

void launch_reduce_ecg(cudaStream_t s, const HeartDev &h, const double *d_partial, const double *d_k0w,
                       int n_sims, double *d_ecg, float2 *d_ecg_ff) {
    dim3 grid((unsigned)((h.steps + 31) / 32), (unsigned)h.nleads, (unsigned)n_sims);
    k_reduce_ecg<<<grid, 256, 0, s>>>(h.steps, h.nleads, h.nchunks, d_partial, d_k0w, d_ecg, d_ecg_ff);
    EKG_CUDA(cudaGetLastError());
}

void launch_criteria(cudaStream_t s, const HeartDev &h, const double *d_ecg, const float2 *d_ecg_ff, int n_sims,
                     int ncrit_stride, int i0, int i1, int mode, const double *d_targets, const float2 *d_targets_ff,
                     const int64_t *d_tlen, const double *d_toff, double *d_crit) {
    if (i1 <= i0) return;
    // one block per (simulation, lead): a warp when the pairs fill the GPU, four warps when few
    const int64_t pairs = (int64_t)(i1 - i0) * n_sims;
    if (pairs >= 1024)
        k_criteria<32><<<(unsigned)pairs, 32, 0, s>>>(h.steps, h.nleads, i0, i1, n_sims, mode, d_ecg, d_ecg_ff,
                                                      d_targets, d_targets_ff, d_tlen, d_toff, ncrit_stride, d_crit);
    else
        k_criteria<128><<<(unsigned)pairs, 128, 0, s>>>(h.steps, h.nleads, i0, i1, n_sims, mode, d_ecg, d_ecg_ff,
                                                        d_targets, d_targets_ff, d_tlen, d_toff, ncrit_stride, d_crit);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace ekg
