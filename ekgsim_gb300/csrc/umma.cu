// umma.cu -- the lead contraction on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// For one simulation and one K chunk (a range of de-duplicated APs inside one layer L) the CTA
// walks the tiles of 128 time steps and computes
//     P[t, l] = sum_a H_a(t) W'[l, a]        (M = 128 steps, N = leads padded to 16..256, K = APs)
// and writes partial[s][chunk][l][t] = P[t, l] * F_L(t) in FP64.  Tiles before the chunk's
// upstrokes are zero and tiles after them separate into two per-lead sums over the chunk; the
// tiles in between (the band) go through the tensor cores.  H_a(t) (see ecg.cu) is evaluated
// in FP32 by all 256 threads straight into shared memory, split into BF16 hi + lo parts, as the A
// operand; W' (FP32 in HBM) is split the same way as the B operand.  One elected thread issues
// three MMAs per 16-wide K step (hi*hi, hi*lo, lo*hi) into an FP32 accumulator in tensor memory;
// a two-stage shared-memory ring lets the producers fill stage k+1 while the tensor core consumes
// stage k, tracked by an mbarrier per stage that tcgen05.commit arrives on.
//
// Operand layout: K-major, no swizzle.  A core matrix is 8 rows x 16 bytes (8 BF16 along K),
// stored contiguously; core matrix (row group g, K chunk c) sits at byte (c * G + g) * 128 for a
// tile of G row groups, so the descriptor's leading byte offset (next core matrix along K) is
// G * 128 and its stride byte offset (next 8-row group) is 128.
//
// Every mbarrier wait is bounded: on timeout the CTA records KERR_MBAR_TIMEOUT in the error word,
// waits (bounded) for the last commit, releases its tensor memory and skips its remaining tiles.
#include <cuda_bf16.h>
#include <cstdio>

#include "ekg_internal.h"
#include "umma_ptx.h"

namespace ekg {

namespace {

constexpr int UM_M = 128;       // time steps per tile
constexpr int UM_KT = 64;       // APs per pipeline stage (4 MMA K steps)
constexpr int UM_THREADS = 256;
constexpr int STEADY_CAP = 4096;  // APs per chunk up to which a steady block stages its AP factors

using namespace ptx;

template <int N>
struct UmmaSmem {
    // two stages; A: 128 x 64 BF16 = 16 KB per part; B: N x 64 BF16 per part
    alignas(1024) uint8_t a_hi[2][UM_M * UM_KT * 2];
    alignas(1024) uint8_t a_lo[2][UM_M * UM_KT * 2];
    alignas(1024) uint8_t b_hi[2][N * UM_KT * 2];
    alignas(1024) uint8_t b_lo[2][N * UM_KT * 2];
    float2 at[2][UM_KT];
    float sums[2][N];                // steady tiles: per-lead sums of W' 2^(-k4' (tref - at)) and of W'
    float ext[2][UM_THREADS / 32];   // per-warp earliest / latest activation time of the chunk
    alignas(8) uint64_t bar[2];
    uint32_t tmem_base;
};

template <int N>
__global__ void __launch_bounds__(UM_THREADS, 1) k_contract_umma(
    int steps, int nleads, int64_t apad, int nl, const float2 *__restrict__ t_hilo, const float2 *__restrict__ at_hilo,
    const int32_t *__restrict__ chunk_a0, const int32_t *__restrict__ chunk_a1, const int32_t *__restrict__ chunk_layer,
    const float *__restrict__ Wp, const float *__restrict__ layer_c, const double *__restrict__ F, int nchunks,
    int nlb, double *__restrict__ partial, uint32_t *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    UmmaSmem<N> &S = *reinterpret_cast<UmmaSmem<N> *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr uint32_t TCOLS = N < 32 ? 32 : N;
    constexpr uint32_t IDESC = idesc_bf16(UM_M, N);
    constexpr uint32_t A_LBO = (UM_M / 8) * 128, A_SBO = 128;
    constexpr uint32_t B_LBO = (N / 8) * 128, B_SBO = 128;
    constexpr float STEADY_X = 26.5f, ZERO_X = 30.5f;
    constexpr int NW = UM_THREADS / 32;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c = blockIdx.x;
    const int s = blockIdx.y / nlb, lb = blockIdx.y % nlb;
    const int a0 = chunk_a0[c], a1 = chunk_a1[c], L = chunk_layer[c];
    const int l0 = lb * N;
    const int ntiles = (steps + UM_M - 1) / UM_M;
    const float4 kc = reinterpret_cast<const float4 *>(layer_c)[(size_t)s * nl + L];
    double *out = partial + ((size_t)s * nchunks + c) * nleads * (size_t)steps;
    const double *Fl = F + ((size_t)s * nl + L) * steps;

    // Tiles away from the chunk's upstrokes skip the contraction.  From the chunk's earliest and
    // latest finite activation times: when every (step, AP) pair of a tile has k1 tau log2(e) >=
    // STEADY_X the sigmoid is 1 in FP32 and H_a(t) = (1 - k3) 2^(-k4' (t - tref)) 2^(-k4' (tref -
    // at_a)) + k3 separates into two sums over the chunk per lead (steady tile); when every pair lies
    // before the upstroke by (k1 - k4) |tau| log2(e) >= ZERO_X and k1 |tau| log2(e) >= ZERO_X, H is
    // below 2^-30 of its amplitude and the tile is zero (the batched form's truncation).  APs with an
    // infinite activation time (unreached cells, padding) contribute nothing.  As t grows the tiles
    // run zero*, band*, steady*; only band tiles go through the tensor-core pipeline.
    float amin = INFINITY, amax = -INFINITY;
    for (int a = a0 + tid; a < a1; a += UM_THREADS) {
        const float x = at_hilo[a].x;
        if (isfinite(x)) {
            amin = fminf(amin, x);
            amax = fmaxf(amax, x);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    }
    if (lane == 0) {
        S.ext[0][warp] = amin;
        S.ext[1][warp] = amax;
    }
    __syncthreads();
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        amin = fminf(amin, S.ext[0][w]);
        amax = fmaxf(amax, S.ext[1][w]);
    }
    const bool any_finite = amin <= amax;
    const bool classify = any_finite && kc.x > 0.f && kc.y >= 0.f;
    int nzero = 0, nsteady = 0;
    for (int jb = 0; jb < ntiles; jb += UM_THREADS) {
        const int j = jb + tid;
        bool z = false, st = false;
        if (j < ntiles && classify) {
            const float tf = t_hilo[j * UM_M].x, tl = t_hilo[min(j * UM_M + UM_M - 1, steps - 1)].x;
            z = kc.x * (amin - tl) >= ZERO_X && (kc.x - kc.y) * (amin - tl) >= ZERO_X;
            st = kc.x * (tf - amax) >= STEADY_X && a1 - a0 <= STEADY_CAP;
        }
        nzero += __syncthreads_count(z);
        nsteady += __syncthreads_count(st);
    }
    if (!any_finite) nzero = ntiles;
    const int jb0 = nzero, jb1 = ntiles - nsteady;  // band tiles [jb0, jb1)

    for (int i = tid; i < jb0 * UM_M * N; i += UM_THREADS) {
        const int t = (i / (UM_M * N)) * UM_M + (i & (UM_M - 1)), l = l0 + (i / UM_M) % N;
        if (t < steps && l < nleads) out[(size_t)l * steps + t] = 0.0;
    }
    if (nsteady > 0) {
        // the AP factors 2^(-k4' (tref - at_a)) and finiteness masks staged in the A ring (not yet
        // in use), the per-lead sums in S.sums
        float *s_g = reinterpret_cast<float *>(S.a_hi[0]);
        float *s_m = s_g + STEADY_CAP;
        const float tref = amax;
        const int na = a1 - a0;
        for (int i = tid; i < na; i += UM_THREADS) {
            const float2 at = at_hilo[a0 + i];
            const bool fin = isfinite(at.x);
            s_g[i] = fin ? ex2_approx(-kc.y * ((tref - at.x) - at.y)) : 0.f;
            s_m[i] = fin ? 1.f : 0.f;
        }
        __syncthreads();
        // one lead per warp at a time, four APs per lane and load
        for (int n = warp; n < N && l0 + n < nleads; n += NW) {
            const float *w = Wp + ((size_t)s * nleads + l0 + n) * apad + a0;
            float u0 = 0.f, u1 = 0.f;
#pragma unroll 4
            for (int i = 4 * lane; i < na; i += 128) {
                const float4 wa = __ldg(reinterpret_cast<const float4 *>(w + i));
                const float4 g = *reinterpret_cast<const float4 *>(s_g + i);
                const float4 m = *reinterpret_cast<const float4 *>(s_m + i);
                u0 = fmaf(wa.x, g.x, fmaf(wa.y, g.y, fmaf(wa.z, g.z, fmaf(wa.w, g.w, u0))));
                u1 = fmaf(wa.x, m.x, fmaf(wa.y, m.y, fmaf(wa.z, m.z, fmaf(wa.w, m.w, u1))));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                u0 += __shfl_xor_sync(0xffffffffu, u0, o);
                u1 += __shfl_xor_sync(0xffffffffu, u1, o);
            }
            if (lane == 0) {
                S.sums[0][n] = u0;
                S.sums[1][n] = u1;
            }
        }
        __syncthreads();
        for (int t = jb1 * UM_M + (tid & (UM_M - 1)); t < steps; t += UM_M) {
            const float2 th = t_hilo[t];
            const float e = kc.z * ex2_approx(-kc.y * ((th.x - tref) + th.y));
            const double f = Fl[t];
            for (int n = tid / UM_M; n < N; n += UM_THREADS / UM_M) {
                const int l = l0 + n;
                if (l < nleads) out[(size_t)l * steps + t] = (double)fmaf(e, S.sums[0][n], kc.w * S.sums[1][n]) * f;
            }
        }
    }
    if (jb0 >= jb1) return;

    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
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

    // producer roles: row (time step) and half of the 64-wide K stage
    const int row = tid & (UM_M - 1), half = tid >> 7;
    const int nkt = (a1 - a0) / UM_KT;
    // B operand W'[l][a] (N rows l, 64 a's; thread -> (row n, 8-wide K chunk)) and the stage's
    // activation times: loaded into registers one stage ahead, so that the global loads of stage
    // k+1 are in flight while the producers evaluate stage k
    constexpr int BPT = (N * (UM_KT / 8) + UM_THREADS - 1) / UM_THREADS;
    float4 pw[BPT][2];
    float2 pat = make_float2(0.f, 0.f);
    auto load_stage = [&](int abase) {
        if (tid < UM_KT) pat = at_hilo[abase + tid];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tid + k * UM_THREADS;
            const int n = i % N, kcn = i / N, l = l0 + n;
            if (i < N * (UM_KT / 8) && l < nleads) {
                const float4 *src = reinterpret_cast<const float4 *>(Wp + ((size_t)s * nleads + l) * apad + abase + kcn * 8);
                pw[k][0] = __ldg(src);
                pw[k][1] = __ldg(src + 1);
            } else {
                pw[k][0] = pw[k][1] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    };
    auto store_stage = [&](int b) {
        if (tid < UM_KT) S.at[b][tid] = pat;
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tid + k * UM_THREADS;
            if (i >= N * (UM_KT / 8)) break;
            const int n = i % N, kcn = i / N;
            uint4 hv, lv;
            split2(pw[k][0].x, pw[k][0].y, hv.x, lv.x);
            split2(pw[k][0].z, pw[k][0].w, hv.y, lv.y);
            split2(pw[k][1].x, pw[k][1].y, hv.z, lv.z);
            split2(pw[k][1].z, pw[k][1].w, hv.w, lv.w);
            const uint32_t off = (uint32_t)((kcn * (N / 8) + n / 8) * 128 + (n % 8) * 16);
            *reinterpret_cast<uint4 *>(S.b_hi[b] + off) = hv;
            *reinterpret_cast<uint4 *>(S.b_lo[b] + off) = lv;
        }
    };
    bool ok = true;
    int g = 0;  // operand stages issued so far, over all band tiles of the block
    for (int j = jb0; j < jb1 && ok && nkt > 0; ++j) {
        const int t0 = j * UM_M;
        const float2 th = t_hilo[min(t0 + row, steps - 1)];
        load_stage(a0);
        for (int kt = 0; kt < nkt; ++kt, ++g) {
            const int b = g & 1;
            if (g >= 2) {
                // stage b's previous use (stage g - 2) has been consumed by the tensor core
                if (!mbar_wait(&S.bar[b], (uint32_t)(((g - 2) >> 1) & 1))) ok = false;
                if (__syncthreads_or(!ok)) {
                    ok = false;
                    break;
                }
            }
            store_stage(b);
            if (kt + 1 < nkt) load_stage(a0 + (kt + 1) * UM_KT);
            __syncthreads();  // S.at visible
            // A operand: H_a(t) for this thread's row and 32 K columns
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int kc8 = half * 4 + q;
                float hv8[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float2 at = S.at[b][kc8 * 8 + e];
                    const float tau = (th.x - at.x) + (th.y - at.y);
                    hv8[e] = h_value_fast(tau, kc);
                }
                uint4 hv, lv;
                split2(hv8[0], hv8[1], hv.x, lv.x);
                split2(hv8[2], hv8[3], hv.y, lv.y);
                split2(hv8[4], hv8[5], hv.z, lv.z);
                split2(hv8[6], hv8[7], hv.w, lv.w);
                const uint32_t off = (uint32_t)((kc8 * (UM_M / 8) + row / 8) * 128 + (row % 8) * 16);
                *reinterpret_cast<uint4 *>(S.a_hi[b] + off) = hv;
                *reinterpret_cast<uint4 *>(S.a_lo[b] + off) = lv;
            }
            fence_proxy_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const uint32_t ah = smem_u32(S.a_hi[b]), al = smem_u32(S.a_lo[b]);
                const uint32_t bh = smem_u32(S.b_hi[b]), bl = smem_u32(S.b_lo[b]);
#pragma unroll
                for (int q = 0; q < UM_KT / 16; ++q) {
                    const uint64_t dah = sdesc(ah + q * 2 * A_LBO, A_LBO, A_SBO);
                    const uint64_t dal = sdesc(al + q * 2 * A_LBO, A_LBO, A_SBO);
                    const uint64_t dbh = sdesc(bh + q * 2 * B_LBO, B_LBO, B_SBO);
                    const uint64_t dbl = sdesc(bl + q * 2 * B_LBO, B_LBO, B_SBO);
                    mma_bf16(tmem, dah, dbh, IDESC, (kt > 0 || q > 0) ? 1u : 0u);
                    mma_bf16(tmem, dah, dbl, IDESC, 1u);
                    mma_bf16(tmem, dal, dbh, IDESC, 1u);
                }
                mma_commit(&S.bar[b]);
            }
        }
        if (!ok) break;
        // the tile's last commit (MMAs complete in issue order)
        if (!mbar_wait(&S.bar[(g - 1) & 1], (uint32_t)(((g - 1) >> 1) & 1))) ok = false;
        ok = !__syncthreads_or(!ok);
        tc_fence_after();
        if (!ok) break;
        // epilogue: warp quadrant q reads TMEM lanes 32q..32q+31, column half (warp >> 2)
        const int q = warp & 3, ch = warp >> 2;
        const int t = t0 + 32 * q + lane;
        const double f = (t < steps) ? Fl[t] : 0.0;
        for (int cb = ch * (N / 2); cb < (ch + 1) * (N / 2); cb += 8) {
            float v[8];
            tmem_ld8(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)cb, v);
            if (t < steps) {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int l = l0 + cb + e;
                    if (l < nleads) out[(size_t)l * steps + t] = (double)v[e] * f;
                }
            }
        }
        // the accumulator is read before the next tile's first MMA overwrites it
        tc_fence_before();
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicOr(err, KERR_MBAR_TIMEOUT);
        // bounded wait for the last issued commit before the tensor memory is released
        if (g > 0) mbar_wait(&S.bar[(g - 1) & 1], (uint32_t)(((g - 1) >> 1) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TCOLS);
}

template <int N>
void launch_n(cudaStream_t st, const ContractArgs &A) {
    const int nlb = (A.rows + N - 1) / N;
    const size_t smem = sizeof(UmmaSmem<N>) + 1024;
    static bool attr = false;
    if (!attr) {
        EKG_CUDA(cudaFuncSetAttribute(k_contract_umma<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    dim3 grid((unsigned)A.nchunks, (unsigned)(A.n_sims * nlb));
    k_contract_umma<N><<<grid, UM_THREADS, smem, st>>>(A.steps, A.rows, A.apad, A.nl, A.t_hilo, A.at_hilo, A.chunk_a0,
                                                       A.chunk_a1, A.chunk_layer, A.Wp, A.layer_c, A.F, A.nchunks, nlb,
                                                       A.partial, A.err);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace

// N (padded rows) chosen from the row count: 16, 32, 64, 128 or 256 per block of rows.
void launch_contract_umma_args(cudaStream_t s, const ContractArgs &A) {
    if (A.rows <= 16) launch_n<16>(s, A);
    else if (A.rows <= 32) launch_n<32>(s, A);
    else if (A.rows <= 64) launch_n<64>(s, A);
    else if (A.rows <= 128) launch_n<128>(s, A);
    else launch_n<256>(s, A);
}

void launch_contract_umma(cudaStream_t s, const HeartDev &h, const float *d_Wp, const float *d_layer_c,
                          const double *d_F, int n_sims, double *d_partial, uint32_t *d_err) {
    ContractArgs A;
    A.steps = h.steps;
    A.rows = h.nleads;
    A.nl = h.nlayers;
    A.nchunks = h.nchunks;
    A.n_sims = n_sims;
    A.apad = h.apad;
    A.t_hilo = h.t_hilo.p;
    A.at_hilo = h.at_hilo.p;
    A.chunk_a0 = h.chunk_a0.p;
    A.chunk_a1 = h.chunk_a1.p;
    A.chunk_layer = h.chunk_layer.p;
    A.Wp = d_Wp;
    A.layer_c = d_layer_c;
    A.F = d_F;
    A.partial = d_partial;
    A.err = d_err;
    launch_contract_umma_args(s, A);
}

// ------------------------------------------------------------------ bounded-wait self-test
// One block does what a contraction CTA does around a wait that runs out: warp 0 takes tensor
// memory, thread 0 waits on an mbarrier that nothing arrives on (the kernels' bounded wait with a
// short poll limit), records KERR_MBAR_TIMEOUT in the error word, and warp 0 releases the tensor
// memory before the block returns.  Nothing else waits, so the kernel always ends.
__global__ void k_selftest_bounded_wait(uint32_t limit, uint32_t *err) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        ptx::mbar_init(&bar, 1);
        ptx::fence_barrier_init();
    }
    if (warp == 0) {
        ptx::tmem_alloc(&tmem_base, 32);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (threadIdx.x == 0 && !ptx::mbar_wait_n(&bar, 0, limit)) atomicOr(err, KERR_MBAR_TIMEOUT);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 0) ptx::tmem_dealloc(tmem_base, 32);
}

}  // namespace ekg

extern "C" int ekg_selftest_bounded_wait(int32_t device, uint32_t wait_limit) {
    using namespace ekg;
    return guard([&] {
        EKG_CHECK(wait_limit >= 1 && wait_limit <= ptx::WAIT_LIMIT, EKG_ERR_BAD_INPUT,
                  "wait limit must be in 1 .. the kernels' own limit");
        EKG_CUDA(cudaSetDevice(device));
        DBuf<uint32_t> err;
        err.alloc(1);
        EKG_CUDA(cudaMemset(err.p, 0, sizeof(uint32_t)));
        k_selftest_bounded_wait<<<1, 128>>>(wait_limit, err.p);
        EKG_CUDA(cudaGetLastError());
        EKG_CUDA(cudaDeviceSynchronize());
        uint32_t e = 0;
        EKG_CUDA(cudaMemcpy(&e, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (e & KERR_MBAR_TIMEOUT)
            throw Error{EKG_ERR_TIMEOUT, "a bounded device wait ran out (error word " + std::to_string(e) + ")"};
    });
}
