// ca.cu -- activation times of the excitation-sequence cellular automaton on the device.
//
// The reference runs a Dijkstra search over the 26-neighbour cube (simlib/simulator.cpp:212-286):
// start voxels get time 1.0; a popped voxel u offers time(u) + lag to each unexcited non-empty
// neighbour v, lag = T[L(u)][L(v)] * sqrt(|u - v|^2), each step rounded in FP64.  With positive
// lags that search returns the unique fixed point of
//     at(v) = min(init(v), min_u fl(at(u) + fl(T[L(u)][L(v)] * sqrt(k))))
// (every offered time is >= the offering voxel's own time), so a chaotic min-relaxation from
// +inf converges to the same doubles bit for bit, in any order.  Products and sums use
// __dmul_rn / __dadd_rn so the compiler cannot fuse them into an FMA.
//
// Layout: the grid is cut into 8x8x8 tiles.  A round processes the active tiles, one CTA each:
// the tile and a one-voxel halo are staged in shared memory (the FP64 times as their bit patterns,
// which order like the values for non-negative doubles, + uint8 layers).  The tile relaxes
// locally: a first sweep pulls every voxel's candidates from its 26 neighbours, later sweeps only
// push from the voxels that improved in the sweep before (64-bit atomicMin on the bit patterns),
// until a block-wide vote (__syncthreads_or) finds no change.  A candidate is skipped without the
// FP64 add when the offering voxel is not earlier than the receiving one (lags are positive).  The
// changed interior voxels are written back and the neighbour tiles that touch a changed face,
// edge or corner are flagged.  A compaction kernel turns the flags into the next round's tile list
// with warp ballots and one atomic per warp.  The host loops until no tile is active.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "ekg_internal.h"

namespace ekg {

namespace {

constexpr int TS = 8;            // tile edge
constexpr int HS = TS + 2;       // tile + halo
constexpr int CA_THREADS = 256;  // 2 voxels per thread
constexpr int MAX_LOCAL_ITERS = 64;

__device__ __forceinline__ uint8_t layer_id(uint8_t v) { return v; }
__device__ __forceinline__ uint8_t layer_id(int32_t v) { return (uint8_t)(v < 0 ? -v : v); }

// One tile of a round (all threads of the block): stage, relax, write back, flag neighbours.
template <typename LT>
__device__ __forceinline__ void ca_tile(const int tile, int nz, int ny, int nx, int ntz, int nty, int ntx,
                                        const LT *__restrict__ layers, const double *__restrict__ lag, int nl1,
                                        double *__restrict__ at, uint8_t *__restrict__ next_flag) {
    __shared__ unsigned long long s_b[HS][HS][HS];  // activation-time bits
    __shared__ uint8_t s_l[HS][HS][HS];
    __shared__ uint8_t s_ch[2][HS][HS][HS];         // improved in the last sweep (tile interior)
    __shared__ uint32_t s_mark;  // 27-bit mask of neighbour tiles to flag (bit = (dz+1)*9+(dy+1)*3+(dx+1))

    const int tx0 = (tile % ntx) * TS;
    const int ty0 = ((tile / ntx) % nty) * TS;
    const int tz0 = (tile / (ntx * nty)) * TS;
    const int tid = threadIdx.x;
    if (tid == 0) s_mark = 0;

    // stage tile + halo
    const unsigned long long INF_BITS = 0x7ff0000000000000ULL;
    for (int i = tid; i < HS * HS * HS; i += CA_THREADS) {
        int hx = i % HS, hy = (i / HS) % HS, hz = i / (HS * HS);
        int gx = tx0 + hx - 1, gy = ty0 + hy - 1, gz = tz0 + hz - 1;
        unsigned long long b = INF_BITS;
        uint8_t l = 0;
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz) {
            size_t g = ((size_t)gz * ny + gy) * nx + gx;
            l = layer_id(layers[g]);
            if (l) b = (unsigned long long)__double_as_longlong(at[g]);
        }
        s_b[hz][hy][hx] = b;
        s_l[hz][hy][hx] = l;
        s_ch[0][hz][hy][hx] = 0;
        s_ch[1][hz][hy][hx] = 0;
    }
    __syncthreads();

    const int lx = (tid & 7) + 1, ly = ((tid >> 3) & 7) + 1, lz0 = (tid >> 6) + 1;
    unsigned long long orig[2];
    uint8_t myl[2];
    bool inside[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        int lz = lz0 + 4 * r;
        orig[r] = s_b[lz][ly][lx];
        myl[r] = s_l[lz][ly][lx];
        inside[r] = (tx0 + lx - 1 < nx) && (ty0 + ly - 1 < ny) && (tz0 + lz - 1 < nz);
    }

    // sweep 0: pull from the 26 neighbours (the halo may carry new times from other tiles)
    bool changed = false;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (!inside[r] || myl[r] == 0) continue;
        const int lz = lz0 + 4 * r;
        unsigned long long best = s_b[lz][ly][lx];
        const double *lagd = lag + (size_t)myl[r] * 3;  // lag[src][dst=myl][k]
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    if (dz == 0 && dy == 0 && dx == 0) continue;
                    const uint8_t lu = s_l[lz + dz][ly + dy][lx + dx];
                    if (lu == 0) continue;
                    const unsigned long long bu = s_b[lz + dz][ly + dy][lx + dx];
                    if (bu >= best) continue;
                    const int k = (dz != 0) + (dy != 0) + (dx != 0);
                    const double c = __dadd_rn(__longlong_as_double((long long)bu),
                                               __ldg(lagd + (size_t)lu * nl1 * 3 + (k - 1)));
                    const unsigned long long cb = (unsigned long long)__double_as_longlong(c);
                    if (cb < best) best = cb;
                }
        if (best < s_b[lz][ly][lx]) {
            s_b[lz][ly][lx] = best;
            s_ch[0][lz][ly][lx] = 1;
            changed = true;
        }
    }
    int iters = 1, cur = 0;
    bool again = __syncthreads_or(changed);
    // later sweeps: the voxels that improved push to their interior neighbours
    while (again && iters < MAX_LOCAL_ITERS) {
        changed = false;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int lz = lz0 + 4 * r;
            if (!inside[r] || myl[r] == 0 || !s_ch[cur][lz][ly][lx]) continue;
            s_ch[cur][lz][ly][lx] = 0;
            const unsigned long long bu = s_b[lz][ly][lx];
            const double au = __longlong_as_double((long long)bu);
            const double *lags = lag + (size_t)myl[r] * nl1 * 3;  // lag[src=myl][dst][k]
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (dz == 0 && dy == 0 && dx == 0) continue;
                        const int wz = lz + dz, wy = ly + dy, wx = lx + dx;
                        if (wz < 1 || wz > TS || wy < 1 || wy > TS || wx < 1 || wx > TS) continue;
                        const uint8_t lw = s_l[wz][wy][wx];
                        if (lw == 0) continue;
                        const unsigned long long bw = s_b[wz][wy][wx];
                        if (bu >= bw) continue;
                        const int k = (dz != 0) + (dy != 0) + (dx != 0);
                        const unsigned long long cb = (unsigned long long)__double_as_longlong(
                            __dadd_rn(au, __ldg(lags + (size_t)lw * 3 + (k - 1))));
                        if (cb < bw && cb < atomicMin(&s_b[wz][wy][wx], cb)) {
                            s_ch[cur ^ 1][wz][wy][wx] = 1;
                            changed = true;
                        }
                    }
        }
        cur ^= 1;
        again = __syncthreads_or(changed);
        ++iters;
    }

    // write back and flag neighbour tiles touched by changed boundary voxels
    uint32_t mark = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int lz = lz0 + 4 * r;
        if (!inside[r] || myl[r] == 0) continue;
        const unsigned long long v = s_b[lz][ly][lx];
        if (v < orig[r]) {
            size_t g = ((size_t)(tz0 + lz - 1) * ny + (ty0 + ly - 1)) * nx + (tx0 + lx - 1);
            at[g] = __longlong_as_double((long long)v);
            const int fz = (lz == 1) ? -1 : (lz == TS ? 1 : 0);
            const int fy = (ly == 1) ? -1 : (ly == TS ? 1 : 0);
            const int fx = (lx == 1) ? -1 : (lx == TS ? 1 : 0);
            for (int a = 0; a <= (fz != 0); ++a)
                for (int b = 0; b <= (fy != 0); ++b)
                    for (int c = 0; c <= (fx != 0); ++c) {
                        int dz = a ? fz : 0, dy = b ? fy : 0, dx = c ? fx : 0;
                        if (dz || dy || dx) mark |= 1u << ((dz + 1) * 9 + (dy + 1) * 3 + (dx + 1));
                    }
        }
    }
    if (again) mark |= 1u << 13;  // local iteration cap hit: run this tile again
    // warp-level OR, then one shared atomic per warp
    for (int o = 16; o > 0; o >>= 1) mark |= __shfl_xor_sync(0xffffffffu, mark, o);
    if ((tid & 31) == 0 && mark) atomicOr(&s_mark, mark);
    __syncthreads();
    if (tid < 27) {
        const uint32_t m = s_mark;
        if (m & (1u << tid)) {
            int dz = tid / 9 - 1, dy = (tid / 3) % 3 - 1, dx = tid % 3 - 1;
            int tzz = tz0 / TS + dz, tyy = ty0 / TS + dy, txx = tx0 / TS + dx;
            if (tzz >= 0 && tzz < ntz && tyy >= 0 && tyy < nty && txx >= 0 && txx < ntx)
                next_flag[((size_t)tzz * nty + tyy) * ntx + txx] = 1;
        }
    }
}

// A round with one block per active tile (the tile list's length is the grid).
template <typename LT>
__global__ void k_ca_round(int nz, int ny, int nx, int ntz, int nty, int ntx, const LT *__restrict__ layers,
                           const double *__restrict__ lag, int nl1, double *__restrict__ at,
                           const int32_t *__restrict__ active, uint8_t *__restrict__ next_flag) {
    ca_tile<LT>(active[blockIdx.x], nz, ny, nx, ntz, nty, ntx, layers, lag, nl1, at, next_flag);
}

// A round over a device-resident tile list: a fixed grid walks the count_cur active tiles, so
// rounds can be queued back to back without the host reading the count.  Block 0 clears the next
// round's count, which only the compaction after this kernel adds to.
__global__ void __launch_bounds__(CA_THREADS) k_ca_round_list(int nz, int ny, int nx, int ntz, int nty, int ntx,
                                                              const uint8_t *__restrict__ layers,
                                                              const double *__restrict__ lag, int nl1,
                                                              double *__restrict__ at,
                                                              const int32_t *__restrict__ active,
                                                              const int32_t *__restrict__ count_cur,
                                                              int32_t *__restrict__ count_next,
                                                              uint8_t *__restrict__ next_flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *count_next = 0;
    const int n = *count_cur;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        ca_tile<uint8_t>(active[i], nz, ny, nx, ntz, nty, ntx, layers, lag, nl1, at, next_flag);
        __syncthreads();  // the next tile restages the shared arrays
    }
}

// next_flag -> compact list (order irrelevant); clears the flags.
__global__ void k_ca_compact(int ntiles, uint8_t *__restrict__ flag, int32_t *__restrict__ list,
                             int32_t *__restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool f = (i < ntiles) && flag[i];
    const unsigned b = __ballot_sync(0xffffffffu, f);
    int base = 0;
    if ((threadIdx.x & 31) == 0 && b) base = atomicAdd(count, __popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (f) {
        list[base + __popc(b & ((1u << (threadIdx.x & 31)) - 1))] = i;
        flag[i] = 0;
    }
}

__global__ void k_ca_init(size_t n, const uint8_t *__restrict__ layers, const uint8_t *__restrict__ start,
                          double *__restrict__ at) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        if (layers[i]) v = start[i] ? 1.0 : __longlong_as_double(0x7ff0000000000000LL);
        at[i] = v;
    }
}

__global__ void k_ca_finish(size_t n, double *__restrict__ at) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (isinf(at[i])) at[i] = 0.0;  // unreachable voxels keep excitationDelay 0
}

// ------------------------------------------------------------------ bucketed relaxation
// Dijkstra by time buckets (delta-stepping with a bucket width just below the smallest lag): the
// voxels whose time falls into bucket k = floor(t / delta) are final once every earlier bucket has
// been relaxed, because each of their predecessors on a shortest path is at least one lag, so more
// than delta, earlier.  Bucket k is one launch: a warp per queued entry (cell, layer, time), one
// lane per neighbour, offers fl(at(u) + lag) with a 64-bit atomicMin on the time bits; an improved
// neighbour is queued in the bucket of its new time with its new time (warp-aggregated appends per
// bucket).  A cell can be queued more than once: an entry whose cell has improved since offers a
// later time than the one already offered from the cell's better entry, which was relaxed in an
// earlier bucket or in this one, so it changes nothing.  Offers reach at most
// ceil(max lag / delta) + 1 buckets ahead, so the lists form a ring of that many slots; the slot
// of bucket k - 1 is emptied by bucket k's launch (nothing can still be queued there).
struct QEntry {
    int32_t cell, layer;
    unsigned long long bits;
};
struct BucketArgs {
    int nz, ny, nx;
    const uint8_t *layers;
    const double *lag;  // [nl1][nl1][3]
    int nl1;
    unsigned long long *at;  // time bits per cell (non-negative doubles order like their bits)
    QEntry *lists;           // [ring][cap]
    int32_t *counts;         // [ring]
    int32_t *overflow;
    int ring, cap;
    double inv_delta;
};

__device__ __forceinline__ int bucket_of(double t, double inv_delta) {
    return (int)floor(__dmul_rn(t, inv_delta));
}

__global__ void k_ca_bucket_init(size_t n, const uint8_t *__restrict__ layers, const uint8_t *__restrict__ start,
                                 BucketArgs A) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        if (layers[i]) v = start[i] ? 1.0 : __longlong_as_double(0x7ff0000000000000LL);
        const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        A.at[i] = bits;
        if (layers[i] && start[i]) {
            const int b = bucket_of(1.0, A.inv_delta);
            const int idx = atomicAdd(&A.counts[b % A.ring], 1);
            if (idx < A.cap) A.lists[(size_t)(b % A.ring) * A.cap + idx] = QEntry{(int32_t)i, (int32_t)layers[i], bits};
            else atomicOr(A.overflow, 1);
        }
    }
}

__global__ void __launch_bounds__(256) k_ca_bucket(int k, BucketArgs A) {
    const int slot = k % A.ring;
    if (blockIdx.x == 0 && threadIdx.x == 0) A.counts[(k + A.ring - 1) % A.ring] = 0;
    const int n = min(A.counts[slot], A.cap);
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    // lane -> neighbour offset (26 of the 32 lanes)
    int dz = 0, dy = 0, dx = 0, kind = 1;
    const bool nb = lane < 26;
    if (nb) {
        const int c = lane < 13 ? lane : lane + 1;  // skip the centre of the 3x3x3 cube
        dz = c / 9 - 1;
        dy = (c / 3) % 3 - 1;
        dx = c % 3 - 1;
        kind = (dz != 0) + (dy != 0) + (dx != 0);
    }
    // the loop bound is uniform over the warp, so every lane reaches the warp votes below
    for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += warps) {
        const QEntry q = A.lists[(size_t)slot * A.cap + e];
        const int u = q.cell;
        const int x = u % A.nx, y = (u / A.nx) % A.ny, z = u / (A.nx * A.ny);
        const int vz = z + dz, vy = y + dy, vx = x + dx;
        const bool inside = nb && vz >= 0 && vz < A.nz && vy >= 0 && vy < A.ny && vx >= 0 && vx < A.nx;
        const int v = inside ? (vz * A.ny + vy) * A.nx + vx : u;
        const uint8_t lv = inside ? A.layers[v] : 0;
        const unsigned long long bv = inside ? A.at[v] : 0ull;
        bool improved = false;
        double c = 0.0;
        if (lv != 0 && q.bits < bv) {
            c = __dadd_rn(__longlong_as_double((long long)q.bits),
                          __ldg(A.lag + ((size_t)q.layer * A.nl1 + lv) * 3 + (kind - 1)));
            const unsigned long long cb = (unsigned long long)__double_as_longlong(c);
            improved = cb < bv && cb < atomicMin(&A.at[v], cb);
        }
        // queue the improved neighbours: one atomic per bucket and warp
        const int b = improved ? bucket_of(c, A.inv_delta) : -1;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        if (improved) {
            const int leader = __ffs(same) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&A.counts[b % A.ring], __popc(same));
            base = __shfl_sync(same, base, leader);
            const int idx = base + __popc(same & ((1u << lane) - 1u));
            if (idx < A.cap)
                A.lists[(size_t)(b % A.ring) * A.cap + idx] =
                    QEntry{v, (int32_t)lv, (unsigned long long)__double_as_longlong(c)};
            else
                atomicOr(A.overflow, 1);
        }
    }
}

__global__ void k_ca_bucket_finish(size_t n, const unsigned long long *__restrict__ bits, double *__restrict__ at) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = __longlong_as_double((long long)bits[i]);
        at[i] = isinf(v) ? 0.0 : v;  // unreachable voxels keep excitationDelay 0
    }
}

}  // namespace

// Bucketed relaxation when the smallest lag allows it (returns false to fall back to the tile
// rounds: a zero lag, a time span of too many buckets, or a full bucket list).
bool ca_run_buckets(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_layers, const uint8_t *d_start,
                    const std::vector<double> &lag_h, int nl1, const double *d_lag, double *d_at, int64_t nvox,
                    int round_cap, int sm_count, CaResult &res) {
    double min_lag = INFINITY, max_lag = 0;
    for (int a = 1; a < nl1; ++a)
        for (int b = 1; b < nl1; ++b)
            for (int k = 0; k < 3; ++k) {
                const double l = lag_h[((size_t)a * nl1 + b) * 3 + k];
                min_lag = std::min(min_lag, l);
                max_lag = std::max(max_lag, l);
            }
    if (!(min_lag >= 0.05) || !std::isfinite(max_lag)) return false;
    // a bucket width just below the smallest lag keeps a margin far above FP64 rounding
    const double delta = min_lag * (1.0 - 1e-6);
    const int ring = (int)std::ceil(max_lag / delta) + 3;
    if (ring > 256) return false;
    const size_t n = (size_t)nz * ny * nx;
    // bucket indices stay far inside int: the latest time is below 1 + n * max_lag
    if ((1.0 + (double)n * max_lag) / delta > 1e9) return false;
    // per bucket slot; a cell can be queued more than once, a full slot falls back to the tile rounds
    const int cap = (int)std::min<int64_t>(std::max<int64_t>(65536, nvox / 2), INT32_MAX / 32);
    DBuf<unsigned long long> bits;
    DBuf<QEntry> lists;
    DBuf<int32_t> counts;
    bits.alloc(n);
    lists.alloc((size_t)ring * cap);
    counts.alloc(ring + 1);  // + the overflow flag
    BucketArgs A;
    A.nz = nz;
    A.ny = ny;
    A.nx = nx;
    A.layers = d_layers;
    A.lag = d_lag;
    A.nl1 = nl1;
    A.at = bits.p;
    A.lists = lists.p;
    A.counts = counts.p;
    A.overflow = counts.p + ring;
    A.ring = ring;
    A.cap = cap;
    A.inv_delta = 1.0 / delta;
    EKG_CUDA(cudaMemsetAsync(counts.p, 0, (ring + 1) * sizeof(int32_t), s));
    cudaEvent_t e0, e1;
    EKG_CUDA(cudaEventCreate(&e0));
    EKG_CUDA(cudaEventCreate(&e1));
    struct Events {
        cudaEvent_t a, b;
        ~Events() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ev{e0, e1};
    EKG_CUDA(cudaEventRecord(e0, s));
    k_ca_bucket_init<<<1024, 256, 0, s>>>(n, d_layers, d_start, A);
    EKG_CUDA(cudaGetLastError());
    // buckets before the first start time are empty
    int k = (int)std::floor(1.0 * A.inv_delta);
    const int grid = std::max(1, sm_count) * 8;
    std::vector<int32_t> h(ring + 1);
    int32_t *hc = nullptr;
    EKG_CUDA(cudaMallocHost(&hc, (ring + 1) * sizeof(int32_t)));
    struct Pinned {
        int32_t *p;
        ~Pinned() { cudaFreeHost(p); }
    } pin{hc};
    // every cell settles at most once per bucket it is queued in; more buckets than cells plus the
    // ring means the queues never drain
    const int64_t kmax = round_cap > 0 ? (int64_t)round_cap : (int64_t)n + 4LL * ring + 1024;
    constexpr int CHUNK = 16;
    int steps = 0;
    for (;;) {
        for (int i = 0; i < CHUNK; ++i, ++k, ++steps) {
            if (steps >= kmax) throw Error{EKG_ERR_CA_NOT_CONVERGED, "activation-time relaxation did not converge"};
            k_ca_bucket<<<grid, 256, 0, s>>>(k, A);
            EKG_CUDA(cudaGetLastError());
        }
        EKG_CUDA(cudaMemcpyAsync(hc, counts.p, (ring + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        EKG_CUDA(cudaStreamSynchronize(s));
        if (hc[ring]) return false;  // a bucket list overflowed: the tile rounds redo it
        // the slot of the last bucket launched holds processed entries; any other non-empty slot
        // is a bucket still to come
        bool pending = false;
        for (int r = 0; r < ring; ++r)
            if (r != (k - 1) % ring && hc[r] > 0) pending = true;
        if (!pending) break;
    }
    k_ca_bucket_finish<<<1024, 256, 0, s>>>(n, bits.p, d_at);
    EKG_CUDA(cudaGetLastError());
    EKG_CUDA(cudaEventRecord(e1, s));
    EKG_CUDA(cudaEventSynchronize(e1));
    EKG_CUDA(cudaEventElapsedTime(&res.ms, e0, e1));
    res.rounds = steps;
    res.buckets = true;
    return true;
}

CaResult ca_run(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_layers, const uint8_t *d_start,
                const std::vector<int32_t> &start_tiles, int nl1, const double *d_lag, double *d_at, int round_cap,
                int sm_count) {
    CaResult res;
    const int ntz = (nz + TS - 1) / TS, nty = (ny + TS - 1) / TS, ntx = (nx + TS - 1) / TS;
    const int ntiles = ntz * nty * ntx;
    const size_t n = (size_t)nz * ny * nx;
    DBuf<int32_t> lists, count;
    DBuf<uint8_t> flag;
    lists.alloc(2 * (size_t)ntiles);
    count.alloc(2);
    flag.alloc(ntiles);
    int32_t *list[2] = {lists.p, lists.p + ntiles};
    const int32_t n_start = (int32_t)start_tiles.size();
    EKG_CUDA(cudaMemsetAsync(flag.p, 0, ntiles, s));
    EKG_CUDA(cudaMemcpyAsync(list[0], start_tiles.data(), start_tiles.size() * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(count.p, &n_start, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    cudaEvent_t e0, e1;
    EKG_CUDA(cudaEventCreate(&e0));
    EKG_CUDA(cudaEventCreate(&e1));
    EKG_CUDA(cudaEventRecord(e0, s));
    k_ca_init<<<1024, 256, 0, s>>>(n, d_layers, d_start, d_at);
    EKG_CUDA(cudaGetLastError());
    // Every round finalises at least the next tile along each shortest path; a path can
    // cross a tile boundary at most once per hop, so this cap is far above any real heart.
    const int cap = round_cap > 0 ? round_cap : 16 * (ntz + nty + ntx) + 4 * ntiles + 64;
    // Rounds are queued in chunks (round over the device-resident list, then its compaction); the
    // host reads the active count once per chunk.  Rounds after convergence find an empty list.
    constexpr int CHUNK = 8;
    int blocks_per_sm = 0;
    EKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_ca_round_list, CA_THREADS, 0));
    const int grid = std::max(1, std::min(ntiles, std::max(1, blocks_per_sm) * std::max(1, sm_count)));
    int32_t *h_count = nullptr;
    EKG_CUDA(cudaMallocHost(&h_count, sizeof(int32_t)));
    int n_active = n_start, r = 0;
    while (n_active > 0) {
        if (r >= cap) {
            cudaFreeHost(h_count);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw Error{EKG_ERR_CA_NOT_CONVERGED, "activation-time relaxation did not converge"};
        }
        const int chunk = std::min(CHUNK, cap - r);
        for (int k = 0; k < chunk; ++k, ++r) {
            const int c = r & 1;
            k_ca_round_list<<<grid, CA_THREADS, 0, s>>>(nz, ny, nx, ntz, nty, ntx, d_layers, d_lag, nl1, d_at,
                                                       list[c], count.p + c, count.p + (c ^ 1), flag.p);
            EKG_CUDA(cudaGetLastError());
            k_ca_compact<<<(ntiles + 255) / 256, 256, 0, s>>>(ntiles, flag.p, list[c ^ 1], count.p + (c ^ 1));
            EKG_CUDA(cudaGetLastError());
        }
        EKG_CUDA(cudaMemcpyAsync(h_count, count.p + (r & 1), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        EKG_CUDA(cudaStreamSynchronize(s));
        n_active = *h_count;
    }
    cudaFreeHost(h_count);
    res.rounds = r;
    k_ca_finish<<<1024, 256, 0, s>>>(n, d_at);
    EKG_CUDA(cudaGetLastError());
    EKG_CUDA(cudaEventRecord(e1, s));
    EKG_CUDA(cudaEventSynchronize(e1));
    EKG_CUDA(cudaEventElapsedTime(&res.ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return res;
}



// ------------------------------------------------------------------ no-allocation entry point
// ekg_activation_noalloc: the same relaxation for callers that cannot allocate device memory
// (for example code running under a memory pool or allocator that forbids new cudaMalloc calls
// after start-up, or inside a host loop that must not touch the allocator).  All scratch lives in
// one file-scope device array, g_noalloc, of fixed size; the caller supplies the layer grid and
// the output as device buffers it already owns.  Every call shares g_noalloc and leaves its last
// contents behind, so the counters and flags are cleared at the start of each call; a host mutex
// serialises callers in this process, and calls whose device work overlaps (for example from
// another thread that bypasses this entry point's lock) would race on the array.
namespace {
constexpr int NOALLOC_MAX_TILES = 65536;  // 8x8x8 tiles, e.g. a 320^3 grid
constexpr int NOALLOC_MAX_LAYER = 31;     // highest layer id (lag table 32 x 32 x 3)
struct NoAllocScratch {
    int32_t list[2][NOALLOC_MAX_TILES];
    uint8_t flag[NOALLOC_MAX_TILES];
    int32_t count;
    int32_t nstart;
    uint32_t layer_mask;
    int32_t bad;
    double lag[(NOALLOC_MAX_LAYER + 1) * (NOALLOC_MAX_LAYER + 1) * 3];
};
static __device__ __align__(256) NoAllocScratch g_noalloc;

// per-device address of g_noalloc (host code may not use the symbol itself as an address)
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_ptr[64] = {nullptr};

__global__ void k_na_validate(size_t n, const int32_t *__restrict__ layers, NoAllocScratch *sc) {
    uint32_t mask = 0;
    int32_t starts = 0, bad = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int32_t v = layers[i];
        // widened before the negation: INT32_MIN is out of range, not a negative shift
        const int64_t a = v < 0 ? -(int64_t)v : (int64_t)v;
        if (a > NOALLOC_MAX_LAYER) bad = 1;
        else mask |= 1u << (uint32_t)a;
        starts += v < 0;
    }
    mask = __reduce_or_sync(0xffffffffu, mask);
    starts = __reduce_add_sync(0xffffffffu, starts);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (mask) atomicOr(&sc->layer_mask, mask);
        if (starts) atomicAdd(&sc->nstart, starts);
        if (bad) atomicOr(&sc->bad, 1);
    }
}

__global__ void k_na_init(int nz, int ny, int nx, int nty, int ntx, const int32_t *__restrict__ layers,
                          double *__restrict__ at, uint8_t *__restrict__ flag) {
    const size_t n = (size_t)nz * ny * nx;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int32_t v = layers[i];
        double a = 0.0;
        if (v < 0) {
            a = 1.0;
            const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((size_t)nx * ny));
            flag[((size_t)(z / TS) * nty + (y / TS)) * ntx + (x / TS)] = 1;
        } else if (v > 0) {
            a = __longlong_as_double(0x7ff0000000000000LL);
        }
        at[i] = a;
    }
}

NoAllocScratch *noalloc_scratch() {
    int dev = 0;
    EKG_CUDA(cudaGetDevice(&dev));
    EKG_CHECK(dev >= 0 && dev < 64, EKG_ERR_DEVICE, "device index out of range");
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        EKG_CUDA(cudaGetSymbolAddress(&p, g_noalloc));
        g_noalloc_ptr[dev] = reinterpret_cast<NoAllocScratch *>(p);
    }
    return g_noalloc_ptr[dev];
}
}  // namespace

}  // namespace ekg

extern "C" int ekg_activation_noalloc(int32_t nz, int32_t ny, int32_t nx, const int32_t *d_layers, int32_t n_transfer,
                                      const double *transfer, double *d_at, int32_t *rounds_out) {
    using namespace ekg;
    return guard([&] {
        EKG_CHECK(d_layers && transfer && d_at && n_transfer >= 1, EKG_ERR_BAD_INPUT, "null argument");
        EKG_CHECK(nz >= 1 && ny >= 1 && nx >= 1, EKG_ERR_BAD_INPUT, "grid extents must be positive");
        const int ntz = (nz + TS - 1) / TS, nty = (ny + TS - 1) / TS, ntx = (nx + TS - 1) / TS;
        const int64_t ntiles = (int64_t)ntz * nty * ntx;
        EKG_CHECK(ntiles <= NOALLOC_MAX_TILES, EKG_ERR_BAD_INPUT,
                  "grid too large for ekg_activation_noalloc: at most 65536 tiles of 8x8x8 cells");
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        NoAllocScratch *sc = noalloc_scratch();
        const size_t n = (size_t)nz * ny * nx;
        cudaStream_t s = 0;
        // clear what must start at zero: flags, counters, layer mask
        EKG_CUDA(cudaMemsetAsync(sc->flag, 0, sizeof(sc->flag), s));
        EKG_CUDA(cudaMemsetAsync(&sc->count, 0, 4 * sizeof(int32_t), s));
        k_na_validate<<<1024, 256, 0, s>>>(n, d_layers, sc);
        EKG_CUDA(cudaGetLastError());
        struct {
            int32_t count, nstart;
            uint32_t mask;
            int32_t bad;
        } hdr;
        EKG_CUDA(cudaMemcpy(&hdr, &sc->count, sizeof(hdr), cudaMemcpyDeviceToHost));
        EKG_CHECK(!hdr.bad, EKG_ERR_BAD_INPUT, "layer ids must be at most 31 for ekg_activation_noalloc");
        EKG_CHECK(hdr.nstart > 0, EKG_ERR_NO_START, "Could not find starting point for excitation sequence");
        int nl = 0;
        for (int a = 1; a <= NOALLOC_MAX_LAYER; ++a)
            if (hdr.mask & (1u << a)) {
                nl = a;
                if (a >= n_transfer)
                    throw Error{EKG_ERR_TRANSFER, "transfer (conduction) matrix does not define layer " + std::to_string(a)};
            }
        const int nl1 = nl + 1;
        double lag[(NOALLOC_MAX_LAYER + 1) * (NOALLOC_MAX_LAYER + 1) * 3];
        for (int i = 0; i < nl1 * nl1 * 3; ++i) lag[i] = 0.0;
        for (int a = 1; a <= nl; ++a)
            for (int b = 1; b <= nl; ++b) {
                if (!((hdr.mask >> a) & 1u) || !((hdr.mask >> b) & 1u)) continue;
                const double t = transfer[(size_t)a * n_transfer + b];
                EKG_CHECK(t >= 0 && std::isfinite(t), EKG_ERR_BAD_INPUT,
                          "conduction delays between present layers must be finite and non-negative");
                for (int k = 1; k <= 3; ++k) {
                    double l = t;
                    l *= std::sqrt((double)k);
                    lag[((size_t)a * nl1 + b) * 3 + (k - 1)] = l;
                }
            }
        EKG_CUDA(cudaMemcpy(sc->lag, lag, (size_t)nl1 * nl1 * 3 * sizeof(double), cudaMemcpyHostToDevice));
        k_na_init<<<1024, 256, 0, s>>>(nz, ny, nx, nty, ntx, d_layers, d_at, sc->flag);
        EKG_CUDA(cudaGetLastError());
        int32_t *cur = sc->list[0], *nxt = sc->list[1];
        k_ca_compact<<<(unsigned)((ntiles + 255) / 256), 256, 0, s>>>((int)ntiles, sc->flag, cur, &sc->count);
        EKG_CUDA(cudaGetLastError());
        int32_t n_active = 0;
        EKG_CUDA(cudaMemcpy(&n_active, &sc->count, sizeof(int32_t), cudaMemcpyDeviceToHost));
        const int cap = 16 * (ntz + nty + ntx) + 4 * (int)ntiles + 64;
        int rounds = 0;
        while (n_active > 0) {
            EKG_CHECK(rounds < cap, EKG_ERR_CA_NOT_CONVERGED, "activation-time relaxation did not converge");
            k_ca_round<int32_t><<<n_active, CA_THREADS, 0, s>>>(nz, ny, nx, ntz, nty, ntx, d_layers, sc->lag, nl1,
                                                               d_at, cur, sc->flag);
            EKG_CUDA(cudaGetLastError());
            EKG_CUDA(cudaMemsetAsync(&sc->count, 0, sizeof(int32_t), s));
            k_ca_compact<<<(unsigned)((ntiles + 255) / 256), 256, 0, s>>>((int)ntiles, sc->flag, nxt, &sc->count);
            EKG_CUDA(cudaGetLastError());
            EKG_CUDA(cudaMemcpy(&n_active, &sc->count, sizeof(int32_t), cudaMemcpyDeviceToHost));
            std::swap(cur, nxt);
            ++rounds;
        }
        k_ca_finish<<<1024, 256, 0, s>>>(n, d_at);
        EKG_CUDA(cudaGetLastError());
        EKG_CUDA(cudaStreamSynchronize(s));
        if (rounds_out) *rounds_out = rounds;
    });
}
