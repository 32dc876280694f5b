// setup.cu -- the de-duplication part of a heart's set-up on the device.
//
// Simulation::setApIndices (simlib/simulator.cpp:561-621) gives every distinct (layer, activation
// time) pair of the non-empty voxels an AP.  Here the voxels are listed in raster order
// (compaction by a two-level scan), sorted by (layer, activation time) with a stable LSD radix
// sort on 8-bit digits of the time's bit pattern (non-negative doubles order like their bit
// patterns) and then of the layer -- stability keeps raster (cell) order inside an AP -- and the
// runs of equal keys are the APs.  Then the per-AP arrays in the padded per-layer K layout and the
// per-voxel records of the dipole kernels are written by one thread per AP slot / voxel.  The
// results are the arrays a host sort by (layer, time bits, cell) gives, element for element.
#include <cstdint>
#include <vector>

#include "ekg_internal.h"

namespace ekg {

namespace {

constexpr int ST = 256;             // threads per block
constexpr int SITEMS = 8;           // items per thread in the scans
constexpr int STILE = ST * SITEMS;  // scan tile
constexpr unsigned FULL = 0xffffffffu;

// Exclusive scan of one value per thread across the block (fixed order); *total gets the sum.
__device__ __forceinline__ int block_exscan(int v, int *total, int *s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < ST / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, t, o);
            if (lane >= o) t += y;
        }
        if (lane < ST / 32) s_warp[lane] = t;
    }
    __syncthreads();
    const int r = (w > 0 ? s_warp[w - 1] : 0) + x - v;
    *total = s_warp[ST / 32 - 1];
    __syncthreads();
    return r;
}

// Flag functions: cell c is a voxel; sorted voxel i starts a new (layer, time) run.
struct IsVoxel {
    const uint8_t *lay;
    __device__ int operator()(int64_t c) const { return lay[c] != 0; }
};
struct StartsRun {
    const uint8_t *lay;
    const uint64_t *key;
    __device__ int operator()(int64_t i) const {
        return i == 0 || lay[i] != lay[i - 1] || key[i] != key[i - 1];
    }
};

// Flags per STILE tile: tile sums, then (one block) their exclusive scan, then each tile writes the
// indices of its flagged items to out[] at their ranks.
template <class F>
__global__ void __launch_bounds__(ST) k_tile_counts(F f, int64_t n, int *__restrict__ tsum) {
    __shared__ int s_warp[ST / 32];
    const int64_t base = (int64_t)blockIdx.x * STILE + (int64_t)threadIdx.x * SITEMS;
    int c = 0;
#pragma unroll
    for (int k = 0; k < SITEMS; ++k)
        if (base + k < n) c += f(base + k);
    int total;
    block_exscan(c, &total, s_warp);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

// exclusive scan of tsum[0..nt) in place by one block; tsum[nt] = total
__global__ void __launch_bounds__(ST) k_scan_counts(int *__restrict__ tsum, int nt) {
    __shared__ int s_warp[ST / 32];
    int carry = 0;
    for (int b = 0; b < nt; b += ST) {
        const int i = b + (int)threadIdx.x;
        const int v = i < nt ? tsum[i] : 0;
        int total;
        const int ex = block_exscan(v, &total, s_warp);
        if (i < nt) tsum[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) tsum[nt] = carry;
}

template <class F>
__global__ void __launch_bounds__(ST) k_compact(F f, int64_t n, const int *__restrict__ tsum, int *__restrict__ out) {
    __shared__ int s_warp[ST / 32];
    const int64_t base = (int64_t)blockIdx.x * STILE + (int64_t)threadIdx.x * SITEMS;
    int flags = 0, c = 0;
#pragma unroll
    for (int k = 0; k < SITEMS; ++k)
        if (base + k < n && f(base + k)) {
            flags |= 1 << k;
            ++c;
        }
    int total;
    int pos = tsum[blockIdx.x] + block_exscan(c, &total, s_warp);
#pragma unroll
    for (int k = 0; k < SITEMS; ++k)
        if (flags & (1 << k)) out[pos++] = (int)(base + k);
}

template <class F>
int compact(cudaStream_t s, F f, int64_t n, DBuf<int> &tsum, int *out, int *host_total) {
    const int nt = (int)((n + STILE - 1) / STILE);
    if (tsum.n < (size_t)nt + 1) tsum.alloc((size_t)nt + 1);
    k_tile_counts<<<nt, ST, 0, s>>>(f, n, tsum.p);
    k_scan_counts<<<1, ST, 0, s>>>(tsum.p, nt);
    k_compact<<<nt, ST, 0, s>>>(f, n, tsum.p, out);
    EKG_CUDA(cudaGetLastError());
    EKG_CUDA(cudaMemcpyAsync(host_total, tsum.p + nt, sizeof(int), cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaStreamSynchronize(s));
    return *host_total;
}

// ---- stable LSD radix sort of (layer, time bits) with the cell as payload, 8-bit digits
// pass p < 8: byte p of the time bits; pass 8: the layer.  One element per thread, tiles of ST.
__device__ __forceinline__ int digit(int pass, uint64_t key, uint8_t lay) {
    return pass < 8 ? (int)((key >> (8 * pass)) & 0xffu) : (int)lay;
}

__global__ void __launch_bounds__(ST) k_digit_hist(int pass, int n, const uint64_t *__restrict__ key,
                                                   const uint8_t *__restrict__ lay, int nblk, int *__restrict__ hist) {
    __shared__ int s_h[256];
    s_h[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * ST + threadIdx.x;
    if (i < n) atomicAdd(&s_h[digit(pass, key[i], lay[i])], 1);
    __syncthreads();
    hist[(size_t)threadIdx.x * nblk + blockIdx.x] = s_h[threadIdx.x];
}

// per digit (block): exclusive scan of its counts over the tiles; totals[d] = the digit's count
__global__ void __launch_bounds__(ST) k_digit_scan(int *__restrict__ hist, int nblk, int *__restrict__ totals) {
    __shared__ int s_warp[ST / 32];
    int *h = hist + (size_t)blockIdx.x * nblk;
    int carry = 0;
    for (int b = 0; b < nblk; b += ST) {
        const int i = b + (int)threadIdx.x;
        const int v = i < nblk ? h[i] : 0;
        int total;
        const int ex = block_exscan(v, &total, s_warp);
        if (i < nblk) h[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(ST) k_digit_base(const int *__restrict__ totals, int *__restrict__ base) {
    __shared__ int s_warp[ST / 32];
    int total;
    base[threadIdx.x] = block_exscan(totals[threadIdx.x], &total, s_warp);
}

// rank = digit base + the tile's offset for the digit + equal digits before it in the tile (earlier
// warps' counts from shared memory, earlier lanes of the warp from a match mask): stable
__global__ void __launch_bounds__(ST) k_digit_scatter(int pass, int n, const uint64_t *__restrict__ key_in,
                                                      const uint8_t *__restrict__ lay_in, const int *__restrict__ val_in,
                                                      int nblk, const int *__restrict__ hist,
                                                      const int *__restrict__ base, uint64_t *__restrict__ key_out,
                                                      uint8_t *__restrict__ lay_out, int *__restrict__ val_out) {
    __shared__ int s_cnt[ST / 32][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < (ST / 32) * 256; k += ST) (&s_cnt[0][0])[k] = 0;
    __syncthreads();
    const int i = blockIdx.x * ST + threadIdx.x;
    const bool valid = i < n;
    uint64_t kv = 0;
    uint8_t lv = 0;
    int vv = 0;
    if (valid) {
        kv = key_in[i];
        lv = lay_in[i];
        vv = val_in[i];
    }
    const int d = valid ? digit(pass, kv, lv) : 256 + lane;  // invalid lanes match nothing
    const unsigned m = __match_any_sync(FULL, d);
    const int rank_w = __popc(m & ((1u << lane) - 1u));
    if (valid && rank_w == 0) s_cnt[w][d] = __popc(m);
    __syncthreads();
    if (valid) {
        int off = 0;
        for (int k = 0; k < w; ++k) off += s_cnt[k][d];
        const int pos = base[d] + hist[(size_t)d * nblk + blockIdx.x] + off + rank_w;
        key_out[pos] = kv;
        lay_out[pos] = lv;
        val_out[pos] = vv;
    }
}

__global__ void k_gather_keys(int nv, const int *__restrict__ cell, const double *__restrict__ at,
                              const uint8_t *__restrict__ lay, uint64_t *__restrict__ key, uint8_t *__restrict__ vl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int64_t c = cell[i];
    key[i] = (uint64_t)__double_as_longlong(at[c]);
    vl[i] = lay[c];
}

// first AP of each layer (APs are ordered by layer): lfirst[L] (-1 when the layer has none)
__global__ void k_layer_first(int na, const int *__restrict__ gstart, const uint8_t *__restrict__ vl,
                              int *__restrict__ lfirst) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na) return;
    const uint8_t L = vl[gstart[a]];
    if (a == 0 || vl[gstart[a - 1]] != L) lfirst[L] = a;
}

// per padded AP slot p: its layer (present layer k with pbase[k] <= p < pbase[k + 1]), the AP's
// time (FP64 and FP32 hi/lo), layer index and first voxel; padding slots get +inf and the first
// voxel of the layer's next AP
__global__ void k_ap_arrays(int64_t apad, int npl, const int *__restrict__ pl_layer, const int64_t *__restrict__ pbase,
                            const int *__restrict__ pfirst, const int *__restrict__ pcount, int na, int nv,
                            const int *__restrict__ gstart, const int *__restrict__ cell, const double *__restrict__ at_cells,
                            double *__restrict__ at, float2 *__restrict__ at_hilo, int32_t *__restrict__ a_layer,
                            int64_t *__restrict__ a_vb) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p == apad) a_vb[apad] = nv;
    if (p >= apad) return;
    int lo = 0, hi = npl - 1;  // last k with pbase[k] <= p
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (pbase[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    const int64_t j = p - pbase[lo];
    a_layer[p] = pl_layer[lo] - 1;
    if (j < pcount[lo]) {
        const int ap = pfirst[lo] + (int)j;
        const double t = at_cells[cell[gstart[ap]]];
        at[p] = t;
        const float h = __double2float_rn(t);
        at_hilo[p] = make_float2(h, __double2float_rn(t - (double)h));
        a_vb[p] = gstart[ap];
    } else {
        const int next = pfirst[lo] + pcount[lo];
        at[p] = __longlong_as_double(0x7ff0000000000000ll);
        at_hilo[p] = make_float2(__int_as_float(0x7f800000), 0.f);
        a_vb[p] = next < na ? gstart[next] : nv;
    }
}

// per voxel (sorted order): packed position, neighbour masks, bordered position relative to the
// centre with the mask and flags (interior, few absent neighbours, last voxel of its AP), out-offset sum
struct VoxelGeom {
    int nz, ny, nx, nnb;
    int8_t dif[26 * 3];
    uint32_t interior_mask;
    int few_max;
    double cz, cy, cx;  // heart centre; bordered coordinates relative to it, (float)((z + 1) - cz)
};
__global__ void k_voxel_records(int nv, VoxelGeom g, const int *__restrict__ cell, const uint8_t *__restrict__ lay,
                                const uint8_t *__restrict__ vl, const uint64_t *__restrict__ key,
                                int32_t *__restrict__ vzyx, uint32_t *__restrict__ vin, uint32_t *__restrict__ vout,
                                float4 *__restrict__ vpos, float4 *__restrict__ vosum,
                                unsigned long long *__restrict__ n_interior) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool interior = false;
    if (i < nv) {
        const int64_t c = cell[i];
        const int z = (int)(c / ((int64_t)g.ny * g.nx)), y = (int)((c / g.nx) % g.ny), x = (int)(c % g.nx);
        vzyx[i] = (z << 20) | (y << 10) | x;
        uint32_t mi = 0, mo = 0;
        int oz = 0, oy = 0, ox = 0;
        for (int q = 0; q < g.nnb; ++q) {
            const int dz = g.dif[3 * q], dy = g.dif[3 * q + 1], dx = g.dif[3 * q + 2];
            int z2 = z + dz, y2 = y + dy, x2 = x + dx;
            if (z2 >= 0 && z2 < g.nz && y2 >= 0 && y2 < g.ny && x2 >= 0 && x2 < g.nx &&
                lay[((int64_t)z2 * g.ny + y2) * g.nx + x2])
                mi |= 1u << q;
            z2 = z - dz;
            y2 = y - dy;
            x2 = x - dx;
            if (z2 >= 0 && z2 < g.nz && y2 >= 0 && y2 < g.ny && x2 >= 0 && x2 < g.nx &&
                lay[((int64_t)z2 * g.ny + y2) * g.nx + x2]) {
                mo |= 1u << q;
                oz += dz;
                oy += dy;
                ox += dx;
            }
        }
        vin[i] = mi;
        vout[i] = mo;
        uint32_t mbits = mi;
        if (g.interior_mask && mi == g.interior_mask && oz == 0 && oy == 0 && ox == 0) {
            mbits |= 1u << 31;
            interior = true;
        } else if (g.interior_mask && __popc(g.interior_mask & ~mi) <= g.few_max) {
            mbits |= 1u << 29;
        }
        const bool ends = i == nv - 1 || vl[i + 1] != vl[i] || key[i + 1] != key[i];
        if (ends) mbits |= 1u << 30;
        vpos[i] = make_float4((float)((double)(z + 1) - g.cz), (float)((double)(y + 1) - g.cy),
                              (float)((double)(x + 1) - g.cx), __uint_as_float(mbits));
        vosum[i] = make_float4((float)oz, (float)oy, (float)ox, mo ? 1.f : 0.f);
    }
    const unsigned b = __ballot_sync(FULL, interior);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(n_interior, (unsigned long long)__popc(b));
}

}  // namespace

void setup_voxels_device(cudaStream_t s, int nz, int ny, int nx, const uint8_t *d_lay, const double *d_at_cells,
                         int nl, DedupResult &r) {
    const int64_t n = (int64_t)nz * ny * nx;
    int *pinned = nullptr;
    EKG_CUDA(cudaMallocHost(&pinned, 8 * sizeof(int)));
    struct Free {
        int *p;
        ~Free() { cudaFreeHost(p); }
    } free_pinned{pinned};
    DBuf<int> tsum;
    // 1. voxels in raster order
    DBuf<int> cellA, cellB;
    const int nv = [&] {
        // an upper bound for the list: count first
        const int nt = (int)((n + STILE - 1) / STILE);
        tsum.alloc((size_t)nt + 1);
        k_tile_counts<<<nt, ST, 0, s>>>(IsVoxel{d_lay}, n, tsum.p);
        k_scan_counts<<<1, ST, 0, s>>>(tsum.p, nt);
        EKG_CUDA(cudaGetLastError());
        EKG_CUDA(cudaMemcpyAsync(pinned, tsum.p + nt, sizeof(int), cudaMemcpyDeviceToHost, s));
        EKG_CUDA(cudaStreamSynchronize(s));
        const int c = pinned[0];
        cellA.alloc((size_t)std::max(c, 1));
        k_compact<<<nt, ST, 0, s>>>(IsVoxel{d_lay}, n, tsum.p, cellA.p);
        EKG_CUDA(cudaGetLastError());
        return c;
    }();
    r.nvox = nv;
    if (nv == 0) return;
    // 2. stable radix sort by (layer, time bits); payload = cell
    DBuf<uint64_t> keyA, keyB;
    DBuf<uint8_t> layA, layB;
    keyA.alloc(nv);
    keyB.alloc(nv);
    layA.alloc(nv);
    layB.alloc(nv);
    cellB.alloc(nv);
    {
        const int g = (nv + 255) / 256;
        k_gather_keys<<<g, 256, 0, s>>>(nv, cellA.p, d_at_cells, d_lay, keyA.p, layA.p);
        EKG_CUDA(cudaGetLastError());
    }
    const int nblk = (nv + ST - 1) / ST;
    DBuf<int> hist, totals, base;
    hist.alloc((size_t)256 * nblk);
    totals.alloc(256);
    base.alloc(256);
    uint64_t *ki = keyA.p, *ko = keyB.p;
    uint8_t *li = layA.p, *lo = layB.p;
    int *vi = cellA.p, *vo = cellB.p;
    for (int pass = 0; pass < 9; ++pass) {
        k_digit_hist<<<nblk, ST, 0, s>>>(pass, nv, ki, li, nblk, hist.p);
        k_digit_scan<<<256, ST, 0, s>>>(hist.p, nblk, totals.p);
        k_digit_base<<<1, ST, 0, s>>>(totals.p, base.p);
        k_digit_scatter<<<nblk, ST, 0, s>>>(pass, nv, ki, li, vi, nblk, hist.p, base.p, ko, lo, vo);
        EKG_CUDA(cudaGetLastError());
        std::swap(ki, ko);
        std::swap(li, lo);
        std::swap(vi, vo);
    }
    // after an odd number of passes the sorted arrays are the B buffers
    DBuf<uint64_t> &key = ki == keyA.p ? keyA : keyB;
    DBuf<uint8_t> &vl = li == layA.p ? layA : layB;
    DBuf<int> &cell = vi == cellA.p ? cellA : cellB;
    // 3. runs of equal (layer, time): the APs
    DBuf<int> gstart;
    gstart.alloc((size_t)nv + 1);
    const int na = compact(s, StartsRun{vl.p, key.p}, nv, tsum, gstart.p, pinned);
    r.naps = na;
    // 4. first AP of each layer
    DBuf<int> lfirst;
    lfirst.alloc(256);
    EKG_CUDA(cudaMemsetAsync(lfirst.p, 0xff, 256 * sizeof(int), s));
    k_layer_first<<<(na + 255) / 256, 256, 0, s>>>(na, gstart.p, vl.p, lfirst.p);
    EKG_CUDA(cudaGetLastError());
    std::vector<int> lf(256);
    EKG_CUDA(cudaMemcpyAsync(lf.data(), lfirst.p, 256 * sizeof(int), cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaStreamSynchronize(s));
    // present layers in order with their AP ranges and padded (multiple of 64) bases
    r.pl_layer.clear();
    r.pfirst.clear();
    r.pcount.clear();
    r.pbase.clear();
    int64_t pad = 0;
    for (int L = 1; L <= nl; ++L)
        if (lf[L] >= 0) {
            int next = na;
            for (int L2 = L + 1; L2 <= nl; ++L2)
                if (lf[L2] >= 0) {
                    next = lf[L2];
                    break;
                }
            r.pl_layer.push_back(L);
            r.pfirst.push_back(lf[L]);
            r.pcount.push_back(next - lf[L]);
            r.pbase.push_back(pad);
            pad += (int64_t)(next - lf[L] + 63) / 64 * 64;
        }
    r.apad = pad;
    // keep the sorted voxel list and run starts for the remaining steps and the host copies
    r.cell = std::move(cell);
    r.gstart = std::move(gstart);
    r.key = std::move(key);
    r.vl = std::move(vl);
}

void setup_ap_arrays_device(cudaStream_t s, const DedupResult &r, const double *d_at_cells, double *at, float2 *at_hilo,
                            int32_t *a_layer, int64_t *a_vb) {
    const int npl = (int)r.pl_layer.size();
    DBuf<int> pl, pf, pc;
    DBuf<int64_t> pb;
    pl.alloc(npl);
    pf.alloc(npl);
    pc.alloc(npl);
    pb.alloc(npl);
    EKG_CUDA(cudaMemcpyAsync(pl.p, r.pl_layer.data(), npl * sizeof(int), cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(pf.p, r.pfirst.data(), npl * sizeof(int), cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(pc.p, r.pcount.data(), npl * sizeof(int), cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(pb.p, r.pbase.data(), npl * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    const int64_t slots = r.apad + 1;
    k_ap_arrays<<<(unsigned)((slots + 255) / 256), 256, 0, s>>>(r.apad, npl, pl.p, pb.p, pf.p, pc.p, (int)r.naps,
                                                                (int)r.nvox, r.gstart.p, r.cell.p, d_at_cells, at,
                                                                at_hilo, a_layer, a_vb);
    EKG_CUDA(cudaGetLastError());
    EKG_CUDA(cudaStreamSynchronize(s));  // the small tables above are freed on return
}

int64_t setup_voxel_records_device(cudaStream_t s, const DedupResult &r, int nz, int ny, int nx, const uint8_t *d_lay,
                                   const HeartDev &D, int few_max, int32_t *vzyx, uint32_t *vin, uint32_t *vout,
                                   float4 *vpos, float4 *vosum) {
    VoxelGeom g;
    g.nz = nz;
    g.ny = ny;
    g.nx = nx;
    g.nnb = D.nnb;
    for (int i = 0; i < 26 * 3; ++i) g.dif[i] = D.nb_dif[i];
    g.interior_mask = D.interior_mask;
    g.few_max = few_max;
    g.cz = D.centre[0];
    g.cy = D.centre[1];
    g.cx = D.centre[2];
    DBuf<unsigned long long> cnt;
    cnt.alloc(1);
    EKG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
    const int nv = (int)r.nvox;
    k_voxel_records<<<(nv + 255) / 256, 256, 0, s>>>(nv, g, r.cell.p, d_lay, r.vl.p, r.key.p, vzyx, vin, vout, vpos,
                                                     vosum, cnt.p);
    EKG_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    EKG_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaStreamSynchronize(s));
    return (int64_t)h;
}

// ------------------------------------------------------------------ stage bounding boxes
// Block per 32-AP stage: the lowest and highest voxel position over the stage's voxels, so that the
// operand kernel can tell for a whole stage whether every voxel is far from a lead.
__global__ void k_stage_boxes(int64_t nst, const int64_t *__restrict__ a_vox_begin, const float4 *__restrict__ vox_pos,
                              float4 *__restrict__ box) {
    __shared__ float red[6][4];
    const int64_t st = blockIdx.x;
    const int64_t v0 = a_vox_begin[st * 32], v1 = a_vox_begin[st * 32 + 32];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
        const float4 p = vox_pos[v];
        lo[0] = fminf(lo[0], p.x);
        lo[1] = fminf(lo[1], p.y);
        lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x);
        hi[1] = fmaxf(hi[1], p.y);
        hi[2] = fmaxf(hi[2], p.z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            red[k][w] = lo[k];
            red[3 + k][w] = hi[k];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 1; j < (int)(blockDim.x >> 5); ++j)
            for (int k = 0; k < 3; ++k) {
                red[k][0] = fminf(red[k][0], red[k][j]);
                red[3 + k][0] = fmaxf(red[3 + k][0], red[3 + k][j]);
            }
        box[2 * st] = make_float4(red[0][0], red[1][0], red[2][0], 0.f);
        box[2 * st + 1] = make_float4(red[3][0], red[4][0], red[5][0], 0.f);
    }
}

void setup_stage_boxes_device(cudaStream_t s, int64_t apad, const int64_t *a_vox_begin, const float4 *vox_pos,
                              float4 *stage_box) {
    const int64_t nst = apad / 32;
    if (nst <= 0) return;
    k_stage_boxes<<<(unsigned)nst, 128, 0, s>>>(nst, a_vox_begin, vox_pos, stage_box);
    EKG_CUDA(cudaGetLastError());
}

}  // namespace ekg
