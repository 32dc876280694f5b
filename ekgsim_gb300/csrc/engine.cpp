// engine.cpp -- C ABI of the engine: engine and heart lifetime, plain and batched evaluation,
// simulator.ini front end.
#include <algorithm>
#include <climits>
#include <array>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <stdexcept>

#include "ekg_engine.h"

namespace ekg {

static thread_local std::string g_last_error;
void set_error(const std::string &m) { g_last_error = m; }

int guard(const std::function<void()> &f) {
    try {
        f();
        g_last_error.clear();
        return EKG_OK;
    } catch (const Error &e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return EKG_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_error(e.what());
        return EKG_ERR_BAD_INPUT;
    }
}

// neighbour offsets (z,y,x) in the reference's creation order (simlib/simulator.h:334-384)
int neighbourhood(int code, int8_t *dif) {
    int cnt = 0;
    for (int a0 = 0; a0 < 3; ++a0)
        for (int a1 = 0; a1 < 3; ++a1)
            for (int a2 = 0; a2 < 3; ++a2) {
                const int d0 = std::abs(a0 - 1), d1 = std::abs(a1 - 1), d2 = std::abs(a2 - 1);
                bool ok = false;
                if (code == EKG_NHOOD_3D4) ok = std::min({d0, d1, d2}) == 1 && std::max({d0, d1, d2}) == 1;
                else if (code == EKG_NHOOD_CUBE) ok = std::max({d0, d1, d2}) == 1;
                else if (code == EKG_NHOOD_2D4) ok = std::min(d1, d2) == 1 && std::max(d1, d2) == 1 && d0 == 0;
                else if (code == EKG_NHOOD_2D8) ok = std::max(d1, d2) == 1 && d0 == 0;
                if (ok) {
                    dif[3 * cnt] = (int8_t)(a0 - 1);
                    dif[3 * cnt + 1] = (int8_t)(a1 - 1);
                    dif[3 * cnt + 2] = (int8_t)(a2 - 1);
                    ++cnt;
                }
            }
    return cnt;
}

// Coefficients of the closed-form interior field (batch.cu, voxel_w_*): for a neighbour set that
// is invariant under the 48 signed axis permutations, sum_n (d.grad)^4 phi = c4 sum_i d_i^4 phi and
// sum_n (d.grad)^6 phi = c6 sum_i d_i^6 phi for harmonic phi, with c4 = a4 - b4/2 and
// c6 = a6 - b6 + g6/3 from the moments a4 = sum d_x^4, b4 = 6 sum d_x^2 d_y^2, a6 = sum d_x^6,
// b6 = 15 sum d_x^4 d_y^2, g6 = 90 sum d_x^2 d_y^2 d_z^2.
void interior_field(HeartDev &D) {
    D.interior_mask = 0;
    std::vector<std::array<int, 3>> set;
    for (int n = 0; n < D.nnb; ++n) set.push_back({D.nb_dif[3 * n], D.nb_dif[3 * n + 1], D.nb_dif[3 * n + 2]});
    std::sort(set.begin(), set.end());
    const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    for (const auto &pm : perms)
        for (int sg = 0; sg < 8; ++sg) {
            std::vector<std::array<int, 3>> t;
            for (const auto &d : set) {
                std::array<int, 3> e;
                for (int i = 0; i < 3; ++i) e[i] = d[pm[i]] * ((sg >> i) & 1 ? -1 : 1);
                t.push_back(e);
            }
            std::sort(t.begin(), t.end());
            if (t != set) return;
        }
    double a4 = 0, b4 = 0, a6 = 0, b6 = 0, g6 = 0;
    for (const auto &d : set) {
        const double x = d[0], y = d[1], z = d[2];
        a4 += x * x * x * x;
        b4 += 6 * x * x * y * y;
        a6 += x * x * x * x * x * x;
        b6 += 15 * x * x * x * x * y * y;
        g6 += 90 * x * x * y * y * z * z;
    }
    const double f4 = (a4 - b4 / 2) / 6, f6 = (a6 - b6 + g6 / 3) / 120;
    // rho^5 (a1 T4 + a0) + rho^7 (b2 T6 + b1 T4 + b0) with a0 = -63 f4, a1 = 105 f4, b0 = 4050 f6,
    // b1 = -14175 f6, b2 = 10395 f6, stored as the coefficients of the symmetric-function form
    // A0 = a0 + a1, A1 = -2 a1, B0 = b0 + b1 + b2, B1 = -3 b2 - 2 b1, B2 = 3 b2
    D.interior_c[0] = (float)(42 * f4);
    D.interior_c[1] = (float)(-210 * f4);
    D.interior_c[2] = (float)(270 * f6);
    D.interior_c[3] = (float)(-2835 * f6);
    D.interior_c[4] = (float)(31185 * f6);
    D.interior_mask = D.nnb >= 32 ? 0xFFFFFFFFu : (1u << D.nnb) - 1u;
}

// ------------------------------------------------------------------ heart setup
// Host worker threads (heart set-up, the FP64 layer-AP fits of a pass): run(n, f) calls f(begin, end)
// on contiguous parts of [0, n), one per thread, the caller taking the first; one job at a time.
class HostPool {
  public:
    static HostPool &get() {
        static HostPool p;
        return p;
    }
    void run(size_t n, const std::function<void(size_t, size_t)> &f) {
        std::lock_guard<std::mutex> one(run_mu_);
        const size_t parts = std::min(n, workers_.size() + 1);
        if (parts <= 1) {
            f(0, n);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &f;
            n_ = n;
            parts_ = parts;
            remaining_ = (int)parts - 1;
            failed_ = false;
            ++gen_;
        }
        cv_.notify_all();
        bool mine_failed = false;
        try {
            f(0, n / parts);
        } catch (...) {
            mine_failed = true;
        }
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return remaining_ == 0; });
        job_ = nullptr;
        if (mine_failed || failed_) throw Error{EKG_ERR_OUT_OF_MEMORY, "host worker failed (allocation)"};
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }

  private:
    HostPool() {
        const unsigned hc = std::thread::hardware_concurrency();
        const size_t nw = hc > 1 ? std::min<unsigned>(hc, 32) - 1 : 0;
        for (size_t w = 0; w < nw; ++w) workers_.emplace_back([this, w] { loop(w + 1); });
    }
    void loop(size_t part) {
        int seen = 0;
        for (;;) {
            const std::function<void(size_t, size_t)> *f;
            size_t n, parts;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                f = job_;
                n = n_;
                parts = parts_;
            }
            bool bad = false;
            if (part < parts) {
                try {
                    (*f)(n * part / parts, n * (part + 1) / parts);
                } catch (...) {
                    bad = true;
                }
                std::lock_guard<std::mutex> lk(mu_);
                failed_ = failed_ || bad;
                if (--remaining_ == 0) done_cv_.notify_all();
            }
        }
    }
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t, size_t)> *job_ = nullptr;
    size_t n_ = 0, parts_ = 0;
    int gen_ = 0, remaining_ = 0;
    bool stop_ = false, failed_ = false;
};

void heart_setup(ekg_heart *h, const ekg_heart_desc *d) {
    auto t0 = std::chrono::steady_clock::now();
    EKG_CHECK(d && d->layers && d->transfer && d->leads_zyx, EKG_ERR_BAD_INPUT, "null heart description field");
    EKG_CHECK(d->nz >= 1 && d->ny >= 1 && d->nx >= 1 && d->nz < 1024 && d->ny < 1024 && d->nx < 1024,
              EKG_ERR_BAD_INPUT, "grid extents must be in 1..1023");
    EKG_CHECK(d->n_leads >= 1 && d->n_leads <= 1024, EKG_ERR_BAD_INPUT, "n_leads must be in 1..1024");
    EKG_CHECK(d->dt > 0 && d->length > 0, EKG_ERR_BAD_INPUT, "time step and length must be positive");
    h->nz = d->nz;
    h->ny = d->ny;
    h->nx = d->nx;
    const int64_t n = (int64_t)d->nz * d->ny * d->nx;
    h->ncell = n;
    h->start = d->start;
    h->length = d->length;
    h->dt = d->dt;
    h->nhood = d->nhood;
    h->leads0.assign(d->leads_zyx, d->leads_zyx + 3 * d->n_leads);
    h->lead_uv.resize(6 * (size_t)d->n_leads);
    lead_frames(d->n_leads, h->leads0.data(), h->lead_uv.data());
    HeartDev &D = h->dev;
    D.nz = d->nz;
    D.ny = d->ny;
    D.nx = d->nx;
    D.nleads = d->n_leads;
    D.nhood = d->nhood;
    D.nnb = neighbourhood(d->nhood, D.nb_dif);
    EKG_CHECK(D.nnb > 0, EKG_ERR_BAD_INPUT, "unknown neighbourhood (only know of these: 2D4, 3D4, 2D8, 3D8 (cube))");
    interior_field(D);

    // time axis: simTime accumulated by += dt from start (simlib/simulator.cpp:496-500, 519)
    const int64_t steps = (int64_t)std::ceil(d->length / d->dt);
    {
        int64_t cnt = 0;
        const double total = d->length + d->start;
        for (double s = d->start; s < total; s += d->dt) ++cnt;
        EKG_CHECK(cnt == steps && steps > 0 && steps < (1 << 24), EKG_ERR_BAD_INPUT,
                  "time step does not divide the simulation length into ceil(length/dt) steps");
    }
    D.steps = (int)steps;
    h->t.resize(steps);
    {
        double s = d->start;
        for (int64_t i = 0; i < steps; ++i) {
            h->t[i] = s;
            s += d->dt;
        }
    }

    // layers, stimulus, validation: in parts on the host pool (per part its largest layer, present
    // layers, first out-of-range cell and stimulus cells in order)
    std::vector<uint8_t> lay(n), st(n);
    const size_t vparts = (size_t)std::min<int64_t>(64, std::max<int64_t>(1, n / 65536));
    struct Part {
        int nl = 0;
        int64_t bad = -1;
        std::vector<int64_t> starts;
        char present[256] = {0};
    };
    std::vector<Part> parts(vparts);
    HostPool::get().run(vparts, [&](size_t pb, size_t pe) {
        for (size_t q = pb; q < pe; ++q) {
            Part &P = parts[q];
            for (int64_t i = n * (int64_t)q / (int64_t)vparts; i < n * (int64_t)(q + 1) / (int64_t)vparts; ++i) {
                const int32_t v = d->layers[i];
                // widened before the negation, so that INT32_MIN is rejected rather than overflowing
                const int64_t a = v < 0 ? -(int64_t)v : (int64_t)v;
                if (a > 254) {
                    if (P.bad < 0) P.bad = i;
                    continue;
                }
                lay[i] = (uint8_t)a;
                st[i] = v < 0;
                if (v < 0) P.starts.push_back(i);
                P.nl = std::max(P.nl, (int)a);
                P.present[a] = 1;
            }
        }
    });
    int nl = 0;
    int64_t nstart = 0;
    std::vector<char> present(256, 0);
    for (const Part &P : parts) {
        EKG_CHECK(P.bad < 0, EKG_ERR_BAD_INPUT, "layer ids must be at most 254");
        nl = std::max(nl, P.nl);
        nstart += (int64_t)P.starts.size();
        for (int a = 0; a < 256; ++a) present[a] = present[a] || P.present[a];
    }
    // a loaded sequence replaces the automaton (simlib/sim_lib.h:224-231): the stimulus and the
    // conduction matrix are not used then
    const bool loaded = d->activation_in != nullptr;
    EKG_CHECK(loaded || nstart > 0, EKG_ERR_NO_START, "Could not find starting point for excitation sequence");
    EKG_CHECK(nl >= 1, EKG_ERR_BAD_INPUT, "model has no non-empty voxel");
    D.nlayers = nl;
    const int nt = d->n_transfer;
    const int nl1 = nl + 1;
    std::vector<double> lag((size_t)nl1 * nl1 * 3, 0.0);
    if (loaded) {
        for (int64_t i = 0; i < n; ++i)
            if (lay[i]) {
                const double v = d->activation_in[i];
                EKG_CHECK(std::isfinite(v) && v >= 0, EKG_ERR_BAD_INPUT,
                          "loaded activation times of non-empty cells must be finite and non-negative");
            }
    } else {
        for (int a = 1; a <= nl; ++a)
            if (present[a] && a >= nt)
                throw Error{EKG_ERR_TRANSFER, "transfer (conduction) matrix does not define layer " + std::to_string(a)};
        for (int s = 1; s <= nl; ++s)
            for (int t = 1; t <= nl; ++t)
                if (present[s] && present[t]) {
                    const double v = d->transfer[(size_t)s * nt + t];
                    EKG_CHECK(v >= 0 && std::isfinite(v), EKG_ERR_BAD_INPUT,
                              "conduction delays between present layers must be finite and non-negative");
                }
        for (int s = 1; s <= nl; ++s)
            for (int t = 1; t <= nl; ++t)
                for (int k = 1; k <= 3; ++k) {
                    double l = d->transfer[(size_t)s * nt + t];
                    l *= std::sqrt((double)k);  // simlib/simulator.cpp:239-240
                    lag[((size_t)s * nl1 + t) * 3 + (k - 1)] = l;
                }
    }
    std::vector<int32_t> start_tiles;
    {
        const int ntx = (d->nx + 7) / 8, nty = (d->ny + 7) / 8;
        std::vector<char> seen((size_t)ntx * nty * ((d->nz + 7) / 8), 0);
        for (const Part &P : parts)
            for (const int64_t i : P.starts) {
                const int64_t z = i / ((int64_t)d->ny * d->nx), y = (i / d->nx) % d->ny, x = i % d->nx;
                const int64_t tile = ((z / 8) * nty + (y / 8)) * ntx + (x / 8);
                if (!seen[tile]) {
                    seen[tile] = 1;
                    start_tiles.push_back((int32_t)tile);
                }
            }
    }

    h->layer_host.assign(lay.begin(), lay.end());
    // activation times on the device
    EKG_CUDA(cudaSetDevice(h->eng->device));
    if (!h->stream) EKG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    if (!h->aux_stream) {
        EKG_CUDA(cudaStreamCreateWithFlags(&h->aux_stream, cudaStreamNonBlocking));
        for (cudaEvent_t *e : {&h->ev_fork, &h->ev_op, &h->ev_join})
            EKG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (!h->err_host) EKG_CUDA(cudaMallocHost(&h->err_host, sizeof(uint32_t)));
    EKG_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->eng->device));
    h->ev.err.alloc(1);
    cudaStream_t s = h->stream;
    // activation times (the layer grid stays on the device for the de-duplication)
    DBuf<uint8_t> dl;
    dl.alloc(n);
    EKG_CUDA(cudaMemcpyAsync(dl.p, lay.data(), n, cudaMemcpyHostToDevice, s));
    if (loaded) {
        // -0.0 keys like +0.0 in the reference's std::map (simlib/simulator.cpp:570-590)
        std::vector<double> at_in(d->activation_in, d->activation_in + n);
        for (double &v : at_in)
            if (v == 0.0) v = 0.0;
        h->at_cells.alloc(n);
        EKG_CUDA(cudaMemcpyAsync(h->at_cells.p, at_in.data(), n * 8, cudaMemcpyHostToDevice, s));
        h->ca_rounds = 0;
        h->ca_ms = 0;
        EKG_CUDA(cudaStreamSynchronize(s));
    } else {
        DBuf<uint8_t> ds;
        DBuf<double> dlag;
        ds.alloc(n);
        dlag.alloc(lag.size());
        h->at_cells.alloc(n);
        EKG_CUDA(cudaMemcpyAsync(ds.p, st.data(), n, cudaMemcpyHostToDevice, s));
        EKG_CUDA(cudaMemcpyAsync(dlag.p, lag.data(), lag.size() * 8, cudaMemcpyHostToDevice, s));
        int64_t nvox_h = 0;
        for (int64_t i = 0; i < n; ++i) nvox_h += lay[i] != 0;
        CaResult r;
        if (h->eng->ca_mode == 1 ||
            !ca_run_buckets(s, d->nz, d->ny, d->nx, dl.p, ds.p, lag, nl1, dlag.p, h->at_cells.p, nvox_h,
                            h->eng->ca_round_cap, h->sm_count, r))
            r = ca_run(s, d->nz, d->ny, d->nx, dl.p, ds.p, start_tiles, nl1, dlag.p, h->at_cells.p,
                       h->eng->ca_round_cap, h->sm_count);
        h->ca_rounds = r.rounds;
        h->ca_ms = r.ms;
        h->ca_buckets = r.buckets;
        EKG_CUDA(cudaStreamSynchronize(s));
    }
    h->at_host.clear();  // copied to the host on first use (ensure_at_host)

    // de-duplicate (layer, at) pairs on the device (setup.cu): voxels sorted by (layer, at bits,
    // cell), equal (layer, at) runs are the APs.  The reference numbers APs by first appearance in
    // raster order (simlib/simulator.cpp:570-590); that numbering is derived on demand.
    EKG_CHECK(n < ((int64_t)1 << 31), EKG_ERR_BAD_INPUT, "grid too large");
    DedupResult dd;
    setup_voxels_device(s, d->nz, d->ny, d->nx, dl.p, h->at_cells.p, nl, dd);
    const int64_t nv = dd.nvox, na = dd.naps, apad = dd.apad;
    h->nvox = nv;
    D.nvox = nv;
    h->naps = na;
    D.naps = na;
    EKG_CHECK(apad < (int64_t)1 << 31, EKG_ERR_BAD_INPUT, "too many distinct activation times");
    D.apad = apad;
    D.centre[0] = 0.5 * d->nz;
    D.centre[1] = 0.5 * d->ny;
    D.centre[2] = 0.5 * d->nx;
    // chunks of up to chunk_len APs inside one layer's padded range
    const int chunk_len = h->eng->chunk_len;
    std::vector<int32_t> c0, c1, cl;
    for (size_t k = 0; k < dd.pl_layer.size(); ++k) {
        const int64_t base = dd.pbase[k], padded = (dd.pcount[k] + 63) / 64 * 64;
        for (int64_t j = 0; j < padded; j += chunk_len) {
            c0.push_back((int32_t)(base + j));
            c1.push_back((int32_t)(base + std::min<int64_t>(padded, j + chunk_len)));
            cl.push_back(dd.pl_layer[k] - 1);
        }
    }
    D.nchunks = (int)c0.size();
    D.chunk_max = 0;
    for (size_t k = 0; k < c0.size(); ++k) D.chunk_max = std::max(D.chunk_max, c1[k] - c0[k]);
    D.at.alloc(apad);
    D.at_hilo.alloc(apad);
    D.a_layer.alloc(apad);
    D.a_vox_begin.alloc(apad + 1);
    D.vox_zyx.alloc(nv);
    D.vox_nb.alloc(nv);
    D.vox_nbo.alloc(nv);
    D.vox_pos.alloc(nv);
    D.vox_out.alloc(nv);
    D.chunk_a0.alloc(c0.size());
    D.chunk_a1.alloc(c0.size());
    D.chunk_layer.alloc(c0.size());
    D.difs.alloc(3 * D.nnb);
    D.t.alloc(steps);
    D.t_hilo.alloc(steps);
    setup_ap_arrays_device(s, dd, h->at_cells.p, D.at.p, D.at_hilo.p, D.a_layer.p, D.a_vox_begin.p);
    // absent neighbours up to which the closed form minus their terms is cheaper than the sum over
    // the present ones (the 8 body diagonals have a cheaper direct sum)
    const int few_max = D.nhood == EKG_NHOOD_3D4 ? 2 : D.nnb / 2;
    D.n_interior = setup_voxel_records_device(s, dd, d->nz, d->ny, d->nx, dl.p, D, few_max, D.vox_zyx.p, D.vox_nb.p,
                                              D.vox_nbo.p, D.vox_pos.p, D.vox_out.p);
    D.stage_box.alloc((size_t)2 * (apad / 32));
    setup_stage_boxes_device(s, apad, D.a_vox_begin.p, D.vox_pos.p, D.stage_box.p);
    {
        // work items of the moved-lead field kernels: stages with the most voxels first
        // (longest-first), ties by index
        const int64_t nst = apad / 32;
        std::vector<int64_t> vb(apad + 1);
        EKG_CUDA(cudaMemcpyAsync(vb.data(), D.a_vox_begin.p, vb.size() * 8, cudaMemcpyDeviceToHost, s));
        EKG_CUDA(cudaStreamSynchronize(s));
        std::vector<int32_t> order(nst);
        for (int64_t st = 0; st < nst; ++st) order[st] = (int32_t)st;
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            return vb[32 * (a + 1)] - vb[32 * a] > vb[32 * (b + 1)] - vb[32 * b];
        });
        D.stage_order.alloc(nst);
        EKG_CUDA(cudaMemcpy(D.stage_order.p, order.data(), nst * 4, cudaMemcpyHostToDevice));
    }
    // host copies of the sorted voxel cells and AP starts, for the reference's AP numbering
    h->vox_cell.resize(nv);
    h->vox_group_start.resize(na + 1);
    EKG_CUDA(cudaMemcpyAsync(h->vox_cell.data(), dd.cell.p, nv * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaMemcpyAsync(h->vox_group_start.data(), dd.gstart.p, na * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    h->ap_index_ref.clear();
    std::vector<float2> th(steps);
    for (int64_t i = 0; i < steps; ++i) {
        const float hi = (float)h->t[i];
        th[i] = make_float2(hi, (float)(h->t[i] - (double)hi));
    }
    EKG_CUDA(cudaMemcpyAsync(D.chunk_a0.p, c0.data(), c0.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.chunk_a1.p, c1.data(), c0.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.chunk_layer.p, cl.data(), c0.size() * 4, cudaMemcpyHostToDevice, s));
    // chunk range of each layer (a layer's chunks are contiguous)
    std::vector<int32_t> lc0v(nl, 0), lc1v(nl, 0);
    for (size_t k = 0; k < cl.size(); ++k) {
        const int L = cl[k];
        if (lc0v[L] == lc1v[L]) lc0v[L] = (int32_t)k;
        lc1v[L] = (int32_t)k + 1;
    }
    D.layer_c0.alloc(nl);
    D.layer_c1.alloc(nl);
    EKG_CUDA(cudaMemcpyAsync(D.layer_c0.p, lc0v.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.layer_c1.p, lc1v.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.difs.p, D.nb_dif, 3 * D.nnb, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.t.p, h->t.data(), steps * 8, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(D.t_hilo.p, th.data(), steps * 8, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaStreamSynchronize(s));
    h->vox_group_start[na] = (int32_t)nv;
    // resident lead field for the loaded lead positions
    h->leads0_dev.alloc(3 * D.nleads);
    EKG_CUDA(cudaMemcpyAsync(h->leads0_dev.p, h->leads0.data(), h->leads0.size() * 8, cudaMemcpyHostToDevice, s));
    h->W0.alloc((size_t)D.nleads * apad);
    launch_lead_field(s, D, h->leads0_dev.p, D.nleads, D.nleads, 1, h->W0.p, D.nleads);
    EKG_CUDA(cudaStreamSynchronize(s));
    h->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

int64_t heart_device_bytes(const ekg_heart *h) {
    const HeartDev &D = h->dev;
    int64_t b = D.at.bytes() + D.at_hilo.bytes() + D.a_layer.bytes() + D.a_vox_begin.bytes() + D.vox_zyx.bytes() +
                D.vox_nb.bytes() + D.vox_nbo.bytes() + D.chunk_a0.bytes() * 3 + D.t.bytes() + D.t_hilo.bytes() +
                h->W0.bytes() + h->at_cells.bytes() + D.vox_pos.bytes() + D.vox_out.bytes() + D.stage_box.bytes();
    const EvalDev &E = h->ev;
    b += (int64_t)h->stg[0].dev.bytes() + (int64_t)h->stg[1].dev.bytes() + E.layer_c.bytes() + E.F.bytes() + E.k0w.bytes() + E.W.bytes() +
         E.Wp.bytes() + E.partial.bytes() + E.ecg.bytes() + E.ecg_ff.bytes() + E.coef.bytes() + E.crit.bytes() + E.targets.bytes() +
         E.targets_ff.bytes();
    return b;
}

// ------------------------------------------------------------------ evaluation
int64_t eval_bytes_per_sim(const ekg_heart *h) {
    const HeartDev &D = h->dev;
    const int64_t L = D.nleads, nl = D.nlayers;
    return nl * 9 * 8 + L * 3 * 8 + nl * 4 * 4 + nl * D.steps * 8 + L * 8 + 2 * L * D.apad * 4 +
           (int64_t)D.nchunks * L * D.steps * 8 + 2 * L * D.steps * 8 + std::max<int64_t>(1, L) * 2 * 8;
}
int64_t eval_bytes_held(const ekg_heart *h) { return (int64_t)h->ev.cap_sims * eval_bytes_per_sim(h); }

void ensure_eval_capacity(ekg_heart *h, int n_sims) {
    EvalDev &E = h->ev;
    const HeartDev &D = h->dev;
    if (E.cap_sims >= n_sims) return;
    const size_t S = (size_t)n_sims;
    E.layer_c.alloc(S * D.nlayers * 4);
    E.F.alloc(S * D.nlayers * D.steps);
    E.Ff.alloc(S * D.nlayers * D.steps);
    E.k0w.alloc(S * D.nleads);
    E.ecg.alloc(S * D.nleads * D.steps);
    E.ecg_ff.alloc(S * D.nleads * D.steps);
    E.crit.alloc(S * std::max(1, D.nleads) * 2);
    E.err.alloc(1);
    E.cap_sims = n_sims;
}
// moved rows (simulations x moved leads) from which the per-simulation form evaluates their field
// with the persistent row kernel (below: one thread per (AP, simulation)); measured at 160^3 with 2
// moved leads: 8 rows 0.067 ms both, 2 rows 0.036 against 0.067, 32 rows 0.073 against 0.197
constexpr int SIM_ROWS_PERSISTENT = 8;
// whether the per-simulation form contracts with the band form (compact outputs)
bool band_contraction(const ekg_heart *h) {
    return h->eng->contract == EKG_CONTRACT_BAND && h->dev.chunk_max <= CONTRACT_BAND_CAP;
}
// buffers of the general (per-simulation AP) form
void ensure_general_capacity(ekg_heart *h, int n_sims) {
    EvalDev &E = h->ev;
    const HeartDev &D = h->dev;
    const size_t S = (size_t)n_sims;
    const size_t nw = S * D.nleads * D.apad, np = S * D.nchunks * D.nleads * D.steps;
    if (E.W.n < nw) {
        E.W.alloc(nw);
        E.Wp.alloc(nw);
    }
    if (E.work.n < 1) E.work.alloc(1);
    if (band_contraction(h)) {
        if (E.band.n < np) E.band.alloc(np);
        if (E.csum.n < S * D.nchunks * D.nleads) E.csum.alloc(S * D.nchunks * D.nleads);
        if (E.cinfo.n < S * D.nchunks) E.cinfo.alloc(S * D.nchunks);
    } else if (E.partial.n < np) {
        E.partial.alloc(np);
    }
}

// Device pass for n_sims simulations, split into upload / compute / download so the benchmark
// can time the compute part with its inputs resident.  layer_k [S][nl][9], leads [S][L][3] (host).
struct PassTiming {
    // start, after the lead-field part, after the contraction, end, around the moved-lead operand kernel
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool on = false;
};
static int g_launch_count = 0;

// Taylor order for exp(x) on |x| <= xmax with truncation bound xmax^J / J! * e^xmax <= 1e-12.
int taylor_terms(double xmax, int jmax) {
    double term = 1.0;  // xmax^J / J!
    for (int J = 1; J <= jmax; ++J) {
        term *= xmax / J;
        if (term * std::exp(xmax) <= 1e-12) return J;
    }
    return -1;
}

// Band structure of the moved-lead GEMM for per-layer (k1, k4) = key (batch.cu explains the
// split).  Per layer L (APs [a0, a1), finite ones ascending first, padding after) and 128-step tile
// j starting at t0: the steady prefix of the tile ends at the first AP with at >= t0 - T+ rounded
// down to a 32-AP stage (the whole layer once every finite AP is steady), the band ends at the first
// AP with at > t_last + T- rounded up.  Tiles before the first all-steady tile jf share at most
// MAXE - 1 steady prefixes ("entries"): a tile uses the prefix of the first tile of its group,
// which is shorter, so its band only grows.  Tiles from jf on use the whole-layer entry.  Rounding
// and grouping only move APs into the band, where they are exact.
void build_band(ekg_heart *h, const std::vector<double> &key, const std::vector<double> &at_h,
                const std::vector<int32_t> &al) {
    constexpr int MAXE = 8;
    BatchState &B = h->bs;
    const HeartDev &D = h->dev;
    cudaStream_t s = h->stream;
    const int nl = D.nlayers, steps = D.steps, ntt = (steps + 127) / 128;
    const double LN2 = 0.69314718055994531;
    std::vector<int64_t> la0(nl, -1), la1(nl, -1), nfin(nl, 0);
    for (int64_t a = 0; a < D.apad; ++a) {
        const int L = al[a];
        if (la0[L] < 0) la0[L] = a;
        la1[L] = a + 1;
        if (std::isfinite(at_h[a])) ++nfin[L];
    }
    B.ntt = ntt;
    B.band_s0.assign((size_t)nl * ntt, 0);
    B.band_s1.assign((size_t)nl * ntt, 0);
    std::vector<int32_t> nent(nl, 0), esplit((size_t)nl * MAXE, 0), ent((size_t)nl * ntt, -1);
    std::vector<int32_t> ls0(nl, 0), ls1(nl, 0);
    // per 32-AP stage its last finite activation time (hi, lo as the device's at_hilo), 0 if none
    const int64_t nst = D.apad / 32;
    std::vector<double> tr(nst, NAN);
    std::vector<float2> tref(nst, make_float2(0.f, 0.f));
    for (int64_t st = 0; st < nst; ++st)
        for (int64_t a = 32 * st + 31; a >= 32 * st; --a)
            if (std::isfinite(at_h[a])) {
                tr[st] = at_h[a];
                const float hi = (float)at_h[a];
                tref[st] = make_float2(hi, (float)(at_h[a] - (double)hi));
                break;
            }
    std::vector<int64_t> goff((size_t)nl * MAXE, 0);
    std::vector<float> gtab;
    std::vector<float> E((size_t)nl * steps, 1.f);
    int max_ent = 1;
    for (int L = 0; L < nl; ++L) {
        if (la0[L] < 0) continue;
        const double k1 = key[2 * L], k4 = key[2 * L + 1];
        const int64_t a0 = la0[L], a1 = la1[L], af = a0 + nfin[L];
        ls0[L] = (int32_t)(a0 / 32);
        ls1[L] = (int32_t)(a1 / 32);
        bool ok = k1 > 0 && k4 >= 0 && k1 > 1.05 * k4 && std::isfinite(k1) && std::isfinite(k4);
        for (int64_t a = a0; ok && a < a1; ++a)
            ok = a < af ? (std::isfinite(at_h[a]) && (a == a0 || at_h[a] >= at_h[a - 1])) : !std::isfinite(at_h[a]);
        const double Tp = 30 * LN2 / k1, Tn = 30 * LN2 / (k1 - k4);
        std::vector<int64_t> sp(ntt, a0), en(ntt, a1);
        int jf = ntt;
        for (int j = 0; j < ntt; ++j) {
            if (ok) {
                const double t0 = h->t[128 * j], tl = h->t[std::min(128 * j + 127, steps - 1)];
                const int64_t i = std::lower_bound(at_h.begin() + a0, at_h.begin() + af, t0 - Tp) - at_h.begin();
                sp[j] = i >= af ? a1 : i / 32 * 32;
                const int64_t e = std::upper_bound(at_h.begin() + a0, at_h.begin() + af, tl + Tn) - at_h.begin();
                en[j] = std::min(a1, (e + 31) / 32 * 32);
            }
            if (jf == ntt && sp[j] == a1) jf = j;
        }
        // entries: groups of gs tiles before jf, then the whole layer
        const int gs = std::max(1, (jf + MAXE - 2) / (MAXE - 1));
        const int ngroups = (jf + gs - 1) / gs;
        std::vector<int64_t> esp;
        std::vector<double> eref;
        for (int g = 0; g < ngroups; ++g) {
            esp.push_back(sp[g * gs]);
            eref.push_back(h->t[128 * g * gs]);
        }
        if (jf < ntt) {
            esp.push_back(a1);
            eref.push_back(h->t[128 * jf]);
        }
        nent[L] = (int32_t)esp.size();
        max_ent = std::max(max_ent, nent[L]);
        for (int j = 0; j < ntt; ++j) {
            const int e = j < jf ? j / gs : ngroups;
            ent[(size_t)L * ntt + j] = e;
            const int64_t split = esp[e];
            B.band_s0[(size_t)L * ntt + j] = (int32_t)(split / 32);
            B.band_s1[(size_t)L * ntt + j] = (int32_t)(std::max(split, en[j]) / 32);
            for (int t = 128 * j; t < std::min(steps, 128 * j + 128); ++t)
                E[(size_t)L * steps + t] = (float)std::exp(-k4 * (h->t[t] - eref[e]));
        }
        for (int e = 0; e < nent[L]; ++e) {
            // prefix ends are multiples of 32 APs from a layer start padded to 64: whole stages
            esplit[(size_t)L * MAXE + e] = (int32_t)(esp[e] / 32);
            goff[(size_t)L * MAXE + e] = (int64_t)gtab.size();
            for (int64_t st = a0 / 32; st < esp[e] / 32; ++st)
                gtab.push_back(std::isfinite(tr[st]) ? (float)std::exp(-k4 * (eref[e] - tr[st])) : 0.f);
        }
    }
    if (gtab.empty()) gtab.push_back(0.f);
    B.max_ent = max_ent;
    B.k0s_ok = false;  // the layer stage ranges are rebuilt below
    B.ls0.alloc(nl);
    B.ls1.alloc(nl);
    B.tref.alloc(nst);
    B.nent.alloc(nl);
    B.esplit.alloc((size_t)nl * MAXE);
    B.goff.alloc((size_t)nl * MAXE);
    B.gtab.alloc(gtab.size());
    B.ent.alloc((size_t)nl * ntt);
    B.E.alloc((size_t)nl * steps);
    EKG_CUDA(cudaMemcpyAsync(B.ls0.p, ls0.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.ls1.p, ls1.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.tref.p, tref.data(), nst * sizeof(float2), cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.nent.p, nent.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.esplit.p, esplit.data(), esplit.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.goff.p, goff.data(), goff.size() * 8, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.gtab.p, gtab.data(), gtab.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.ent.p, ent.data(), ent.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.E.p, E.data(), E.size() * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaStreamSynchronize(s));
}

// Build (or reuse) the static-lead Taylor basis for per-layer (k1, k4) = key.
void ensure_basis(ekg_heart *h, const std::vector<double> &key) {
    BatchState &B = h->bs;
    HeartDev &D = h->dev;
    if (B.basis_ok && B.key == key) return;
    cudaStream_t s = h->stream;
    const int nl = D.nlayers, L = D.nleads, J = 10;
    // centre and half-range of the activation times of each layer
    std::vector<double> at_h(D.apad);
    std::vector<int32_t> al(D.apad);
    EKG_CUDA(cudaMemcpyAsync(at_h.data(), D.at.p, D.apad * 8, cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaMemcpyAsync(al.data(), D.a_layer.p, D.apad * 4, cudaMemcpyDeviceToHost, s));
    EKG_CUDA(cudaStreamSynchronize(s));
    std::vector<double> lo(nl, INFINITY), hi(nl, -INFINITY);
    for (int64_t a = 0; a < D.apad; ++a)
        if (std::isfinite(at_h[a])) {
            lo[al[a]] = std::min(lo[al[a]], at_h[a]);
            hi[al[a]] = std::max(hi[al[a]], at_h[a]);
        }
    B.centre.assign(nl, 0.0);
    B.scale.assign(nl, 1.0);
    for (int i = 0; i < nl; ++i)
        if (lo[i] <= hi[i]) {
            B.centre[i] = 0.5 * (lo[i] + hi[i]);
            B.scale[i] = std::max(0.5 * (hi[i] - lo[i]), 1e-6);
        }
    B.d_centre.alloc(nl);
    B.d_scale.alloc(nl);
    EKG_CUDA(cudaMemcpyAsync(B.d_centre.p, B.centre.data(), nl * 8, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.d_scale.p, B.scale.data(), nl * 8, cudaMemcpyHostToDevice, s));
    // chunk ranges per layer (chunks of one layer are contiguous)
    std::vector<int32_t> cl(D.nchunks), c0(nl, 0), c1(nl, 0);
    EKG_CUDA(cudaMemcpy(cl.data(), D.chunk_layer.p, D.nchunks * 4, cudaMemcpyDeviceToHost));
    for (int i = 0; i < nl; ++i) {
        c0[i] = c1[i] = 0;
        bool seen = false;
        for (int c = 0; c < D.nchunks; ++c)
            if (cl[c] == i) {
                if (!seen) c0[i] = c;
                seen = true;
                c1[i] = c + 1;
            }
    }
    B.lc0.alloc(nl);
    B.lc1.alloc(nl);
    EKG_CUDA(cudaMemcpyAsync(B.lc0.p, c0.data(), nl * 4, cudaMemcpyHostToDevice, s));
    EKG_CUDA(cudaMemcpyAsync(B.lc1.p, c1.data(), nl * 4, cudaMemcpyHostToDevice, s));
    const int rows = L * J;
    DBuf<float> Wt, lc;
    DBuf<double> ones, part;
    Wt.alloc((size_t)rows * D.apad);
    lc.alloc((size_t)nl * 4);
    ones.alloc((size_t)nl * D.steps);
    part.alloc((size_t)D.nchunks * rows * D.steps);
    std::vector<double> one((size_t)nl * D.steps, 1.0);
    EKG_CUDA(cudaMemcpyAsync(ones.p, one.data(), one.size() * 8, cudaMemcpyHostToDevice, s));
    launch_taylor_w(s, D, h->W0.p, J, B.d_centre.p, B.d_scale.p, Wt.p);
    B.Q1.alloc((size_t)nl * rows * D.steps);
    B.Q2.alloc((size_t)nl * rows * D.steps);
    const double L2E = 1.4426950408889634;
    for (int basis = 0; basis < 2; ++basis) {
        std::vector<float> c((size_t)nl * 4);
        for (int i = 0; i < nl; ++i) {
            c[4 * i + 0] = (float)(key[2 * i] * L2E);
            c[4 * i + 1] = (float)(key[2 * i + 1] * L2E);
            c[4 * i + 2] = basis == 0 ? 1.f : 0.f;  // B1 = sigma(k1 tau) exp(-k4 tau)
            c[4 * i + 3] = basis == 0 ? 0.f : 1.f;  // B2 = sigma(k1 tau)
        }
        EKG_CUDA(cudaMemcpyAsync(lc.p, c.data(), c.size() * 4, cudaMemcpyHostToDevice, s));
        ContractArgs A;
        A.steps = D.steps;
        A.rows = rows;
        A.nl = nl;
        A.nchunks = D.nchunks;
        A.n_sims = 1;
        A.apad = D.apad;
        A.t_hilo = D.t_hilo.p;
        A.at_hilo = D.at_hilo.p;
        A.chunk_a0 = D.chunk_a0.p;
        A.chunk_a1 = D.chunk_a1.p;
        A.chunk_layer = D.chunk_layer.p;
        A.Wp = Wt.p;
        A.layer_c = lc.p;
        A.F = ones.p;
        A.partial = part.p;
        A.err = h->ev.err.p;
        EKG_CUDA(cudaMemsetAsync(h->ev.err.p, 0, 4, s));
        launch_contract_umma_args(s, A);
        launch_reduce_layers(s, D.steps, rows, nl, B.lc0.p, B.lc1.p, part.p, basis == 0 ? B.Q1.p : B.Q2.p);
        EKG_CUDA(cudaMemcpyAsync(h->err_host, h->ev.err.p, 4, cudaMemcpyDeviceToHost, s));
        EKG_CUDA(cudaStreamSynchronize(s));
        if (*h->err_host) throw Error{EKG_ERR_TIMEOUT, "a bounded device wait ran out (basis build)"};
    }
    build_band(h, key, at_h, al);
    B.J = J;
    B.key = key;
    B.basis_ok = true;
}

// ------------------------------------------------------------------ autotuner (batched form)
// A pass shape is the heart (grid, voxels, APs, leads, steps, neighbourhood, SM count) with the
// pass's simulations, moved leads and bases; the tuner keeps one launch shape per pass shape.
std::string tune_key(const ekg_heart *h, int n_sims, int nmove, int two_bases) {
    std::ostringstream k;
    k << "sm" << h->sm_count << ":" << h->nz << "x" << h->ny << "x" << h->nx << ":v" << h->nvox << ":a" << h->naps
      << ":L" << h->dev.nleads << ":T" << h->dev.steps << ":nh" << h->nhood << ":S" << n_sims << ":m" << nmove
      << ":b" << two_bases;
    return k.str();
}

// Launch shapes worth timing: row tiles 32 / 128 / 256 (256 not with two bases; a tile at most
// twice the rows used), GEMM work-item targets of 1, 2 and 4 CTAs per SM, for passes of up to 64
// simulations both operand-kernel forms, and for the persistent operand kernel as many blocks per
// SM as fit or 4 (a different balance of latency hiding and per-SM contention).
std::vector<TuneChoice> tune_candidates(int two_bases, int rows_used, int n_sims) {
    std::vector<TuneChoice> c;
    for (int N : {32, 128, 256}) {
        if (N == 256 && two_bases) continue;
        if (N > 32 && N / 2 >= rows_used) continue;
        for (int mult : {1, 2, 4})
            for (int small : {1, 0}) {
                if (small && n_sims > 64) continue;
                for (int bps : {0, 4}) {
                    if (small && bps) continue;
                    TuneChoice t;
                    t.tile_rows = N;
                    t.cta_mult = mult;
                    t.op_small = small;
                    t.op_bps = bps;
                    c.push_back(t);
                }
            }
    }
    return c;
}

// Cache file: one line per pass shape, "key tile_rows cta_mult op_small ms candidates"; later lines
// win.
void tune_cache_write(const std::string &path, const std::string &key, const TuneChoice &t) {
    std::ofstream f(path, std::ios::app);
    if (!f) throw Error{EKG_ERR_IO, "could not open autotuner cache " + path};
    f << key << " " << t.tile_rows << " " << t.cta_mult << " " << t.op_small << " " << t.ms << " " << t.candidates
      << " " << t.op_bps << "\n";
}
bool tune_cache_read(const std::string &path, const std::string &key, TuneChoice &out) {
    std::ifstream f(path);
    bool found = false;
    for (std::string line; std::getline(f, line);) {
        std::istringstream ss(line);
        std::string k;
        TuneChoice t;
        if (!(ss >> k >> t.tile_rows >> t.cta_mult >> t.op_small >> t.ms >> t.candidates)) continue;
        if (!(ss >> t.op_bps)) t.op_bps = 0;
        if (t.op_bps < 0 || t.op_bps > 64) continue;
        if (k != key) continue;
        if (t.tile_rows != 32 && t.tile_rows != 128 && t.tile_rows != 256) continue;
        if (t.cta_mult < 1 || t.cta_mult > 64 || t.op_small < 0 || t.op_small > 1) continue;
        out = t;
        found = true;
    }
    return found;
}

// Decide the pass: the batched (separable) form when the batch shares k1 and k4 per layer and
// exp(k5 at) has a short Taylor expansion (a single simulation once its k1, k4 are settled).
PassPlan plan_pass(ekg_heart *h, int n_sims, const double *layer_k, const double *leads) {
    PassPlan P;
    P.n_sims = n_sims;
    const HeartDev &D = h->dev;
    const int nl = D.nlayers, L = D.nleads;
    for (int si = 0; si < n_sims; ++si) {
        const double *p = leads + (size_t)si * L * 3;
        for (int l = 0; l < L; ++l)
            if (p[3 * l] != h->leads0[3 * l] || p[3 * l + 1] != h->leads0[3 * l + 1] || p[3 * l + 2] != h->leads0[3 * l + 2])
                P.nmove = std::max(P.nmove, l + 1);
    }
    if (n_sims < 1 || !h->eng->batched || nl > 255) return P;
    std::vector<double> key(2 * nl);
    bool k3_uniform = true;
    for (int i = 0; i < nl; ++i) {
        key[2 * i] = layer_k[9 * i + 1];
        key[2 * i + 1] = layer_k[9 * i + 4];
    }
    for (int si = 0; si < n_sims; ++si)
        for (int i = 0; i < nl; ++i) {
            const double *k = layer_k + ((size_t)si * nl + i) * 9;
            if (k[1] != key[2 * i] || k[4] != key[2 * i + 1]) return P;
            // the resting potential k0 leaves sum_L k0_L sum_{a in L} W[l, a], which vanishes when k0
            // is the same in every layer, since the AP differences of the dipoles make
            // sum_a W[l, a] = 0 (simlib/simulator.cpp:509-525); otherwise the pass adds it
            if (k[0] != layer_k[(size_t)si * nl * 9]) P.k0 = true;
            if (k[3] != layer_k[9 * i + 3]) k3_uniform = false;
        }
    // A single simulation takes the batched form once its (k1, k4) is settled: when the basis for it
    // exists, or when the previous single call had the same values (callers that vary k1, k4 from
    // call to call keep the per-simulation form instead of rebuilding the basis each time).
    if (n_sims == 1) {
        BatchState &Bm = h->bs;
        const bool have = Bm.basis_ok && Bm.key == key;
        const bool repeat = Bm.single_key == key;
        Bm.single_key = key;
        if (!have && !repeat) return P;
    }
    ensure_basis(h, key);
    const BatchState &B = h->bs;
    double xmax = 0;
    for (int si = 0; si < n_sims; ++si)
        for (int i = 0; i < nl; ++i) xmax = std::max(xmax, std::fabs(layer_k[((size_t)si * nl + i) * 9 + 5]) * B.scale[i]);
    const int J = taylor_terms(xmax, B.J);
    if (J < 0) return P;
    P.batch = true;
    P.J = J;
    P.two_bases = k3_uniform ? 0 : 1;
    P.k3.resize((size_t)n_sims * nl);
    for (size_t i = 0; i < P.k3.size(); ++i) P.k3[i] = layer_k[9 * i + 3];
    const double L2E = 1.4426950408889634;
    for (int i = 0; i < nl; ++i)
        P.hc[i] = make_float4((float)(key[2 * i] * L2E), (float)(key[2 * i + 1] * L2E), (float)(1.0 - layer_k[9 * i + 3]),
                              (float)layer_k[9 * i + 3]);
    if (P.nmove > 0) {
        P.rows_used = n_sims * P.nmove;
        // launch shape: the autotuner's choice for this pass shape, else the built-in one
        const TuneChoice *tc = h->tune_force;
        if (!tc) {
            const std::string key = tune_key(h, n_sims, P.nmove, P.two_bases);
            auto it = h->tuned.find(key);
            if (it == h->tuned.end() && !h->eng->tune_cache.empty()) {
                TuneChoice t;
                if (tune_cache_read(h->eng->tune_cache, key, t)) it = h->tuned.emplace(key, t).first;
            }
            if (it != h->tuned.end()) tc = &it->second;
        }
        const int N = tc && tc->tile_rows > 0 ? tc->tile_rows : batch_tile_rows(P.two_bases, P.rows_used);
        P.tile_rows = N;
        P.op_small = tc && tc->op_small >= 0 ? tc->op_small : (n_sims <= small_operand_sims() ? 1 : 0);
        P.op_bps = tc ? tc->op_bps : 0;
        P.ntiles = (P.rows_used + N - 1) / N;
        P.rows = P.ntiles * N;
        // band work items: each (tile, layer) band cut into pieces of at most `per` stages, `per`
        // the smallest that keeps all items x N tiles within one wave of CTAs (one per SM)
        const int ntt = B.ntt;
        int64_t total = 0;
        for (size_t i = 0; i < B.band_s0.size(); ++i) total += B.band_s1[i] - B.band_s0[i];
        const int mult = tc && tc->cta_mult > 0 ? tc->cta_mult : (N <= 32 ? 2 : 1);
        const int target = std::max(1, h->eng->batch_ctas > 0 ? h->eng->batch_ctas : h->sm_count * mult);
        int64_t per = std::max<int64_t>(1, (total * P.ntiles + target - 1) / target);
        for (;; ++per) {
            int64_t cnt = 0;
            for (size_t i = 0; i < B.band_s0.size(); ++i) cnt += (B.band_s1[i] - B.band_s0[i] + per - 1) / per;
            if (cnt * P.ntiles <= target || per >= total) break;
        }
        P.ti0.assign((size_t)ntt * nl, 0);
        P.ti1.assign((size_t)ntt * nl, 0);
        for (int j = 0; j < ntt; ++j) {
            for (int i = 0; i < nl; ++i) {
                const int s0 = B.band_s0[(size_t)i * ntt + j], n = B.band_s1[(size_t)i * ntt + j] - s0;
                P.ti0[(size_t)j * nl + i] = P.ti1[(size_t)j * nl + i] = (int32_t)P.items.size();
                if (n <= 0) continue;
                const int nc = (int)((n + per - 1) / per);
                for (int c = 0; c < nc; ++c)
                    P.items.push_back(make_int4(j, s0 + (int)((int64_t)n * c / nc), s0 + (int)((int64_t)n * (c + 1) / nc), i));
                P.ti1[(size_t)j * nl + i] = (int32_t)P.items.size();
            }
        }
        P.nitems = (int)P.items.size();
        // per-simulation k5 and moved lead positions for the operand kernel
        P.k5l.resize((size_t)n_sims * nl);
        for (size_t i = 0; i < P.k5l.size(); ++i) P.k5l[i] = (float)(layer_k[9 * i + 5] * L2E);
        P.lrel.resize((size_t)n_sims * P.nmove);
        for (int si = 0; si < n_sims; ++si)
            for (int l = 0; l < P.nmove; ++l) {
                const double *r = leads + ((size_t)si * L + l) * 3;
                P.lrel[(size_t)si * P.nmove + l] =
                    make_float4((float)(r[0] - D.centre[0]), (float)(r[1] - D.centre[1]), (float)(r[2] - D.centre[2]), 0.f);
            }
    }
    return P;
}



void upload_inputs(ekg_heart *h, const PassPlan &P, const double *layer_k, const double *leads) {
    HeartDev &D = h->dev;
    cudaStream_t s = h->stream;
    const int n_sims = P.n_sims;
    ensure_eval_capacity(h, n_sims);
    const size_t L = D.nleads, S = n_sims, nl = D.nlayers;
    h->any_k0 = false;
    for (size_t i = 0; i < S * nl; ++i) h->any_k0 = h->any_k0 || layer_k[9 * i] != 0.0;
    // small passes: the repolarisation constant ln(2^(k7/k6) - 1) per (sim, layer) on the host
    h->cpre_on = S <= 16;
    std::vector<double> cpre;
    if (h->cpre_on) {
        cpre.resize(S * nl);
        for (size_t i = 0; i < S * nl; ++i) cpre[i] = std::log(std::pow(2.0, layer_k[9 * i + 7] / layer_k[9 * i + 6]) - 1);
    }
    // layout of the staging buffer (16-byte aligned slots)
    struct Slot {
        const void *src;
        size_t bytes, off;
    };
    std::vector<Slot> slots;
    size_t off = 0;
    auto add = [&](const void *src, size_t bytes) {
        const size_t o = off;
        if (bytes) slots.push_back(Slot{src, bytes, o});
        off = (off + bytes + 15) / 16 * 16;
        return o;
    };
    const size_t o_lk = add(layer_k, S * nl * 9 * 8);
    const size_t o_cp = add(cpre.data(), cpre.size() * 8);
    const size_t o_ld = add(leads, P.nmove > 0 ? S * L * 3 * 8 : 0);
    size_t o_k3 = 0, o_hc = 0, o_ti0 = 0, o_ti1 = 0, o_it = 0, o_k5 = 0, o_lr = 0;
    if (P.batch) {
        o_k3 = add(P.k3.data(), P.k3.size() * 8);
        o_hc = add(P.hc, nl * sizeof(float4));
        if (P.nmove > 0) {
            o_ti0 = add(P.ti0.data(), P.ti0.size() * 4);
            o_ti1 = add(P.ti1.data(), P.ti1.size() * 4);
            o_it = add(P.items.data(), P.items.size() * sizeof(int4));
            o_k5 = add(P.k5l.data(), P.k5l.size() * 4);
            o_lr = add(P.lrel.data(), P.lrel.size() * sizeof(float4));
        }
    }
    ekg_heart::Staging &sg = h->stg[h->cur];
    if (off > sg.cap) {
        const size_t cap = std::max(off, 2 * sg.cap);
        EKG_CUDA(cudaStreamSynchronize(s));  // the old buffers may still be read
        if (sg.host) cudaFreeHost(sg.host);
        sg.host = nullptr;
        sg.cap = 0;
        EKG_CUDA(cudaMallocHost(&sg.host, cap));
        sg.dev.alloc(cap);
        sg.cap = cap;
    }
    for (const Slot &sl : slots) std::memcpy(sg.host + sl.off, sl.src, sl.bytes);
    if (off) EKG_CUDA(cudaMemcpyAsync(sg.dev.p, sg.host, off, cudaMemcpyHostToDevice, s));
    const uint8_t *dv = sg.dev.p;
    ekg_heart::PassInputs &in = sg.in;
    in = ekg_heart::PassInputs();
    in.layer_k = reinterpret_cast<const double *>(dv + o_lk);
    in.cpre = h->cpre_on ? reinterpret_cast<const double *>(dv + o_cp) : nullptr;
    in.leads = P.nmove > 0 ? reinterpret_cast<const double *>(dv + o_ld) : nullptr;
    if (!P.batch && h->any_k0 && band_contraction(h) && P.nmove < D.nleads && !h->W0_layer_ok) {
        // per-layer sums of the resident lead field, once per heart
        h->W0_layer.alloc((size_t)D.nlayers * D.nleads);
        launch_w0_layer_sums(s, D, h->W0.p, h->W0_layer.p);
        h->W0_layer_ok = true;
    }
    if (P.batch) {
        in.k3 = reinterpret_cast<const double *>(dv + o_k3);
        in.hconst = reinterpret_cast<const float4 *>(dv + o_hc);
        if (P.nmove > 0) {
            in.ti0 = reinterpret_cast<const int32_t *>(dv + o_ti0);
            in.ti1 = reinterpret_cast<const int32_t *>(dv + o_ti1);
            in.items = reinterpret_cast<const int4 *>(dv + o_it);
            in.k5l = reinterpret_cast<const float *>(dv + o_k5);
            in.lrel = reinterpret_cast<const float4 *>(dv + o_lr);
        }
        BatchState &B = h->bs;
        const size_t nc = (size_t)n_sims * D.nlayers * std::max(1, P.J);
        if (h->ev.coef.n < nc) h->ev.coef.alloc(nc);
        if (P.k0 && P.nmove < (int)D.nleads) {
            if (B.cst.n < (size_t)n_sims * D.nleads) B.cst.alloc((size_t)n_sims * D.nleads);
            if (!B.k0s_ok) {
                // layer sums of the resident lead field, once per band tables (the layer ranges)
                if (B.K0s.n < (size_t)D.nlayers * D.nleads) B.K0s.alloc((size_t)D.nlayers * D.nleads);
                launch_k0_static_sums(h->stream, D.nleads, D.apad, D.nlayers, B.ls0.p, B.ls1.p, h->W0.p, B.K0s.p);
                B.k0s_ok = true;
            }
        }
        if (P.nmove > 0) {
            const size_t bt = (size_t)P.rows * D.apad * 4;
            if (B.Bt.n < bt) B.Bt.alloc(bt);
            const size_t pb = (size_t)std::max(1, P.nitems) * P.rows * 128 * (P.two_bases ? 2 : 1);
            if (B.partial.n < pb) B.partial.alloc(pb);
            const size_t p1 = (size_t)(D.apad / 32) * P.rows_used;
            if (B.P1.n < p1) B.P1.alloc(p1);
            if (P.k0) {
                if (B.P2.n < 4 * p1) B.P2.alloc(4 * p1);
                if (B.cmov.n < (size_t)P.rows_used) B.cmov.alloc(P.rows_used);
            }
            if (!B.work.p) B.work.alloc(1);
            const size_t ub = (size_t)P.rows_used * D.nlayers * B.max_ent;
            if (B.U.n < ub) {
                B.U.alloc(ub);
                B.Up.alloc(ub * band_u_parts());
            }
        }
    } else {
        ensure_general_capacity(h, n_sims);
    }
}

void compute(ekg_heart *h, const PassPlan &P, int n_crit_leads, int mode, PassTiming *tm, bool mark_static = false) {
    HeartDev &D = h->dev;
    EvalDev &E = h->ev;
    cudaStream_t s = h->stream;
    const int n_sims = P.n_sims, nmove = P.nmove;
    const size_t L = D.nleads, S = n_sims;
    int launches = 0;
    if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[0], s));
    EKG_CUDA(cudaMemsetAsync(E.err.p, 0, sizeof(uint32_t), s));
    const ekg_heart::PassInputs &in = h->in();
    // batched form with both static and moved leads: the layer factors and the static combine
    // (beside the moved-lead operand kernel, which needs neither) and the steady-sum reduction
    // (beside the band GEMM) run on the auxiliary stream, joined before the band reduction
    // (measured: other placements of the small kernels, such as the criteria of the static leads
    // beside the GEMM, lengthen the pass)
    const bool fork = P.batch && nmove > 0 && nmove < (int)L;
    cudaStream_t sx = fork ? h->aux_stream : s;
    if (fork) {
        EKG_CUDA(cudaEventRecord(h->ev_fork, s));
        EKG_CUDA(cudaStreamWaitEvent(sx, h->ev_fork, 0));
    }
    launch_layer_factors(sx, D, in.layer_k, in.cpre, n_sims, E.F.p, E.Ff.p, E.layer_c.p,
                         P.batch ? h->bs.d_centre.p : nullptr, P.batch ? h->bs.d_scale.p : nullptr, P.J,
                         P.batch ? E.coef.p : nullptr);
    ++launches;
    if (P.batch) {
        BatchState &B = h->bs;
        auto static_part = [&]() {
            launch_static_combine(sx, D, P.J, B.J, nmove, n_sims, E.Ff.p, E.coef.p, in.k3, B.Q1.p, B.Q2.p, E.ecg.p,
                                  E.ecg_ff.p, P.k0 ? B.cst.p : nullptr);
            launches += nmove < (int)L;
            if (mark_static) {
                // inside a graph capture the record must be an external event node (the copy stream
                // waits on it outside the graph)
                cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
                EKG_CUDA(cudaStreamIsCapturing(s, &cs));
                EKG_CUDA(cudaEventRecordWithFlags(h->static_done, sx,
                                                  cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                                      : cudaEventRecordDefault));
            }
        };
        if (P.k0 && nmove < (int)L) {
            launch_k0_static(sx, n_sims, (int)L, nmove, D.nlayers, B.K0s.p, in.layer_k, B.cst.p);
            ++launches;
        }
        static_part();
        if (nmove > 0) {
            if (P.rows_used < P.rows) EKG_CUDA(cudaMemsetAsync(B.Bt.p, 0, (size_t)P.rows * D.apad * 4, s));
            BandArgs U;
            U.n_sims = n_sims;
            U.nmove = nmove;
            U.nl = D.nlayers;
            U.ntt = B.ntt;
            U.steps = D.steps;
            U.rows = P.rows;
            U.rows_used = P.rows_used;
            U.nleads = (int)L;
            U.max_ent = B.max_ent;
            U.tref = B.tref.p;
            U.stage_order = D.stage_order.p;
            U.nent = B.nent.p;
            U.esplit = B.esplit.p;
            U.ls0 = B.ls0.p;
            U.ls1 = B.ls1.p;
            U.ent = B.ent.p;
            U.goff = B.goff.p;
            U.gtab = B.gtab.p;
            U.E = B.E.p;
            U.F = E.Ff.p;
            U.nb = P.two_bases ? 2 : 1;
            U.ti0 = in.ti0;
            U.ti1 = in.ti1;
            U.k3 = in.k3;
            U.partial = B.partial.p;
            U.P1 = B.P1.p;
            U.P2 = P.k0 ? B.P2.p : nullptr;
            U.cmov = P.k0 ? B.cmov.p : nullptr;
            U.U = B.U.p;
            U.Up = B.Up.p;
            U.ecg = E.ecg.p;
            U.ecg_ff = E.ecg_ff.p;
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[4], s));
            launch_batch_lead_field(s, D, P.tile_rows, P.op_small != 0, P.op_bps, in.k5l, in.hconst, in.lrel, nmove,
                                    n_sims, U, B.Bt.p, B.work.p, h->sm_count);
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[5], s));
            if (fork) {
                EKG_CUDA(cudaEventRecord(h->ev_op, s));
                EKG_CUDA(cudaStreamWaitEvent(sx, h->ev_op, 0));
            }
            launch_band_u(sx, U);
            if (P.k0) {
                launch_k0_moved(sx, U, B.ls0.p, B.ls1.p, in.layer_k, B.cmov.p);
                ++launches;
            }
            if (fork) EKG_CUDA(cudaEventRecord(h->ev_join, sx));
            launches += 2;
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[1], s));
            BatchArgs A;
            A.steps = D.steps;
            A.nl = D.nlayers;
            A.nkt = (int)(D.apad / 64);
            A.rows = P.rows;
            A.rows_used = P.rows_used;
            A.nmove = nmove;
            A.n_sims = n_sims;
            A.ntiles = P.ntiles;
            A.nitems = P.nitems;
            A.two_bases = P.two_bases;
            A.tile_rows = P.tile_rows;
            A.t_hilo = D.t_hilo.p;
            A.at_hilo = D.at_hilo.p;
            A.items = in.items;
            A.hconst = in.hconst;
            A.Bt = B.Bt.p;
            A.partial = B.partial.p;
            A.err = E.err.p;
            launch_batch_gemm(s, A);
            launches += P.nitems > 0;
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[2], s));
            if (fork) EKG_CUDA(cudaStreamWaitEvent(s, h->ev_join, 0));
            launch_reduce_band(s, U);
            ++launches;
            if (mark_static) {
                // the moved-lead rows are final too: their copy to the host overlaps the criteria
                cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
                EKG_CUDA(cudaStreamIsCapturing(s, &cs));
                EKG_CUDA(cudaEventRecordWithFlags(h->moved_done, s,
                                                  cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                                      : cudaEventRecordDefault));
            }
        } else if (tm && tm->on) {
            EKG_CUDA(cudaEventRecord(tm->ev[1], s));
            EKG_CUDA(cudaEventRecord(tm->ev[2], s));
        }
    } else {
        // lead field: recomputed rows for moved leads; the leads at their loaded position take the
        // resident field W0 (scaled inside the band contraction, or written out for the dense ones)
        const bool band = band_contraction(h);
        if (h->any_k0 && !band)
            for (size_t si = 0; si < S; ++si)
                EKG_CUDA(cudaMemcpyAsync(E.W.p + si * L * D.apad, h->W0.p, L * D.apad * 4, cudaMemcpyDeviceToDevice, s));
        if (band && nmove > 0 && n_sims * nmove >= SIM_ROWS_PERSISTENT) {
            launch_sim_lead_field_rows(s, D, in.leads, nmove, (int)L, n_sims, E.W.p, E.work.p, h->sm_count);
            ++launches;
        } else if (nmove > 0 || !band) {
            launch_sim_lead_field(s, D, in.leads, nmove, (int)L, n_sims, in.layer_k, h->W0.p, E.W.p,
                                  band ? nullptr : E.Wp.p, !band);
            ++launches;
        }
        // k0 leaves a constant term only when some layer's k0 differs from zero (AP differences
        // within a layer cancel it): sum_a k0_{layer(a)} W[l, a], from W for the moved rows and from
        // the layer sums of W0 for the others
        if (h->any_k0) {
            const int wrows = band ? nmove : (int)L;
            if (wrows > 0) {
                launch_k0_term(s, D, E.W.p, in.layer_k, n_sims, E.k0w.p, wrows);
                ++launches;
            }
            if (wrows < (int)L) {
                launch_k0_static(s, n_sims, (int)L, wrows, D.nlayers, h->W0_layer.p, in.layer_k, E.k0w.p, false);
                ++launches;
            }
        } else {
            EKG_CUDA(cudaMemsetAsync(E.k0w.p, 0, S * L * sizeof(double), s));
        }
        if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[1], s));
        if (band) {
            launch_contract_band(s, D, E.W.p, nmove, h->W0.p, in.layer_k, E.layer_c.p, n_sims, E.band.p, E.csum.p,
                                 E.cinfo.p);
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[2], s));
            launch_reduce_chunks(s, D, E.layer_c.p, E.F.p, E.band.p, E.csum.p, E.cinfo.p, E.k0w.p, n_sims, E.ecg.p,
                                 E.ecg_ff.p);
        } else {
            if (h->eng->contract != EKG_CONTRACT_DENSE_CUDA)
                launch_contract_umma(s, D, E.Wp.p, E.layer_c.p, E.F.p, n_sims, E.partial.p, E.err.p);
            else
                launch_contract_cuda(s, D, E.Wp.p, E.layer_c.p, E.F.p, n_sims, E.partial.p);
            if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[2], s));
            launch_reduce_ecg(s, D, E.partial.p, E.k0w.p, n_sims, E.ecg.p, E.ecg_ff.p);
        }
        launches += 2;
    }
    if (n_crit_leads > 0) {
        launch_criteria(s, D, E.ecg.p, E.ecg_ff.p, n_sims, n_crit_leads, 0, n_crit_leads, mode, E.targets.p,
                        E.targets_ff.p, E.target_len.p, E.target_off.p, E.crit.p);
        ++launches;
    }
    if (tm && tm->on) EKG_CUDA(cudaEventRecord(tm->ev[3], s));
    g_launch_count = launches;
}

// Everything the launches of compute() depend on: the pass shape and every device pointer it passes.
std::vector<uint64_t> pass_signature(const ekg_heart *h, const PassPlan &P, int ncl, int mode, bool mark_static) {
    const EvalDev &E = h->ev;
    const BatchState &B = h->bs;
    auto u = [](const void *p) { return (uint64_t)(uintptr_t)p; };
    std::vector<uint64_t> v = {(uint64_t)P.batch, (uint64_t)P.n_sims, (uint64_t)P.nmove, (uint64_t)P.J,
                               (uint64_t)P.two_bases, (uint64_t)P.rows, (uint64_t)P.rows_used, (uint64_t)P.ntiles,
                               (uint64_t)P.nitems, (uint64_t)ncl, (uint64_t)mode, (uint64_t)mark_static,
                               (uint64_t)h->cpre_on, (uint64_t)h->any_k0, (uint64_t)h->eng->contract, (uint64_t)B.J,
                               (uint64_t)B.max_ent, (uint64_t)B.ntt, (uint64_t)P.tile_rows, (uint64_t)P.op_small,
                               (uint64_t)P.op_bps, (uint64_t)P.k0};
    const ekg_heart::PassInputs &in = h->in();
    for (const void *p : {(const void *)in.layer_k, (const void *)in.cpre, (const void *)in.leads, (const void *)in.k3,
                          (const void *)B.d_centre.p, (const void *)B.d_scale.p, (const void *)E.coef.p,
                          (const void *)in.k5l, (const void *)in.hconst, (const void *)in.lrel,
                          (const void *)in.items, (const void *)in.ti0, (const void *)in.ti1,
                          (const void *)E.F.p, (const void *)E.Ff.p,
                          (const void *)E.layer_c.p, (const void *)E.ecg.p, (const void *)E.crit.p, (const void *)E.err.p,
                          (const void *)E.ecg_ff.p, (const void *)E.targets_ff.p, (const void *)E.targets.p, (const void *)E.target_len.p, (const void *)E.target_off.p,
                          (const void *)E.W.p, (const void *)E.Wp.p, (const void *)E.partial.p, (const void *)E.k0w.p,
                          (const void *)B.Q1.p,
                          (const void *)B.Q2.p, (const void *)B.Bt.p, (const void *)B.P1.p, (const void *)B.U.p,
                          (const void *)B.Up.p, (const void *)B.partial.p,
                          (const void *)B.tref.p, (const void *)h->dev.stage_order.p, (const void *)B.nent.p, (const void *)B.esplit.p, (const void *)B.ls0.p,
                          (const void *)B.ls1.p, (const void *)B.ent.p, (const void *)B.goff.p, (const void *)B.gtab.p,
                          (const void *)B.E.p, (const void *)B.work.p, (const void *)h->W0.p, (const void *)B.P2.p,
                          (const void *)B.cmov.p, (const void *)B.cst.p, (const void *)B.K0s.p, (const void *)E.band.p,
                          (const void *)E.csum.p, (const void *)E.cinfo.p, (const void *)h->W0_layer.p, (const void *)E.work.p,
                          (const void *)h->dev.stage_order.p})
        v.push_back(u(p));
    return v;
}

// compute() as a CUDA graph: the first pass with a signature runs directly (it also performs the
// launchers' one-time set-up), the second is captured (thread-local capture on the heart's stream)
// and instantiated, later ones replay it.  Up to four graphs per heart, least recently used out.
void run_pass(ekg_heart *h, const PassPlan &P, int ncl, int mode, bool mark_static) {
    if (!h->eng->graphs) {
        compute(h, P, ncl, mode, nullptr, mark_static);
        return;
    }
    const std::vector<uint64_t> sig = pass_signature(h, P, ncl, mode, mark_static);
    ekg_heart::PassGraph *g = nullptr, *victim = &h->graphs[0];
    for (auto &c : h->graphs) {
        if (!c.sig.empty() && c.sig == sig) g = &c;
        if (c.used < victim->used) victim = &c;
    }
    cudaStream_t s = h->stream;
    if (g && g->exec) {
        g->used = ++h->graph_clock;
        EKG_CUDA(cudaGraphLaunch(g->exec, s));
        return;
    }
    if (!g) {
        if (victim->exec) cudaGraphExecDestroy(victim->exec);
        *victim = ekg_heart::PassGraph();
        victim->sig = sig;
        victim->used = ++h->graph_clock;
        compute(h, P, ncl, mode, nullptr, mark_static);
        return;
    }
    cudaGraph_t graph = nullptr;
    EKG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        compute(h, P, ncl, mode, nullptr, mark_static);
    } catch (...) {
        cudaStreamEndCapture(s, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    EKG_CUDA(cudaStreamEndCapture(s, &graph));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    EKG_CUDA(e);
    g->exec = exec;
    g->used = ++h->graph_clock;
    EKG_CUDA(cudaGraphLaunch(exec, s));
}

void assemble_criteria(const ekg_heart *h, const double *crit2, bool done, double approx_crit,
                       const std::vector<double> &approx, double endo_epi, double *out);
TuneChoice tune_pass(ekg_heart *h, int n_sims, const double *layer_k, const double *leads, int reps,
                     double *builtin_ms);

// Queues one device pass from the current staging buffer (h->cur): plan, upload, the pass (a graph
// replay) and the copies of its outputs (ECG to ecg_host; criterion values and the error word to
// the pending slot's pinned buffers).  pend[h->cur].done marks the pass and its copies complete.
// The pass's kernels wait for the previous pass's copies to the host (they overwrite its outputs).
void launch_pass(ekg_heart *h, int n_sims, const double *layer_k, const double *leads, double *ecg_host,
                 int n_crit_leads, int mode) {
    HeartDev &D = h->dev;
    EvalDev &E = h->ev;
    cudaStream_t s = h->stream;
    ekg_heart::Pending &pd = h->pend[h->cur];
    EKG_CUDA(cudaSetDevice(h->eng->device));
    if (!h->copy_stream) {
        EKG_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t *e : {&h->static_done, &h->moved_done, &h->copies_done, &h->pass_end})
            EKG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (!pd.done) {
        EKG_CUDA(cudaEventCreateWithFlags(&pd.done, cudaEventDisableTiming));
        EKG_CUDA(cudaMallocHost(&pd.err, sizeof(uint32_t)));
    }
    const size_t need = (size_t)n_sims * std::max(1, n_crit_leads) * 2;
    if (pd.crit2_cap < need) {
        if (pd.crit2) cudaFreeHost(pd.crit2);
        pd.crit2 = nullptr;
        pd.crit2_cap = 0;
        EKG_CUDA(cudaMallocHost(&pd.crit2, need * sizeof(double)));
        pd.crit2_cap = need;
    }
    if (h->eng->tune && n_sims > 1) {
        // tune a new pass shape on its first pass (the choice is kept for the heart)
        const PassPlan Pt = plan_pass(h, n_sims, layer_k, leads);
        if (Pt.batch && Pt.nmove > 0 && !h->tuned.count(tune_key(h, n_sims, Pt.nmove, Pt.two_bases)))
            tune_pass(h, n_sims, layer_k, leads, 3, nullptr);
    }
    const PassPlan P = plan_pass(h, n_sims, layer_k, leads);
    upload_inputs(h, P, layer_k, leads);
    if (h->copies_pending) EKG_CUDA(cudaStreamWaitEvent(s, h->copies_done, 0));
    const size_t L = D.nleads, S = n_sims, T = D.steps;
    // batched form: the static-lead rows of the ECG are final early, so their copy to the host runs
    // on the copy stream while the moved-lead part is computed
    const bool split = ecg_host && P.batch && P.nmove < (int)L;
    run_pass(h, P, n_crit_leads, mode, split);
    if (split) {
        const size_t nm = P.nmove;
        EKG_CUDA(cudaStreamWaitEvent(h->copy_stream, h->static_done, 0));
        EKG_CUDA(cudaMemcpy2DAsync(ecg_host + nm * T, L * T * 8, E.ecg.p + nm * T, L * T * 8, (L - nm) * T * 8, S,
                                   cudaMemcpyDeviceToHost, h->copy_stream));
    }
    EKG_CUDA(cudaMemcpyAsync(pd.err, E.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (n_crit_leads > 0)
        EKG_CUDA(cudaMemcpyAsync(pd.crit2, E.crit.p, S * n_crit_leads * 2 * 8, cudaMemcpyDeviceToHost, s));
    if (split) {
        if (P.nmove > 0) {
            EKG_CUDA(cudaStreamWaitEvent(h->copy_stream, h->moved_done, 0));
            EKG_CUDA(cudaMemcpy2DAsync(ecg_host, L * T * 8, E.ecg.p, L * T * 8, (size_t)P.nmove * T * 8, S,
                                       cudaMemcpyDeviceToHost, h->copy_stream));
        }
    } else if (ecg_host) {
        EKG_CUDA(cudaMemcpyAsync(ecg_host, E.ecg.p, S * L * T * 8, cudaMemcpyDeviceToHost, s));
    }
    // done = the heart's stream and the copy stream both past this pass
    EKG_CUDA(cudaEventRecord(h->pass_end, s));
    EKG_CUDA(cudaStreamWaitEvent(h->copy_stream, h->pass_end, 0));
    EKG_CUDA(cudaEventRecord(h->copies_done, h->copy_stream));
    EKG_CUDA(cudaEventRecord(pd.done, h->copy_stream));
    h->copies_pending = true;
}

// Hands over a pending batched evaluation: waits for its pass, checks the device error word and
// writes the criteria and violations to the caller's buffers.
void complete_pending(ekg_heart *h, int slot) {
    ekg_heart::Pending &pd = h->pend[slot];
    if (!pd.busy) return;
    pd.busy = false;
    EKG_CUDA(cudaEventSynchronize(pd.done));
    if (*pd.err) throw Error{EKG_ERR_TIMEOUT, "a bounded device wait ran out (error word " + std::to_string(*pd.err) + ")"};
    if (!pd.criteria) return;
    const int nl = h->dev.nlayers, ncl = h->es.n_crit_leads;
    for (int s = 0; s < pd.n_sims; ++s) {
        assemble_criteria(h, &pd.crit2[(size_t)s * ncl * 2], pd.done_flags[s] != 0, pd.acrit[s], pd.approx[s],
                          pd.endo_epi[s], pd.criteria + (size_t)s * h->es.n_criteria);
        pd.violation[s] = pd.viol[s];
    }
    // simulationDone() describes the last single evaluation (sim.cpp:742-745 sets it inside the
    // call); batched evaluations leave it alone
    if (pd.single && pd.n_sims == 1) h->last_simulated = pd.done_flags[0] != 0;
}
void drain_pending(ekg_heart *h) {
    for (int i = 0; i < 2; ++i) complete_pending(h, (h->cur + i) % 2);  // oldest first
}

// One device pass, synchronous (the drop-in simulate call): waits for the evaluations in flight first.
void device_pass(ekg_heart *h, int n_sims, const double *layer_k, const double *leads, double *ecg_host) {
    drain_pending(h);
    const int slot = h->cur;
    launch_pass(h, n_sims, layer_k, leads, ecg_host, 0, 2);
    ekg_heart::Pending &pd = h->pend[slot];
    pd.busy = true;
    pd.criteria = nullptr;
    h->cur ^= 1;
    complete_pending(h, slot);
}

// Device-only timing of `iters` passes with inputs resident (after `warmup` untimed passes).
void benchmark(ekg_heart *h, int n_sims, const double *layer_k, const double *leads, int warmup, int iters,
               double *out, int n_out) {
    std::lock_guard<std::mutex> lk(h->mu);
    drain_pending(h);
    EKG_CUDA(cudaSetDevice(h->eng->device));
    cudaStream_t s = h->stream;
    const PassPlan P = plan_pass(h, n_sims, layer_k, leads);
    upload_inputs(h, P, layer_k, leads);
    const int ncl = h->has_eval ? h->es.n_crit_leads : 0;
    const int mode = h->has_eval ? h->es.comparison_mode : 2;
    // the passes as an evaluation runs them (graph replays, see run_pass); the second warm-up pass
    // captures the graph
    for (int i = 0; i < std::max(warmup, 2); ++i) run_pass(h, P, ncl, mode, false);
    PassTiming tm;
    tm.on = true;
    for (auto &e : tm.ev) EKG_CUDA(cudaEventCreate(&e));
    cudaEvent_t t0, t1;
    EKG_CUDA(cudaEventCreate(&t0));
    EKG_CUDA(cudaEventCreate(&t1));
    EKG_CUDA(cudaStreamSynchronize(s));
    // total: `iters` passes back to back on the heart's stream, events around them
    EKG_CUDA(cudaEventRecord(t0, s));
    for (int i = 0; i < iters; ++i) run_pass(h, P, ncl, mode, false);
    EKG_CUDA(cudaEventRecord(t1, s));
    EKG_CUDA(cudaEventSynchronize(t1));
    float total = 0;
    EKG_CUDA(cudaEventElapsedTime(&total, t0, t1));
    // breakdown: as many passes again, launched directly with events between the parts
    double contract = 0, prep = 0, tail = 0, operand = 0;
    const bool op = P.batch && P.nmove > 0;
    for (int i = 0; i < iters; ++i) {
        compute(h, P, ncl, mode, &tm);
        EKG_CUDA(cudaEventSynchronize(tm.ev[3]));
        float a = 0, b = 0, c = 0, d = 0;
        EKG_CUDA(cudaEventElapsedTime(&a, tm.ev[0], tm.ev[1]));
        EKG_CUDA(cudaEventElapsedTime(&b, tm.ev[1], tm.ev[2]));
        EKG_CUDA(cudaEventElapsedTime(&c, tm.ev[2], tm.ev[3]));
        if (op) EKG_CUDA(cudaEventElapsedTime(&d, tm.ev[4], tm.ev[5]));
        prep += a;
        contract += b;
        tail += c;
        operand += d;
    }
    // work per pass of the batched form: tensor flops the band GEMM executes (three BF16 products
    // per K step and basis) and the bytes the moved-lead operand kernel has to move (tile rows in
    // BF16 hi+lo and steady sums written; voxel geometry, AP ranges and times read once)
    double gemm_flops = 0, op_bytes = 0;
    if (op) {
        const HeartDev &D = h->dev;
        const BatchState &B = h->bs;
        const int N = P.tile_rows, nb = P.two_bases ? 2 : 1;
        for (const int4 &it : P.items) gemm_flops += (double)(it.z - it.y) * P.ntiles * 128.0 * N * 32 * 2 * 3 * nb;
        std::vector<int32_t> nent(D.nlayers), esp((size_t)D.nlayers * 8), ls0(D.nlayers);
        EKG_CUDA(cudaMemcpy(nent.data(), B.nent.p, D.nlayers * 4, cudaMemcpyDeviceToHost));
        EKG_CUDA(cudaMemcpy(esp.data(), B.esplit.p, esp.size() * 4, cudaMemcpyDeviceToHost));
        EKG_CUDA(cudaMemcpy(ls0.data(), B.ls0.p, D.nlayers * 4, cudaMemcpyDeviceToHost));
        double p1 = 0;  // stages whose steady sums are written (inside the longest prefix of their layer)
        for (int L = 0; L < D.nlayers; ++L)
            if (nent[L] > 0) p1 += std::max(0, esp[(size_t)L * 8 + nent[L] - 1] - ls0[L]);
        op_bytes = (double)P.rows_used * D.apad * 4 + p1 * P.rows_used * 8 +
                   (double)D.nvox * 16 + (double)(D.nvox - D.n_interior) * 16 + (double)D.apad * 16;
    }
    // bytes the band contraction of the per-simulation form has to move: the moved rows' W' and the
    // activation times per simulation and lead block, the resident field once, and its compact
    // outputs (run limits, steady sums, the band steps' values, counted from the run limits)
    double band_bytes = 0;
    if (!P.batch && band_contraction(h)) {
        const HeartDev &D = h->dev;
        const int nlb = (D.nleads + 15) / 16;
        std::vector<int4> ci((size_t)n_sims * D.nchunks);
        EKG_CUDA(cudaMemcpy(ci.data(), h->ev.cinfo.p, ci.size() * sizeof(int4), cudaMemcpyDeviceToHost));
        double nband = 0;
        for (const int4 &c : ci) nband += std::max(0, c.y - c.x);
        band_bytes = (double)n_sims * ((double)P.nmove * D.apad * 4 + (double)nlb * D.apad * 16 +
                                       (double)D.nchunks * (16 + (double)D.nleads * 8)) +
                     nband * D.nleads * 4 + (double)(D.nleads - P.nmove) * D.apad * 4;
    }
    const double vals[11] = {total, contract, prep, tail, (double)g_launch_count, (double)P.nmove, P.batch ? 1.0 : 0.0,
                             operand, gemm_flops, op_bytes, band_bytes};
    for (int i = 0; i < n_out && i < 11; ++i) out[i] = vals[i];
    for (auto &e : tm.ev) cudaEventDestroy(e);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    EKG_CUDA(cudaMemcpy(h->err_host, h->ev.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (*h->err_host) throw Error{EKG_ERR_TIMEOUT, "a bounded device wait ran out"};
}

// Times every candidate launch shape of the batched form for a pass of n_sims simulations with these
// inputs (CUDA events on the heart's stream, `reps` passes each after one untimed pass), keeps the
// fastest for this pass shape and appends it to the cache file.  out: the choice (with its ms and
// the number of candidates) and the built-in shape's ms.  Passes without moved leads or outside the
// batched form have nothing to tune (candidates = 0).  The caller holds the heart's lock.
TuneChoice tune_pass(ekg_heart *h, int n_sims, const double *layer_k, const double *leads, int reps,
                     double *builtin_ms) {
    drain_pending(h);
    EKG_CUDA(cudaSetDevice(h->eng->device));
    h->tune_force = nullptr;
    const PassPlan P0 = plan_pass(h, n_sims, layer_k, leads);
    TuneChoice best;
    if (builtin_ms) *builtin_ms = 0;
    if (!P0.batch || P0.nmove == 0) return best;
    const std::string key = tune_key(h, n_sims, P0.nmove, P0.two_bases);
    std::vector<TuneChoice> cands = tune_candidates(P0.two_bases, P0.rows_used, n_sims);
    const int ncl = h->has_eval ? h->es.n_crit_leads : 0;
    const int mode = h->has_eval ? h->es.comparison_mode : 2;
    cudaStream_t s = h->stream;
    cudaEvent_t a, b;
    EKG_CUDA(cudaEventCreate(&a));
    EKG_CUDA(cudaEventCreate(&b));
    struct Restore {
        ekg_heart *h;
        cudaEvent_t a, b;
        ~Restore() {
            h->tune_force = nullptr;
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } restore{h, a, b};
    double best_ms = 1e30;
    for (TuneChoice &c : cands) {
        h->tune_force = &c;
        const PassPlan P = plan_pass(h, n_sims, layer_k, leads);
        upload_inputs(h, P, layer_k, leads);
        compute(h, P, ncl, mode, nullptr);
        EKG_CUDA(cudaEventRecord(a, s));
        for (int r = 0; r < reps; ++r) compute(h, P, ncl, mode, nullptr);
        EKG_CUDA(cudaEventRecord(b, s));
        EKG_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        EKG_CUDA(cudaEventElapsedTime(&ms, a, b));
        EKG_CUDA(cudaMemcpy(h->err_host, h->ev.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (*h->err_host) throw Error{EKG_ERR_TIMEOUT, "a bounded device wait ran out (autotuner)"};
        c.ms = ms / reps;
        const int bN = batch_tile_rows(P0.two_bases, P0.rows_used);
        const bool builtin = c.tile_rows == bN && c.op_small == (n_sims <= small_operand_sims() ? 1 : 0) &&
                             c.cta_mult == (bN <= 32 ? 2 : 1) && c.op_bps == 0;
        if (builtin && builtin_ms) *builtin_ms = c.ms;
        if (c.ms < best_ms) {
            best_ms = c.ms;
            best = c;
        }
    }
    best.candidates = (int)cands.size();
    h->tune_last = cands;
    h->tuned[key] = best;
    if (!h->eng->tune_cache.empty()) tune_cache_write(h->eng->tune_cache, key, best);
    return best;
}

// Per-simulation host part of SimImplementation::eval (sim.cpp:443-492): genes -> layer APs and
// lead positions.
void prepare_sim(ekg_heart *h, const double *genes, int n_genes, double *layer_k, double *leads, double *violation,
                 std::vector<LayerFit> &fits) {
    const EvalSettings &es = h->es;
    EKG_CHECK(h->has_eval, EKG_ERR_BAD_INPUT, "evaluation settings not set for this heart");
    const int nw = es.gm.n_free() * (es.gm.interpolation == 2 ? 3 : 2);
    const int nd = es.optimize_points ? 2 * h->dev.nleads : 0;
    if (n_genes < nw + nd) throw Error{EKG_ERR_BAD_INPUT, "Solution does not contain enough values"};
    if (n_genes != nw + nd) {
        std::ostringstream m;
        m << "chromosome size does not agree with the combination of the number of free Wohlfart parameters and "
             "the selected interpolation procedure ("
          << n_genes << " != " << nd << "+" << nw << ")";
        throw Error{EKG_ERR_BAD_INPUT, m.str()};
    }
    for (int i = 0; i < n_genes; ++i)
        EKG_CHECK(std::isfinite(genes[i]), EKG_ERR_BAD_INPUT, "gene values must be finite");
    if (es.optimize_points) {
        // the displacement genes are (u, v) pairs per lead, the layout move_leads takes
        move_leads_framed(h->dev.nleads, h->leads0.data(), h->lead_uv.data(), genes + nw, leads);
    } else {
        std::copy(h->leads0.begin(), h->leads0.end(), leads);
    }
    layer_aps_setup(es.gm, h->dev.nlayers, genes, layer_k, violation, fits);
}

// The fits of a pass, in parallel when there is more than one.
void run_fits(std::vector<LayerFitJob> &jobs) {
    if (jobs.size() <= 1) {
        layer_aps_run_fits(jobs.data(), jobs.size());
        return;
    }
    HostPool::get().run(jobs.size(), [&](size_t b, size_t e) { layer_aps_run_fits(jobs.data() + b, e - b); });
}

// SimImplementation::calculateFitness (sim.cpp:600-702) from the device's per-lead comparison
// values and peak positions, plus the host-side fast approximation and endo-epi terms.
void assemble_criteria(const ekg_heart *h, const double *crit2, bool done, double approx_crit,
                       const std::vector<double> &approx, double endo_epi, double *out) {
    const EvalSettings &es = h->es;
    EKG_CHECK(es.criteria_mode == 1, EKG_ERR_BAD_INPUT, "selected criteria mode is either not implemented yet or invalid");
    const int nm = es.n_crit_leads;
    const int nc = es.n_criteria;
    for (int i = 0; i < nc; ++i) out[i] = 0.0;
    if (es.fast_is_crit) out[nm] = approx_crit;
    for (int i = 0; i < nm; ++i) {
        double value;
        int peak;
        if (done) {
            value = crit2[2 * i];
            peak = (int)crit2[2 * i + 1];
        } else {
            value = approx_crit;
            peak = (int)(std::max_element(approx.begin(), approx.end()) - approx.begin());
        }
        int ci = i;
        if (es.peak) {
            ci = 2 * i;
            out[ci + 1] = std::abs(peak - es.target_peak[i]);
        }
        out[ci] = value;
        if (out[ci] < 0 || !std::isfinite(out[ci]) || !std::isnormal(out[ci])) out[ci] = 2e10;
    }
    if (es.endo_epi_delay >= 0) out[nc - 1] = endo_epi;
}

// the endo-epi criterion (sim.cpp:686-697): squared difference of the first layer's AP, delayed,
// and the last layer's over 1 .. 699 ms
double endo_epi_term(const ekg_heart *h, const double *layer_k) {
    const WohlfartAP endo(layer_k), epi(layer_k + 9 * (h->dev.nlayers - 1));
    double sd = 0.0;
    for (double t = 1.0; t < 700.0; t += 1.0) {
        const double dd = endo(t + h->es.endo_epi_delay) - epi(t);
        sd += dd * dd;
    }
    return sd;
}

// host comparison for the fast approximation (same formulas as the device criteria)
double compare_host(int mode, const std::vector<double> &a, const std::vector<double> &b, double bofs) {
    const size_t len = std::min(a.size(), b.size());
    if (mode == 2) {
        double sa = 0, sb = 0;
        for (size_t i = 0; i < len; ++i) sa += a[i];
        for (size_t i = 0; i < len; ++i) sb += b[i];
        const double inv = 1.0 / (double)len, ma = sa * inv, mb = sb * inv;
        double va = 0, vb = 0, cv = 0;
        for (size_t i = 0; i < len; ++i) {
            va += (a[i] - ma) * (a[i] - ma);
            vb += (b[i] - mb) * (b[i] - mb);
            cv += (a[i] - ma) * (b[i] - mb);
        }
        return 1.0 - (cv / (double)len) / (std::sqrt(va * inv) * std::sqrt(vb * inv));
    } else if (mode == 4) {
        double ab = 0, aa = 0, bb = 0;
        for (size_t i = 0; i < len; ++i) {
            ab += a[i] * b[i];
            aa += a[i] * a[i];
            bb += b[i] * b[i];
        }
        return 1.0 - ab / (std::sqrt(aa) * std::sqrt(bb));
    } else if (mode == 1) {
        double q = 0;
        for (size_t i = 0; i < len; ++i) q += (a[i] - b[i]) * (a[i] - b[i]);
        return std::sqrt(q / (double)len);
    }
    double mn = a[0], mx = a[0];
    for (size_t i = 1; i < a.size(); ++i) {
        if (a[i] < mn) mn = a[i];
        else if (a[i] > mx) mx = a[i];
    }
    const double am = 1.0 / (mx - mn);
    double mean = 0;
    for (size_t i = 0; i < len; ++i) mean += (a[i] * am + bofs) / (b[i] + bofs);
    mean /= (double)len;
    double var = 0;
    for (size_t i = 0; i < len; ++i) {
        const double d = (a[i] * am + bofs) / (b[i] + bofs) - mean;
        var += d * d;
    }
    var /= (double)len;
    return var == 0 ? 1e30 : std::sqrt(var);
}

// fast approximation gate (sim.cpp:712-747; simlib/simulator.cpp:552-559)
bool approx_gate(const ekg_heart *h, const double *layer_k, double &approx_crit, std::vector<double> &approx) {
    const EvalSettings &es = h->es;
    approx_crit = 2;
    if (!(es.fast_is_crit || es.fast_limit < 2)) return true;
    const int nl = h->dev.nlayers;
    const size_t n = (size_t)(h->length / h->dt);
    const WohlfartAP endo(layer_k), epi(layer_k + 9 * (nl - 1));
    approx.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const double t = h->start + i * h->dt;
        approx[i] = endo(t + es.fast_delay) - epi(t);
    }
    approx_crit = compare_host(es.comparison_mode, approx, es.targets[0], es.target_offsets[0]);
    return !(approx_crit > es.fast_limit);
}

// SimImplementation::eval for a batch, asynchronously: the host part (genes -> layer APs and lead
// positions, fits, the fast-approximation gate) and the pass are queued into the current staging
// buffer; the criteria reach the caller's buffers when the evaluation is handed over
// (eval_wait, or when its staging buffer is needed again two submissions later).
int64_t eval_submit(ekg_heart *h, int n_sims, const double *genes, int n_genes, double *criteria, double *violation,
                    double *ecg, double *layer_k_out, double *leads_out, bool single) {
    std::lock_guard<std::mutex> lk(h->mu);
    const int slot = h->cur;
    complete_pending(h, slot);  // the staging buffer's previous evaluation
    ekg_heart::Pending &pd = h->pend[slot];
    const int nl = h->dev.nlayers, L = h->dev.nleads;
    pd.lk_all.assign((size_t)n_sims * nl * 9, 0.0);
    pd.leads_all.assign((size_t)n_sims * L * 3, 0.0);
    pd.viol.assign(n_sims, 0.0);
    pd.done_flags.assign(n_sims, 1);
    pd.acrit.assign(n_sims, 2.0);
    pd.approx.assign(n_sims, {});
    std::vector<LayerFitJob> jobs;
    std::vector<LayerFit> fits;
    for (int s = 0; s < n_sims; ++s) {
        fits.clear();
        prepare_sim(h, genes + (size_t)s * n_genes, n_genes, &pd.lk_all[(size_t)s * nl * 9],
                    &pd.leads_all[(size_t)s * L * 3], &pd.viol[s], fits);
        for (const LayerFit &f : fits) jobs.push_back(LayerFitJob{f, &pd.lk_all[(size_t)s * nl * 9]});
    }
    run_fits(jobs);
    // the fast-approximation gate and the endo-epi criterion: a few thousand FP64 AP values per
    // simulation when enabled, spread over the host pool for larger batches
    const bool gate = h->es.fast_is_crit || h->es.fast_limit < 2, endo = h->es.endo_epi_delay >= 0;
    pd.endo_epi.assign(n_sims, 0.0);
    auto extras = [&](size_t b, size_t e) {
        for (size_t s = b; s < e; ++s) {
            const double *lk = &pd.lk_all[s * nl * 9];
            pd.done_flags[s] = approx_gate(h, lk, pd.acrit[s], pd.approx[s]) ? 1 : 0;
            if (endo) pd.endo_epi[s] = endo_epi_term(h, lk);
        }
    };
    if ((gate || endo) && n_sims >= 8) HostPool::get().run((size_t)n_sims, extras);
    else extras(0, (size_t)n_sims);
    if (layer_k_out) std::copy(pd.lk_all.begin(), pd.lk_all.end(), layer_k_out);
    if (leads_out) std::copy(pd.leads_all.begin(), pd.leads_all.end(), leads_out);
    launch_pass(h, n_sims, pd.lk_all.data(), pd.leads_all.data(), ecg, h->es.n_crit_leads, h->es.comparison_mode);
    pd.busy = true;
    pd.ticket = ++h->next_ticket;
    pd.n_sims = n_sims;
    pd.single = single;
    pd.criteria = criteria;
    pd.violation = violation;
    h->cur ^= 1;
    return pd.ticket;
}

void eval_wait(ekg_heart *h, int64_t ticket) {
    std::lock_guard<std::mutex> lk(h->mu);
    EKG_CHECK(ticket >= 1 && ticket <= h->next_ticket, EKG_ERR_NOT_FOUND, "unknown evaluation ticket");
    for (int i = 0; i < 2; ++i)
        if (h->pend[i].busy && h->pend[i].ticket == ticket) complete_pending(h, i);
}

void eval_many(ekg_heart *h, int n_sims, const double *genes, int n_genes, double *criteria, double *violation,
               double *ecg, double *layer_k_out, double *leads_out, bool single) {
    eval_wait(h, eval_submit(h, n_sims, genes, n_genes, criteria, violation, ecg, layer_k_out, leads_out, single));
}

void set_eval(ekg_heart *h, const ekg_eval_config *c) {
    EKG_CHECK(c, EKG_ERR_BAD_INPUT, "null eval config");
    EKG_CHECK(c->interpolation == 1 || c->interpolation == 2, EKG_ERR_BAD_INPUT,
              "unknown interpolation type (endo-epi or endo-mid-epi)");
    EKG_CHECK(c->n_base_aps >= 2 && c->base_aps && c->k_min && c->k_max, EKG_ERR_BAD_INPUT, "need at least 2 base APs");
    EKG_CHECK(c->comparison_mode >= 1 && c->comparison_mode <= 4, EKG_ERR_BAD_INPUT, "invalid comparison mode");
    EKG_CHECK(c->criteria_mode == 1 || c->criteria_mode == 9, EKG_ERR_BAD_INPUT, "invalid optimization mode");
    EKG_CHECK(c->n_targets >= 1 && c->targets && c->target_len, EKG_ERR_BAD_INPUT, "no targets");
    EvalSettings es;
    es.gm.interpolation = c->interpolation;
    es.gm.mid_position = c->mid_position;
    for (int i = 0; i < c->n_base_aps; ++i) es.gm.base.emplace_back(c->base_aps + 9 * i, c->base_aps + 9 * i + 9);
    es.gm.k_min.assign(c->k_min, c->k_min + 9);
    es.gm.k_max.assign(c->k_max, c->k_max + 9);
    es.gm.free_mask = c->free_k_mask & 0x1ffu;
    es.optimize_points = c->optimize_points != 0;
    es.criteria_mode = c->criteria_mode;
    es.comparison_mode = c->comparison_mode;
    es.peak = c->peak_is_criterion != 0;
    es.fast_is_crit = c->fast_is_criterion != 0;
    es.fast_delay = c->fast_delay;
    es.fast_limit = c->fast_limit;
    es.endo_epi_delay = c->endo_epi_delay;
    size_t off = 0;
    for (int i = 0; i < c->n_targets; ++i) {
        EKG_CHECK(c->target_len[i] >= 1, EKG_ERR_BAD_INPUT, "empty target");
        es.targets.emplace_back(c->targets + off, c->targets + off + c->target_len[i]);
        off += c->target_len[i];
        es.target_offsets.push_back(c->target_offsets ? c->target_offsets[i] : 0.0);
        es.target_peak.push_back((int)(std::max_element(es.targets.back().begin(), es.targets.back().end()) -
                                       es.targets.back().begin()));
    }
    // SimImplementation constructor: number of criteria (sim.cpp:403-429)
    const int base = c->criteria_mode == 1 ? std::min(h->dev.nleads, c->n_targets) : 1;
    es.n_crit_leads = std::min(h->dev.nleads, c->n_targets);
    es.n_criteria = base + (es.peak ? base : 0) + (es.fast_is_crit ? 1 : 0) + (es.endo_epi_delay >= 0 ? 1 : 0);
    es.n_genes = es.gm.n_free() * (es.gm.interpolation == 2 ? 3 : 2) + (es.optimize_points ? 2 * h->dev.nleads : 0);
    if (c->disp_min && c->n_disp_min > 0) es.disp_min_v.assign(c->disp_min, c->disp_min + c->n_disp_min);
    if (c->disp_max && c->n_disp_max > 0) es.disp_max_v.assign(c->disp_max, c->disp_max + c->n_disp_max);
    std::lock_guard<std::mutex> lk(h->mu);
    drain_pending(h);  // evaluations in flight are handed over with the settings they ran with
    // device copies of the targets
    EvalDev &E = h->ev;
    E.targets.alloc(off);
    E.targets_ff.alloc(off);
    E.target_len.alloc(c->n_targets);
    E.target_off.alloc(c->n_targets);
    EKG_CUDA(cudaSetDevice(h->eng->device));
    EKG_CUDA(cudaMemcpy(E.targets.p, c->targets, off * 8, cudaMemcpyHostToDevice));
    {
        // float-float split of the targets for the criteria: hi the nearest float, lo the remainder
        std::vector<float2> ff(off);
        for (size_t i = 0; i < off; ++i) {
            const float hi = (float)c->targets[i];
            ff[i] = make_float2(hi, (float)(c->targets[i] - (double)hi));
        }
        EKG_CUDA(cudaMemcpy(E.targets_ff.p, ff.data(), off * sizeof(float2), cudaMemcpyHostToDevice));
    }
    EKG_CUDA(cudaMemcpy(E.target_len.p, c->target_len, c->n_targets * 8, cudaMemcpyHostToDevice));
    EKG_CUDA(cudaMemcpy(E.target_off.p, es.target_offsets.data(), c->n_targets * 8, cudaMemcpyHostToDevice));
    h->es = es;
    h->has_eval = true;
}

}  // namespace ekg

using namespace ekg;

extern "C" {

const char *ekg_last_error(void) { return g_last_error.c_str(); }

int ekg_engine_create(int device, ekg_engine **out) {
    return guard([&] {
        EKG_CHECK(out, EKG_ERR_BAD_INPUT, "null output pointer");
        int n = 0;
        EKG_CUDA(cudaGetDeviceCount(&n));
        EKG_CHECK(device >= 0 && device < n, EKG_ERR_BAD_INPUT, "no such CUDA device");
        std::unique_ptr<ekg_engine> e(new ekg_engine());
        e->device = device;
        if (const char *v = std::getenv("EKG_CONTRACT"))
            e->contract = std::string(v) == "cuda" ? EKG_CONTRACT_DENSE_CUDA
                          : std::string(v) == "umma" ? EKG_CONTRACT_DENSE_UMMA
                                                     : EKG_CONTRACT_BAND;
        if (const char *v = std::getenv("EKG_CHUNK")) e->chunk_len = std::max(64, std::atoi(v) / 64 * 64);
        if (const char *v = std::getenv("EKG_BATCHED")) e->batched = std::string(v) != "0";
        if (const char *v = std::getenv("EKG_BATCH_CTAS")) e->batch_ctas = std::atoi(v);
        if (const char *v = std::getenv("EKG_GRAPHS")) e->graphs = std::string(v) != "0";
        if (const char *v = std::getenv("EKG_CA_ROUND_CAP")) e->ca_round_cap = std::max(0, std::atoi(v));
        if (const char *v = std::getenv("EKG_CA")) e->ca_mode = std::string(v) == "tiles" ? 1 : 0;
        if (const char *v = std::getenv("EKG_TUNE")) e->tune = std::string(v) == "1";
        if (const char *v = std::getenv("EKG_TUNE_CACHE")) e->tune_cache = v;
        EKG_CUDA(cudaSetDevice(device));
        EKG_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        *out = e.release();
    });
}

int ekg_engine_destroy(ekg_engine *e) {
    return guard([&] {
        if (!e) return;
        cudaSetDevice(e->device);
        if (e->stream) cudaStreamDestroy(e->stream);
        delete e;
    });
}

int ekg_engine_free_bytes(ekg_engine *e, uint64_t *free_bytes) {
    return guard([&] {
        EKG_CHECK(e && free_bytes, EKG_ERR_BAD_INPUT, "null argument");
        size_t f = 0, t = 0;
        EKG_CUDA(cudaSetDevice(e->device));
        EKG_CUDA(cudaMemGetInfo(&f, &t));
        *free_bytes = f;
    });
}

int ekg_heart_create(ekg_engine *e, const ekg_heart_desc *desc, ekg_heart **out) {
    return guard([&] {
        EKG_CHECK(e && desc && out, EKG_ERR_BAD_INPUT, "null argument");
        std::unique_ptr<ekg_heart> h(new ekg_heart());
        h->eng = e;
        heart_setup(h.get(), desc);
        *out = h.release();
    });
}

int ekg_heart_destroy(ekg_heart *h) {
    return guard([&] {
        if (!h) return;
        cudaSetDevice(h->eng->device);
        delete h;
    });
}

int ekg_heart_get_info(ekg_heart *h, ekg_heart_info *info) {
    return guard([&] {
        EKG_CHECK(h && info, EKG_ERR_BAD_INPUT, "null argument");
        info->n_cells = h->ncell;
        info->n_voxels = h->nvox;
        info->n_aps = h->naps;
        info->n_layers = h->dev.nlayers;
        info->n_leads = h->dev.nleads;
        info->steps = h->dev.steps;
        info->ca_rounds = h->ca_rounds;
        info->device_bytes = heart_device_bytes(h);
        info->ca_ms = h->ca_ms;
        info->setup_ms = h->setup_ms;
        info->ca_buckets = h->ca_buckets ? 1 : 0;
    });
}

int ekg_heart_time_axis(ekg_heart *h, double *start, double *length, double *dt) {
    return guard([&] {
        EKG_CHECK(h, EKG_ERR_BAD_INPUT, "null heart");
        if (start) *start = h->start;
        if (length) *length = h->length;
        if (dt) *dt = h->dt;
    });
}

// the activation times per cell on the host, copied from the device when first asked for
void ensure_at_host(ekg_heart *h) {
    if ((int64_t)h->at_host.size() == h->ncell) return;
    h->at_host.resize(h->ncell);
    EKG_CUDA(cudaSetDevice(h->eng->device));
    EKG_CUDA(cudaMemcpyAsync(h->at_host.data(), h->at_cells.p, h->ncell * 8, cudaMemcpyDeviceToHost, h->stream));
    EKG_CUDA(cudaStreamSynchronize(h->stream));
}

int ekg_heart_activation(ekg_heart *h, double *at_out) {
    return guard([&] {
        EKG_CHECK(h && at_out, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_at_host(h);
        std::copy(h->at_host.begin(), h->at_host.end(), at_out);
    });
}

// The reference's AP numbering (first appearance in raster order, simlib/simulator.cpp:570-590),
// derived from the AP groups when first asked for.
void ensure_ap_ref(ekg_heart *h) {
    if (!h->ap_index_ref.empty() || h->ncell == 0) return;
    const int64_t n = h->ncell, na = h->naps;
    std::vector<int64_t> g_of_cell(n, -1);
    for (int64_t g = 0; g < na; ++g)
        for (int64_t i = h->vox_group_start[g]; i < h->vox_group_start[g + 1]; ++i) g_of_cell[h->vox_cell[i]] = g;
    std::vector<int64_t> g2ref(na, -1);
    int64_t next = 0;
    h->ap_index_ref.assign(n, -1);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t g = g_of_cell[i];
        if (g < 0) continue;
        if (g2ref[g] < 0) g2ref[g] = next++;
        h->ap_index_ref[i] = g2ref[g];
    }
}

int ekg_heart_ap_index(ekg_heart *h, int64_t *out) {
    return guard([&] {
        EKG_CHECK(h && out, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_ap_ref(h);
        std::copy(h->ap_index_ref.begin(), h->ap_index_ref.end(), out);
    });
}

int ekg_simulate(ekg_heart *h, const double *layer_k, const double *leads_zyx, double *ecg_out) {
    return guard([&] {
        EKG_CHECK(h && layer_k && ecg_out, EKG_ERR_BAD_INPUT, "null argument");
        for (int i = 0; i < 9 * h->dev.nlayers; ++i)
            EKG_CHECK(std::isfinite(layer_k[i]), EKG_ERR_BAD_INPUT, "AP coefficients must be finite");
        std::lock_guard<std::mutex> lk(h->mu);
        device_pass(h, 1, layer_k, leads_zyx ? leads_zyx : h->leads0.data(), ecg_out);
    });
}

int ekg_heart_set_eval(ekg_heart *h, const ekg_eval_config *cfg) {
    return guard([&] {
        EKG_CHECK(h, EKG_ERR_BAD_INPUT, "null heart");
        set_eval(h, cfg);
    });
}

int ekg_eval_shape(ekg_heart *h, int32_t *n_genes, int32_t *n_criteria) {
    return guard([&] {
        EKG_CHECK(h && h->has_eval, EKG_ERR_BAD_INPUT, "evaluation settings not set for this heart");
        if (n_genes) *n_genes = h->es.n_genes;
        if (n_criteria) *n_criteria = h->es.n_criteria;
    });
}

int ekg_eval_gene_bounds(ekg_heart *h, double *gmin, double *gmax) {
    return guard([&] {
        EKG_CHECK(h && h->has_eval && gmin && gmax, EKG_ERR_BAD_INPUT, "evaluation settings not set for this heart");
        const EvalSettings &es = h->es;
        // SimImplementation::getGeneParams (sim.cpp:523-580)
        const int nf = es.gm.n_free(), nsets = es.gm.interpolation == 2 ? 3 : 2;
        int g = 0;
        for (int i = 0; i < 9; ++i)
            if (es.gm.free_mask & (1u << i)) {
                for (int s = 0; s < nsets; ++s) {
                    gmin[g + s * nf] = es.gm.k_min[i];
                    gmax[g + s * nf] = es.gm.k_max[i];
                }
                ++g;
            }
        int pos = nf * nsets;
        if (es.optimize_points) {
            std::vector<double> dmin = es.disp_min_v, dmax = es.disp_max_v;
            if (dmin.empty()) dmin.push_back(0);
            if (dmax.empty()) dmax.push_back(0);
            for (int i = 0; i < 2 * h->dev.nleads; ++i) {
                gmin[pos + i] = dmin[std::min<size_t>(i, dmin.size() - 1)];
                gmax[pos + i] = dmax[std::min<size_t>(i, dmax.size() - 1)];
            }
        }
    });
}

int ekg_eval(ekg_heart *h, const double *genes, int32_t n_genes, double *criteria_out, double *violation_out,
             double *ecg_out, double *layer_k_out, double *leads_out) {
    return guard([&] {
        EKG_CHECK(h && genes && criteria_out && violation_out, EKG_ERR_BAD_INPUT, "null argument");
        eval_many(h, 1, genes, n_genes, criteria_out, violation_out, ecg_out, layer_k_out, leads_out, true);
    });
}

int ekg_eval_simulated(ekg_heart *h, int32_t *simulated_out) {
    return guard([&] {
        EKG_CHECK(h && simulated_out, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(h->mu);
        *simulated_out = h->last_simulated ? 1 : 0;
    });
}

int ekg_eval_batch(ekg_heart *h, int32_t n_sims, const double *genes, int32_t n_genes, double *criteria_out,
                   double *violation_out, double *ecg_out) {
    return guard([&] {
        EKG_CHECK(h && genes && criteria_out && violation_out && n_sims >= 1, EKG_ERR_BAD_INPUT, "bad argument");
        eval_many(h, n_sims, genes, n_genes, criteria_out, violation_out, ecg_out, nullptr, nullptr, false);
    });
}

int ekg_eval_batch_submit(ekg_heart *h, int32_t n_sims, const double *genes, int32_t n_genes, double *criteria_out,
                          double *violation_out, double *ecg_out, int64_t *ticket_out) {
    return guard([&] {
        EKG_CHECK(h && genes && criteria_out && violation_out && ticket_out && n_sims >= 1, EKG_ERR_BAD_INPUT,
                  "bad argument");
        *ticket_out =
            eval_submit(h, n_sims, genes, n_genes, criteria_out, violation_out, ecg_out, nullptr, nullptr, false);
    });
}

int ekg_eval_batch_wait(ekg_heart *h, int64_t ticket) {
    return guard([&] {
        EKG_CHECK(h, EKG_ERR_BAD_INPUT, "null heart");
        eval_wait(h, ticket);
    });
}

int ekg_host_register(void *ptr, int64_t bytes) {
    return guard([&] {
        EKG_CHECK(ptr && bytes > 0, EKG_ERR_BAD_INPUT, "bad argument");
        EKG_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
    });
}

int ekg_host_unregister(void *ptr) {
    return guard([&] {
        EKG_CHECK(ptr, EKG_ERR_BAD_INPUT, "bad argument");
        EKG_CUDA(cudaHostUnregister(ptr));
    });
}

int ekg_heart_benchmark(ekg_heart *h, int32_t n_sims, const double *layer_k, const double *leads, int32_t warmup,
                        int32_t iters, double *out, int32_t n_out) {
    return guard([&] {
        EKG_CHECK(h && layer_k && out && n_sims >= 1 && iters >= 1 && warmup >= 0, EKG_ERR_BAD_INPUT, "bad argument");
        std::vector<double> lds;
        if (!leads) {
            for (int i = 0; i < n_sims; ++i) lds.insert(lds.end(), h->leads0.begin(), h->leads0.end());
            leads = lds.data();
        }
        benchmark(h, n_sims, layer_k, leads, warmup, iters, out, n_out);
    });
}

int ekg_heart_tune(ekg_heart *h, int32_t n_sims, const double *layer_k, const double *leads, int32_t reps, double *out,
                   int32_t n_out) {
    return guard([&] {
        EKG_CHECK(h && layer_k && out && n_sims >= 1 && reps >= 1, EKG_ERR_BAD_INPUT, "bad argument");
        std::vector<double> lds;
        if (!leads) {
            for (int i = 0; i < n_sims; ++i) lds.insert(lds.end(), h->leads0.begin(), h->leads0.end());
            leads = lds.data();
        }
        std::lock_guard<std::mutex> lk(h->mu);
        double builtin = 0;
        const TuneChoice t = tune_pass(h, n_sims, layer_k, leads, reps, &builtin);
        const double v[7] = {(double)t.tile_rows, (double)t.cta_mult, (double)t.op_small, t.ms, builtin,
                             (double)t.candidates, (double)t.op_bps};
        for (int i = 0; i < n_out && i < 7; ++i) out[i] = v[i];
        // then every candidate: row tile, CTAs per SM, operand form, operand blocks per SM, ms
        for (size_t c = 0; c < h->tune_last.size(); ++c) {
            const TuneChoice &q = h->tune_last[c];
            const double w[5] = {(double)q.tile_rows, (double)q.cta_mult, (double)q.op_small, (double)q.op_bps, q.ms};
            for (int i = 0; i < 5; ++i)
                if (7 + (int)c * 5 + i < n_out) out[7 + c * 5 + i] = w[i];
        }
    });
}

int ekg_tune_candidates(int32_t two_bases, int32_t rows_used, int32_t n_sims, int32_t *shapes_out, int32_t max_shapes,
                        int32_t *n_out) {
    return guard([&] {
        EKG_CHECK(shapes_out && n_out && rows_used >= 1 && n_sims >= 1 && max_shapes >= 0, EKG_ERR_BAD_INPUT,
                  "bad argument");
        const std::vector<TuneChoice> c = tune_candidates(two_bases, rows_used, n_sims);
        *n_out = (int32_t)c.size();
        for (int i = 0; i < (int)c.size() && i < max_shapes; ++i) {
            shapes_out[4 * i] = c[i].tile_rows;
            shapes_out[4 * i + 1] = c[i].cta_mult;
            shapes_out[4 * i + 2] = c[i].op_small;
            shapes_out[4 * i + 3] = c[i].op_bps;
        }
    });
}

int ekg_tune_cache_put(const char *path, const char *key, const int32_t *shape, double ms) {
    return guard([&] {
        EKG_CHECK(path && key && shape && std::strchr(key, ' ') == nullptr && *key, EKG_ERR_BAD_INPUT, "bad argument");
        TuneChoice t;
        t.tile_rows = shape[0];
        t.cta_mult = shape[1];
        t.op_small = shape[2];
        t.op_bps = shape[3];
        t.ms = ms;
        tune_cache_write(path, key, t);
    });
}

int ekg_tune_cache_get(const char *path, const char *key, int32_t *shape_out, double *ms_out) {
    return guard([&] {
        EKG_CHECK(path && key && shape_out, EKG_ERR_BAD_INPUT, "bad argument");
        TuneChoice t;
        if (!tune_cache_read(path, key, t)) throw Error{EKG_ERR_NOT_FOUND, "no autotuner entry for that key"};
        shape_out[0] = t.tile_rows;
        shape_out[1] = t.cta_mult;
        shape_out[2] = t.op_small;
        shape_out[3] = t.op_bps;
        if (ms_out) *ms_out = t.ms;
    });
}

double ekg_ap_value(const double *k9, double at, double t) {
    if (!k9) return NAN;
    double k[9];
    std::copy(k9, k9 + 9, k);
    k[8] -= at;
    return wohlfart(k, t - at);
}

int ekg_heart_cell_ap(ekg_heart *h, int64_t index, int32_t *layer_out, double *at_out) {
    return guard([&] {
        EKG_CHECK(h && layer_out && at_out, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_ap_ref(h);
        ensure_at_host(h);
        for (int64_t i = 0; i < h->ncell; ++i)
            if (h->ap_index_ref[i] == index) {
                *layer_out = h->layer_host[i];
                *at_out = h->at_host[i];
                return;
            }
        throw Error{EKG_ERR_NOT_FOUND, "no cell AP with that index"};
    });
}

int ekg_move_leads(int32_t n, const double *orig, const double *disp, double *out) {
    return guard([&] {
        EKG_CHECK(n >= 0 && orig && out, EKG_ERR_BAD_INPUT, "null argument");
        move_leads(n, orig, disp, out);
    });
}

int ekg_layer_aps(const ekg_eval_config *c, int32_t n_layers, const double *genes, double *layer_k_out,
                  double *violation_out) {
    return guard([&] {
        EKG_CHECK(c && genes && layer_k_out && violation_out && n_layers >= 1, EKG_ERR_BAD_INPUT, "bad argument");
        EKG_CHECK(c->n_base_aps >= 2 && c->base_aps && c->k_min && c->k_max, EKG_ERR_BAD_INPUT, "need at least 2 base APs");
        GeneModel gm;
        gm.interpolation = c->interpolation;
        gm.mid_position = c->mid_position;
        for (int i = 0; i < c->n_base_aps; ++i) gm.base.emplace_back(c->base_aps + 9 * i, c->base_aps + 9 * i + 9);
        gm.k_min.assign(c->k_min, c->k_min + 9);
        gm.k_max.assign(c->k_max, c->k_max + 9);
        gm.free_mask = c->free_k_mask & 0x1ffu;
        std::vector<LayerFit> fits;
        layer_aps_setup(gm, n_layers, genes, layer_k_out, violation_out, fits);
        std::vector<LayerFitJob> jobs;
        for (const LayerFit &f : fits) jobs.push_back(LayerFitJob{f, layer_k_out});
        run_fits(jobs);
    });
}

int ekg_heart_from_ini(ekg_engine *e, const char *ini_path, const char *out_dir, ekg_heart **out) {
    return guard([&] {
        EKG_CHECK(e && ini_path && out, EKG_ERR_BAD_INPUT, "null argument");
        SimConfig c = load_config(ini_path);
        // SimImplementation constructor order (sim.cpp:368-379): the conduction matrix is loaded
        // before the shape, against the simulator's default of 12 layers (simlib/simulator.cpp:201-206)
        int nt = 0;
        std::vector<double> tm;
        read_transfer(c.transfer, nt, tm);
        if (nt < 12) throw Error{EKG_ERR_TRANSFER, "loaded transfer matrix too small"};
        std::vector<double> pts;
        read_points(c.points, pts);
        int nz, ny, nx;
        std::vector<int32_t> lay;
        read_shape(c.shape, nz, ny, nx, lay);
        // a precomputed sequence instead of the automaton (simlib/sim_lib.h:224-231)
        std::vector<double> at_in;
        if (!c.excitation_in.empty()) read_excitation(c.excitation_in, nz, ny, nx, at_in);
        const int nh = nhood_code(c.nhood);
        if (nh < 0) throw Error{EKG_ERR_BAD_INPUT, "\n   unknown neighbourhood (only know of these: 2D4, 3D4, 2D8, 3D8 (cube))"};
        ekg_heart_desc d{};
        d.nz = nz;
        d.ny = ny;
        d.nx = nx;
        d.layers = lay.data();
        d.n_transfer = nt;
        d.transfer = tm.data();
        d.n_leads = (int32_t)(pts.size() / 3);
        d.leads_zyx = pts.data();
        d.nhood = nh;
        d.start = c.start;
        d.length = c.length;
        d.dt = c.dt;
        d.activation_in = at_in.empty() ? nullptr : at_in.data();
        std::unique_ptr<ekg_heart> h(new ekg_heart());
        h->eng = e;
        heart_setup(h.get(), &d);
        if (!c.excitation_out.empty()) {
            // the reference exports right after computing or loading (simlib/simulator.cpp:284-285, :364-366)
            ensure_at_host(h.get());
            write_excitation(c.excitation_out, nz, ny, nx, h->at_host.data());
        }
        if (c.interpolation != "endo-epi" && c.interpolation != "endo-mid-epi")
            throw Error{EKG_ERR_BAD_INPUT, "unknown interpolation type [" + c.interpolation + "]"};
        std::vector<std::vector<double>> targets;
        std::vector<double> offs;
        load_targets(c, c.targets_file, out_dir ? std::string(out_dir) : std::string(), targets, offs);
        std::vector<double> flat, base;
        std::vector<int64_t> tl;
        for (auto &t : targets) {
            flat.insert(flat.end(), t.begin(), t.end());
            tl.push_back((int64_t)t.size());
        }
        for (auto &b : c.base_aps) base.insert(base.end(), b.begin(), b.end());
        std::vector<double> dmin(c.disp_min.begin(), c.disp_min.end()), dmax(c.disp_max.begin(), c.disp_max.end());
        ekg_eval_config ec{};
        ec.interpolation = c.interpolation == "endo-epi" ? 1 : 2;
        ec.mid_position = c.mid_position;
        ec.n_base_aps = (int32_t)c.base_aps.size();
        ec.base_aps = base.data();
        ec.k_min = c.k_min.data();
        ec.k_max = c.k_max.data();
        uint32_t mask = 0;
        for (int k : c.free_k)
            if (k >= 0 && k < 9) mask |= 1u << k;
        ec.free_k_mask = mask;
        ec.optimize_points = c.optimize_points;
        ec.criteria_mode = c.criteria_mode;
        ec.comparison_mode = c.comparison_mode;
        ec.peak_is_criterion = c.peak;
        ec.fast_is_criterion = c.fast_is_crit;
        ec.fast_delay = c.fast_delay;
        ec.fast_limit = c.fast_limit;
        ec.endo_epi_delay = c.endo_epi_delay;
        ec.n_targets = (int32_t)targets.size();
        ec.target_len = tl.data();
        ec.targets = flat.data();
        ec.target_offsets = offs.data();
        ec.n_disp_min = (int32_t)dmin.size();
        ec.disp_min = dmin.data();
        ec.n_disp_max = (int32_t)dmax.size();
        ec.disp_max = dmax.data();
        set_eval(h.get(), &ec);
        h->cfg = c;
        *out = h.release();
    });
}

}  // extern "C"
