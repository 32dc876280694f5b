// server.cpp -- served form: a request loop with continuous batching over resident hearts.
//
// The reference parallelises only across evaluations: an MPI master keeps per-worker job queues
// and ships one chromosome per message (AMS-DEMO/ParallelFramework.h:109-520).  Here one process
// owns the GPU and every registered heart has its own request queue and dispatcher thread:
//   - a request (heart id + genes) is checked on arrival's dispatch (gene count, finite values;
//     the reference's errors, sim.cpp:458-459 and :835-841) and a malformed one fails alone;
//   - the dispatcher takes up to max_batch of its heart's queued requests (waiting at most
//     max_wait_us for more while nothing of the heart is on the device), checks the batch's device
//     memory against free HBM minus a reserve (halving the batch until it fits, refusing with
//     EKG_ERR_OUT_OF_MEMORY when not even one simulation fits), and queues one batched pass
//     (ekg_eval_batch_submit's path: the host part of the pass runs, its device work is queued);
//   - it then hands over the heart's previous pass, so one pass runs on the device while the next
//     one is prepared and queued behind it: requests that arrive during a pass join the next one.
// Hearts run on their own streams, so passes of different hearts overlap on the device.
#include <algorithm>
#include <chrono>
#include <cmath>

#include "ekg_engine.h"

namespace ekg {
int64_t eval_submit(ekg_heart *h, int n_sims, const double *genes, int n_genes, double *criteria, double *violation,
                    double *ecg, double *layer_k_out, double *leads_out, bool single);
void eval_wait(ekg_heart *h, int64_t ticket);
int64_t eval_bytes_per_sim(const ekg_heart *h);
int64_t eval_bytes_held(const ekg_heart *h);
}  // namespace ekg

using namespace ekg;
using Clock = std::chrono::steady_clock;

namespace {
struct Request {
    uint64_t id;
    std::vector<double> genes;
    Clock::time_point submit;
};
struct Result {
    int status = EKG_OK;
    std::string error;
    std::vector<double> crit, ecg;
    double viol = 0;
    ekg_request_stats stats{};
};
// One batched pass of a heart on the device: its requests and the output buffers it writes.
struct InFlight {
    int64_t ticket = 0;
    int buf = 0;
    std::vector<Request> reqs;
    Clock::time_point start;
};
// Host output buffers of a pass (page-locked, so the copies from the device run asynchronously).
struct OutBuf {
    double *crit = nullptr, *viol = nullptr, *ecg = nullptr;
    size_t cap = 0;
};
}  // namespace

struct ekg_server;
namespace {
struct HeartSlot {
    ekg_server *srv = nullptr;
    int id = 0;
    ekg_heart *h = nullptr;
    std::deque<Request> queue;  // guarded by the server's mutex
    std::condition_variable cv;
    std::thread th;
    OutBuf out[2];
    ~HeartSlot() {
        for (OutBuf &b : out) {
            if (b.crit) cudaFreeHost(b.crit);
            if (b.viol) cudaFreeHost(b.viol);
            if (b.ecg) cudaFreeHost(b.ecg);
        }
    }
};
}  // namespace

struct ekg_server {
    ekg_engine *eng = nullptr;
    ekg_server_opts opts{};
    std::vector<std::unique_ptr<HeartSlot>> hearts;
    std::mutex mu;
    std::condition_variable cv_done;
    std::unordered_map<uint64_t, Result> done;
    uint64_t next_id = 1;
    bool stop = false;
    // test hook: free-memory provider (nullptr = cudaMemGetInfo)
    uint64_t (*free_bytes_fn)(void *) = nullptr;
    void *free_bytes_ctx = nullptr;
};

namespace {

uint64_t free_bytes(ekg_server *s) {
    if (s->free_bytes_fn) return s->free_bytes_fn(s->free_bytes_ctx);
    size_t f = 0, t = 0;
    cudaSetDevice(s->eng->device);
    if (cudaMemGetInfo(&f, &t) != cudaSuccess) return 0;
    return f;
}

// The per-request part of the reference's input checks (sim.cpp:458-459, :835-841): a request
// failing them fails alone instead of failing the pass it would join.
bool request_ok(const ekg_heart *h, const Request &r, std::string &msg) {
    const int want = h->es.n_genes;
    const int n = (int)r.genes.size();
    if (n < want) {
        msg = "Solution does not contain enough values";
        return false;
    }
    if (n != want) {
        msg = "chromosome size does not agree with the combination of the number of free Wohlfart parameters and "
              "the selected interpolation procedure";
        return false;
    }
    for (double g : r.genes)
        if (!std::isfinite(g)) {
            msg = "gene values must be finite";
            return false;
        }
    return true;
}

void ensure_out(HeartSlot &hs, int buf, size_t n, bool ecg) {
    OutBuf &b = hs.out[buf];
    const ekg_heart *h = hs.h;
    if (b.cap >= n && (!ecg || b.ecg)) return;
    const size_t cap = std::max(n, b.cap);
    const size_t nc = (size_t)std::max(1, h->es.n_criteria);
    const size_t ecg_len = (size_t)h->dev.nleads * h->dev.steps;
    if (b.crit) cudaFreeHost(b.crit);
    if (b.viol) cudaFreeHost(b.viol);
    if (b.ecg) cudaFreeHost(b.ecg);
    b = OutBuf{};
    EKG_CUDA(cudaMallocHost(&b.crit, cap * nc * sizeof(double)));
    EKG_CUDA(cudaMallocHost(&b.viol, cap * sizeof(double)));
    if (ecg) EKG_CUDA(cudaMallocHost(&b.ecg, cap * ecg_len * sizeof(double)));
    b.cap = cap;
}

void publish(ekg_server *s, std::vector<Request> &reqs, std::vector<Result> &res, Clock::time_point t_start,
             int batch_size) {
    const auto t_end = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t i = 0; i < reqs.size(); ++i) {
        Result &r = res[i];
        r.stats.queue_ms = std::chrono::duration<double, std::milli>(t_start - reqs[i].submit).count();
        r.stats.total_ms = std::chrono::duration<double, std::milli>(t_end - reqs[i].submit).count();
        r.stats.batch_size = batch_size;
        s->done[reqs[i].id] = std::move(r);
    }
    s->cv_done.notify_all();
}

// Hands over a pass: waits for it and publishes its requests' results (or its error to all of them).
void complete(HeartSlot &hs, InFlight &f) {
    ekg_server *s = hs.srv;
    ekg_heart *h = hs.h;
    const int rc = guard([&] { eval_wait(h, f.ticket); });
    const std::string msg = rc ? std::string(ekg_last_error()) : std::string();
    const size_t n = f.reqs.size();
    const size_t nc = (size_t)h->es.n_criteria;
    const size_t ecg_len = (size_t)h->dev.nleads * h->dev.steps;
    const OutBuf &b = hs.out[f.buf];
    std::vector<Result> res(n);
    for (size_t i = 0; i < n; ++i) {
        Result &r = res[i];
        r.status = rc;
        r.error = msg;
        if (!rc) {
            r.crit.assign(b.crit + i * nc, b.crit + (i + 1) * nc);
            if (b.ecg && !s->opts.no_ecg) r.ecg.assign(b.ecg + i * ecg_len, b.ecg + (i + 1) * ecg_len);
            r.viol = b.viol[i];
        }
    }
    publish(s, f.reqs, res, f.start, (int)n);
    f.reqs.clear();
}

// Queues one pass over `batch` into output buffer `buf`; on a host-side error the requests run one
// at a time so that the error stays with the request that caused it.
bool launch(HeartSlot &hs, std::vector<Request> &batch, int buf, InFlight &f) {
    ekg_heart *h = hs.h;
    ekg_server *s = hs.srv;
    const int n = (int)batch.size();
    const int ng = h->es.n_genes;
    const bool ecg = !s->opts.no_ecg;
    int rc = guard([&] { ensure_out(hs, buf, (size_t)n, ecg); });
    if (rc) {
        std::vector<Result> res(n);
        for (Result &r : res) {
            r.status = rc;
            r.error = ekg_last_error();
        }
        publish(s, batch, res, Clock::now(), n);
        return false;
    }
    std::vector<double> g((size_t)n * ng);
    for (int i = 0; i < n; ++i) std::copy(batch[i].genes.begin(), batch[i].genes.end(), g.begin() + (size_t)i * ng);
    f.start = Clock::now();
    const OutBuf &b = hs.out[buf];
    int64_t ticket = 0;
    rc = guard([&] {
        ticket = eval_submit(h, n, g.data(), ng, b.crit, b.viol, ecg ? b.ecg : nullptr, nullptr, nullptr, false);
    });
    if (rc == EKG_OK) {
        f.ticket = ticket;
        f.buf = buf;
        f.reqs = std::move(batch);
        return true;
    }
    if (n == 1) {
        std::vector<Result> res(1);
        res[0].status = rc;
        res[0].error = ekg_last_error();
        publish(s, batch, res, f.start, 1);
        return false;
    }
    // isolate the failing request(s): synchronous single passes
    for (int i = 0; i < n; ++i) {
        std::vector<Request> one(1, std::move(batch[i]));
        InFlight f1;
        if (launch(hs, one, buf, f1)) complete(hs, f1);
    }
    return false;
}

void dispatcher(HeartSlot *hsp) {
    HeartSlot &hs = *hsp;
    ekg_server *s = hs.srv;
    ekg_heart *h = hs.h;
    cudaSetDevice(s->eng->device);
    InFlight prev;
    bool have_prev = false;
    int buf = 0;
    for (;;) {
        std::vector<Request> batch, deferred;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (!have_prev) hs.cv.wait(lk, [&] { return s->stop || !hs.queue.empty(); });
            if (s->stop && hs.queue.empty() && !have_prev) return;
            if (!hs.queue.empty() && !have_prev && !s->stop) {
                // nothing on the device: give others up to max_wait_us (from the oldest request's
                // arrival) to join this pass
                const auto deadline = hs.queue.front().submit + std::chrono::microseconds(s->opts.max_wait_us);
                while (!s->stop && (int)hs.queue.size() < s->opts.max_batch && Clock::now() < deadline)
                    hs.cv.wait_until(lk, deadline);
            }
            while (!hs.queue.empty() && (int)batch.size() < s->opts.max_batch) {
                batch.push_back(std::move(hs.queue.front()));
                hs.queue.pop_front();
            }
        }
        // malformed requests fail alone
        {
            std::vector<Request> good, bad;
            std::vector<Result> bad_res;
            for (Request &r : batch) {
                std::string msg;
                if (request_ok(h, r, msg)) {
                    good.push_back(std::move(r));
                } else {
                    Result e;
                    e.status = EKG_ERR_BAD_INPUT;
                    e.error = msg;
                    bad_res.push_back(std::move(e));
                    bad.push_back(std::move(r));
                }
            }
            if (!bad.empty()) publish(s, bad, bad_res, Clock::now(), 1);
            batch = std::move(good);
        }
        // admission by free device memory: shrink the batch until its scratch fits
        if (!batch.empty()) {
            const int64_t per_sim = eval_bytes_per_sim(h);
            const int64_t held = eval_bytes_held(h);
            const uint64_t fb = free_bytes(s);
            const int64_t avail = (int64_t)fb + held - (int64_t)s->opts.hbm_reserve_bytes;
            const int n_fit =
                per_sim > 0 ? (int)std::min<int64_t>((int64_t)batch.size(), std::max<int64_t>(0, avail / per_sim))
                            : (int)batch.size();
            if (n_fit < (int)batch.size()) {
                int k = (int)batch.size();
                while (k > 1 && k > n_fit) k /= 2;
                if (n_fit < 1) k = 0;
                deferred.assign(std::make_move_iterator(batch.begin() + k), std::make_move_iterator(batch.end()));
                batch.resize(k);
            }
            if (batch.empty() && !deferred.empty()) {
                // not even one simulation fits: fail the oldest request, keep the rest queued
                std::vector<Request> one(1, std::move(deferred.front()));
                deferred.erase(deferred.begin());
                std::vector<Result> res(1);
                res[0].status = EKG_ERR_OUT_OF_MEMORY;
                res[0].error = "admission refused: not enough free device memory for one simulation";
                publish(s, one, res, Clock::now(), 1);
            }
            if (!deferred.empty()) {
                std::lock_guard<std::mutex> lk(s->mu);
                for (auto it = deferred.rbegin(); it != deferred.rend(); ++it) hs.queue.push_front(std::move(*it));
            }
        }
        InFlight cur;
        bool have_cur = false;
        if (!batch.empty()) {
            // the previous pass may still run: it wrote the other output buffer
            have_cur = launch(hs, batch, buf, cur);
            if (have_cur) buf ^= 1;
        }
        if (have_prev) {
            complete(hs, prev);
            have_prev = false;
        }
        if (have_cur) {
            prev = std::move(cur);
            have_prev = true;
        }
    }
}

}  // namespace

extern "C" {

int ekg_server_create(ekg_engine *e, const ekg_server_opts *opts, ekg_server **out) {
    return guard([&] {
        EKG_CHECK(e && out, EKG_ERR_BAD_INPUT, "null argument");
        std::unique_ptr<ekg_server> s(new ekg_server());
        s->eng = e;
        s->opts.max_batch = 256;
        s->opts.max_wait_us = 200;
        s->opts.hbm_reserve_bytes = 2ull << 30;
        s->opts.no_ecg = 0;
        if (opts) {
            if (opts->max_batch > 0) s->opts.max_batch = opts->max_batch;
            if (opts->max_wait_us >= 0) s->opts.max_wait_us = opts->max_wait_us;
            s->opts.hbm_reserve_bytes = opts->hbm_reserve_bytes;
            s->opts.no_ecg = opts->no_ecg ? 1 : 0;
        }
        *out = s.release();
    });
}

int ekg_server_destroy(ekg_server *s) {
    return guard([&] {
        if (!s) return;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        for (auto &hs : s->hearts) hs->cv.notify_all();
        for (auto &hs : s->hearts)
            if (hs->th.joinable()) hs->th.join();
        delete s;
    });
}

int ekg_server_add_heart(ekg_server *s, ekg_heart *h, int32_t *heart_id) {
    return guard([&] {
        EKG_CHECK(s && h && heart_id, EKG_ERR_BAD_INPUT, "null argument");
        EKG_CHECK(h->has_eval, EKG_ERR_BAD_INPUT, "evaluation settings not set for this heart");
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &hs : s->hearts) EKG_CHECK(hs->h != h, EKG_ERR_BAD_INPUT, "heart already registered");
        std::unique_ptr<HeartSlot> hs(new HeartSlot());
        hs->srv = s;
        hs->h = h;
        hs->id = (int)s->hearts.size();
        hs->th = std::thread(dispatcher, hs.get());
        *heart_id = hs->id;
        s->hearts.push_back(std::move(hs));
    });
}

namespace {
void enqueue(ekg_server *s, int32_t heart_id, const double *genes, int32_t n_genes, uint64_t *request_id,
             Clock::time_point now) {
    EKG_CHECK(heart_id >= 0 && heart_id < (int)s->hearts.size(), EKG_ERR_NOT_FOUND, "unknown heart id");
    Request r;
    r.id = s->next_id++;
    r.genes.assign(genes, genes + n_genes);
    r.submit = now;
    *request_id = r.id;
    s->hearts[heart_id]->queue.push_back(std::move(r));
}
}  // namespace

int ekg_server_submit(ekg_server *s, int32_t heart_id, const double *genes, int32_t n_genes, uint64_t *request_id) {
    return guard([&] {
        EKG_CHECK(s && genes && request_id && n_genes >= 0, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        enqueue(s, heart_id, genes, n_genes, request_id, Clock::now());
        s->hearts[heart_id]->cv.notify_one();
    });
}

int ekg_server_submit_many(ekg_server *s, int32_t n, const int32_t *heart_ids, const double *genes, int32_t n_genes,
                           uint64_t *request_ids) {
    return guard([&] {
        EKG_CHECK(s && heart_ids && genes && request_ids && n >= 0 && n_genes >= 0, EKG_ERR_BAD_INPUT,
                  "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        for (int i = 0; i < n; ++i)
            EKG_CHECK(heart_ids[i] >= 0 && heart_ids[i] < (int)s->hearts.size(), EKG_ERR_NOT_FOUND, "unknown heart id");
        const auto now = Clock::now();
        std::vector<char> touched(s->hearts.size(), 0);
        for (int i = 0; i < n; ++i) {
            enqueue(s, heart_ids[i], genes + (size_t)i * n_genes, n_genes, request_ids + i, now);
            touched[heart_ids[i]] = 1;
        }
        for (size_t k = 0; k < touched.size(); ++k)
            if (touched[k]) s->hearts[k]->cv.notify_one();
    });
}

int ekg_server_set_free_bytes_provider(ekg_server *s, uint64_t (*fn)(void *), void *ctx) {
    return guard([&] {
        EKG_CHECK(s, EKG_ERR_BAD_INPUT, "null server");
        std::lock_guard<std::mutex> lk(s->mu);
        s->free_bytes_fn = fn;
        s->free_bytes_ctx = ctx;
    });
}

int ekg_server_poll(ekg_server *s, uint64_t request_id, int32_t wait_ms, double *criteria_out, double *violation_out,
                    double *ecg_out, ekg_request_stats *stats) {
    int status = EKG_OK;
    int rc = guard([&] {
        EKG_CHECK(s, EKG_ERR_BAD_INPUT, "null server");
        std::unique_lock<std::mutex> lk(s->mu);
        auto ready = [&] { return s->done.count(request_id) > 0; };
        if (!ready() && wait_ms > 0) s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
        if (!ready()) {
            if (request_id == 0 || request_id >= s->next_id) throw Error{EKG_ERR_NOT_FOUND, "unknown request id"};
            status = EKG_ERR_BUSY;
            return;
        }
        Result r = std::move(s->done[request_id]);
        s->done.erase(request_id);
        if (r.status != EKG_OK) throw Error{r.status, r.error};
        EKG_CHECK(!ecg_out || !r.ecg.empty(), EKG_ERR_BAD_INPUT, "the server keeps no ECGs (no_ecg option)");
        if (criteria_out) std::copy(r.crit.begin(), r.crit.end(), criteria_out);
        if (violation_out) *violation_out = r.viol;
        if (ecg_out) std::copy(r.ecg.begin(), r.ecg.end(), ecg_out);
        if (stats) *stats = r.stats;
    });
    if (rc == EKG_OK && status == EKG_ERR_BUSY) {
        set_error("request not finished yet");
        return EKG_ERR_BUSY;
    }
    return rc;
}

int ekg_server_poll_many(ekg_server *s, int32_t n, const uint64_t *request_ids, int32_t wait_ms, int32_t crit_stride,
                         double *criteria_out, double *violation_out, int32_t *status_out, ekg_request_stats *stats) {
    int busy = 0;
    int rc = guard([&] {
        EKG_CHECK(s && request_ids && status_out && n >= 0 && crit_stride >= 0, EKG_ERR_BAD_INPUT, "bad argument");
        std::unique_lock<std::mutex> lk(s->mu);
        for (int i = 0; i < n; ++i)
            EKG_CHECK(request_ids[i] >= 1 && request_ids[i] < s->next_id, EKG_ERR_NOT_FOUND, "unknown request id");
        auto all_ready = [&] {
            for (int i = 0; i < n; ++i)
                if (status_out[i] == EKG_ERR_BUSY && !s->done.count(request_ids[i])) return false;
            return true;
        };
        for (int i = 0; i < n; ++i) status_out[i] = EKG_ERR_BUSY;
        if (wait_ms > 0) s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), all_ready);
        for (int i = 0; i < n; ++i) {
            auto it = s->done.find(request_ids[i]);
            if (it == s->done.end()) {
                ++busy;
                continue;
            }
            Result &r = it->second;
            status_out[i] = r.status;
            if (r.status == EKG_OK) {
                if (criteria_out)
                    std::copy(r.crit.begin(), r.crit.begin() + std::min<size_t>(r.crit.size(), (size_t)crit_stride),
                              criteria_out + (size_t)i * crit_stride);
                if (violation_out) violation_out[i] = r.viol;
            }
            if (stats) stats[i] = r.stats;
            s->done.erase(it);
        }
    });
    if (rc == EKG_OK && busy) {
        set_error("some requests are not finished yet");
        return EKG_ERR_BUSY;
    }
    return rc;
}

}  // extern "C"
