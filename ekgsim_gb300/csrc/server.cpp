// server.cpp -- served form: a request loop with continuous batching over resident hearts.
//
// The reference parallelises only across evaluations: an MPI master keeps per-worker job queues
// and ships one chromosome per message (AMS-DEMO/ParallelFramework.h:109-520).  Here one process
// owns the GPU; requests (heart id + genes) enter a queue, worker threads pick the heart whose
// oldest request waited longest among the hearts not already on the device, gather up to
// max_batch of its queued requests (waiting at most max_wait_us for more to arrive), check the
// batch's device memory against free HBM minus a reserve (halving the batch until it fits), and
// run one batched device pass on that heart's stream.  Hearts run concurrently on their own
// streams, so requests that arrive while one batch is on the device join the next one.
#include <algorithm>
#include <chrono>

#include "ekg_engine.h"

namespace ekg {
void eval_many(ekg_heart *h, int n_sims, const double *genes, int n_genes, double *criteria, double *violation,
               double *ecg, double *layer_k_out, double *leads_out, bool single);
int64_t eval_bytes_per_sim(const ekg_heart *h);
int64_t eval_bytes_held(const ekg_heart *h);
}  // namespace ekg

using namespace ekg;
using Clock = std::chrono::steady_clock;

namespace {
struct Request {
    uint64_t id;
    int heart;
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
}  // namespace

struct ekg_server {
    ekg_engine *eng = nullptr;
    ekg_server_opts opts{};
    std::vector<ekg_heart *> hearts;
    std::vector<char> busy;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::unordered_map<uint64_t, Result> done;
    uint64_t next_id = 1;
    bool stop = false;
    std::vector<std::thread> workers;
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

void worker_loop(ekg_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_work.wait(lk, [&] {
            if (s->stop) return true;
            for (const Request &r : s->queue)
                if (!s->busy[r.heart]) return true;
            return false;
        });
        if (s->stop) return;
        // heart of the oldest waiting request that is not on the device
        int heart = -1;
        Clock::time_point oldest;
        for (const Request &r : s->queue)
            if (!s->busy[r.heart]) {
                heart = r.heart;
                oldest = r.submit;
                break;
            }
        if (heart < 0) continue;
        // give others up to max_wait_us (from the oldest request's arrival) to join the batch
        const auto deadline = oldest + std::chrono::microseconds(s->opts.max_wait_us);
        auto count = [&] {
            int c = 0;
            for (const Request &r : s->queue) c += r.heart == heart;
            return c;
        };
        while (!s->stop && count() < s->opts.max_batch && Clock::now() < deadline)
            s->cv_work.wait_until(lk, deadline);
        if (s->stop) return;
        if (s->busy[heart]) continue;
        std::vector<Request> batch;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int)batch.size() < s->opts.max_batch;) {
            if (it->heart == heart) {
                batch.push_back(std::move(*it));
                it = s->queue.erase(it);
            } else {
                ++it;
            }
        }
        if (batch.empty()) continue;
        s->busy[heart] = 1;
        ekg_heart *h = s->hearts[heart];
        lk.unlock();

        // admission by free device memory: shrink the batch until its scratch fits
        const int64_t per_sim = eval_bytes_per_sim(h);
        const int64_t held = eval_bytes_held(h);
        const uint64_t fb = free_bytes(s);
        const int64_t avail = (int64_t)fb + held - (int64_t)s->opts.hbm_reserve_bytes;
        int n_fit = per_sim > 0 ? (int)std::min<int64_t>((int64_t)batch.size(), avail / per_sim) : (int)batch.size();
        std::vector<Request> deferred;
        if (n_fit < (int)batch.size()) {
            int k = (int)batch.size();
            while (k > 1 && k > n_fit) k /= 2;
            if (n_fit < 1) k = 0;
            deferred.assign(std::make_move_iterator(batch.begin() + k), std::make_move_iterator(batch.end()));
            batch.resize(k);
        }
        std::vector<Result> res(batch.size());
        const auto t_start = Clock::now();
        if (!batch.empty()) {
            bool same = true;
            for (const Request &r : batch) same = same && r.genes.size() == batch[0].genes.size();
            const int nc = h->es.n_criteria;
            const size_t ecg_len = (size_t)h->dev.nleads * h->dev.steps;
            // one device pass over requests [b0, b1), which all have the same gene count
            auto run = [&](size_t b0, size_t b1) {
                const int n = (int)(b1 - b0);
                const int n_genes = (int)batch[b0].genes.size();
                std::vector<double> g((size_t)n * n_genes), crit((size_t)n * nc), viol(n), ecg((size_t)n * ecg_len);
                for (int i = 0; i < n; ++i) std::copy(batch[b0 + i].genes.begin(), batch[b0 + i].genes.end(),
                                                      g.begin() + (size_t)i * n_genes);
                int rc = guard([&] { eval_many(h, n, g.data(), n_genes, crit.data(), viol.data(), ecg.data(),
                                               nullptr, nullptr, false); });
                std::string msg = rc ? std::string(ekg_last_error()) : std::string();
                for (int i = 0; i < n; ++i) {
                    Result &r = res[b0 + i];
                    r.status = rc;
                    r.error = msg;
                    if (!rc) {
                        r.crit.assign(crit.begin() + (size_t)i * nc, crit.begin() + (size_t)(i + 1) * nc);
                        r.ecg.assign(ecg.begin() + (size_t)i * ecg_len, ecg.begin() + (size_t)(i + 1) * ecg_len);
                        r.viol = viol[i];
                    }
                }
                return rc;
            };
            int rc = same ? run(0, batch.size()) : -1;
            if (rc != EKG_OK) {
                // a bad request must not fail the others: run one at a time
                for (size_t i = 0; i < batch.size(); ++i) run(i, i + 1);
            }
        }
        const auto t_end = Clock::now();
        lk.lock();
        for (size_t i = 0; i < batch.size(); ++i) {
            Result &r = res[i];
            r.stats.queue_ms = std::chrono::duration<double, std::milli>(t_start - batch[i].submit).count();
            r.stats.total_ms = std::chrono::duration<double, std::milli>(t_end - batch[i].submit).count();
            r.stats.batch_size = (int)batch.size();
            s->done[batch[i].id] = std::move(r);
        }
        if (batch.empty() && !deferred.empty()) {
            // not even one simulation fits: fail the oldest deferred request, keep the rest queued
            Result r;
            r.status = EKG_ERR_OUT_OF_MEMORY;
            r.error = "admission refused: not enough free device memory for one simulation";
            s->done[deferred.front().id] = std::move(r);
            deferred.erase(deferred.begin());
        }
        for (auto it = deferred.rbegin(); it != deferred.rend(); ++it) s->queue.push_front(std::move(*it));
        s->busy[heart] = 0;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
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
        if (opts) {
            if (opts->max_batch > 0) s->opts.max_batch = opts->max_batch;
            if (opts->max_wait_us >= 0) s->opts.max_wait_us = opts->max_wait_us;
            s->opts.hbm_reserve_bytes = opts->hbm_reserve_bytes;
        }
        const int nworkers = 4;
        for (int i = 0; i < nworkers; ++i) s->workers.emplace_back(worker_loop, s.get());
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
        s->cv_work.notify_all();
        for (std::thread &t : s->workers) t.join();
        delete s;
    });
}

int ekg_server_add_heart(ekg_server *s, ekg_heart *h, int32_t *heart_id) {
    return guard([&] {
        EKG_CHECK(s && h && heart_id, EKG_ERR_BAD_INPUT, "null argument");
        EKG_CHECK(h->has_eval, EKG_ERR_BAD_INPUT, "evaluation settings not set for this heart");
        std::lock_guard<std::mutex> lk(s->mu);
        s->hearts.push_back(h);
        s->busy.push_back(0);
        *heart_id = (int32_t)s->hearts.size() - 1;
    });
}

int ekg_server_submit(ekg_server *s, int32_t heart_id, const double *genes, int32_t n_genes, uint64_t *request_id) {
    return guard([&] {
        EKG_CHECK(s && genes && request_id && n_genes >= 0, EKG_ERR_BAD_INPUT, "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        EKG_CHECK(heart_id >= 0 && heart_id < (int)s->hearts.size(), EKG_ERR_NOT_FOUND, "unknown heart id");
        Request r;
        r.id = s->next_id++;
        r.heart = heart_id;
        r.genes.assign(genes, genes + n_genes);
        r.submit = Clock::now();
        *request_id = r.id;
        s->queue.push_back(std::move(r));
        s->cv_work.notify_all();
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
            bool known = false;
            for (const Request &r : s->queue) known = known || r.id == request_id;
            if (!known && request_id >= s->next_id) throw Error{EKG_ERR_NOT_FOUND, "unknown request id"};
            status = EKG_ERR_BUSY;
            return;
        }
        Result r = std::move(s->done[request_id]);
        s->done.erase(request_id);
        if (r.status != EKG_OK) throw Error{r.status, r.error};
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

}  // extern "C"
