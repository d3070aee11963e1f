// Request server for many forward simulations on one GPU.
//
// Each request is one Earth model with 1..n sources (one simulation per
// source) and a receiver set, for its own grid and step count. A scheduler
// thread admits queued requests while their device footprint fits the
// budget and a slot is free (backfilling past requests that do not fit yet),
// splits a request whose sources do not fit at once into batches of
// simulations, and advances every admitted batch in turns of `chunk_steps`
// steps on its own CUDA stream, so the work of requests that arrive while
// others run overlaps on the device. A batch that has run all its steps
// hands its seismograms back, frees its memory and makes room for the next.
// Handles are created and loaded (model upload, precompute) by a set-up
// thread, so the scheduler keeps launching the running batches meanwhile.
// Latency is measured from submission to the last batch's completion.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sesnt.h"
#include "sesnt_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long long id = 0;
    sesnt_grid_t grid{};
    std::vector<float> model[7];
    int nsrc = 0, nrec = 0;
    std::vector<int> src_elem, src_kind, rec_elem;
    std::vector<float> src_vm, src_comp, src_stf, rec_vm;
    std::vector<unsigned> rec_mask;
    // progress
    int batches_total = 0, batches_done = 0, next_src = 0;
    std::vector<float> seis;  // [nsrc][nrec][3][nt]
    Clock::time_point t_submit, t_start, t_done;
    bool started = false, done = false, failed = false, cancelled = false;
    std::string error;
    long long updates = 0;  // element-local points x steps x simulations
};

struct Batch {
    Request *req;
    int src0, nsim;
    sesnt_t *h = nullptr;
    long long bytes = 0;
    int it = 1;  // next step
    cudaEvent_t ev = nullptr;
    bool in_flight = false;
    bool ready = false;  // handle created and loaded by the set-up thread
};

}  // namespace

struct sesnt_server {
    sesnt_server_config_t cfg{};
    std::mutex mu;
    std::condition_variable cv_done, cv_work;
    std::deque<Request *> queue;
    std::map<long long, std::unique_ptr<Request>> requests;
    std::vector<std::unique_ptr<Batch>> active;
    long long next_id = 1, used_bytes = 0, budget = 0;
    std::atomic<bool> stop{false};
    std::thread worker, setup;
    std::deque<Batch *> setup_queue;
    std::condition_variable cv_setup;
    int device = 0;
    // statistics
    std::vector<double> latencies, queue_waits;
    long long completed = 0, failed = 0, total_updates = 0;
    Clock::time_point t_first{}, t_last{};
    bool any = false;
    double busy_seconds = 0.0;
    std::string err;

    void run();
    void run_setup();
    bool admit_locked();
    void finish_batch(Batch *b);
    void request_settled_locked(Request *r, const Batch *gone);
    void remove_active_locked(const Batch *b);
};

namespace {

long long request_footprint(const sesnt_grid_t &g, int nsim) {
    sesnt_grid_t x = g;
    x.batch = nsim;
    return sesnt_footprint_bytes(&x);
}

}  // namespace

// Admission: walk the queue in arrival order and start the next batch of
// every request whose next batch fits the remaining budget and a free slot.
bool sesnt_server::admit_locked() {
    bool any_started = false;
    for (auto it = queue.begin(); it != queue.end() && (int)active.size() < cfg.max_active;) {
        Request *r = *it;
        if (r->cancelled || r->failed) {
            it = queue.erase(it);
            continue;
        }
        // largest batch of this request's remaining sources that fits
        const int left = r->nsrc - r->next_src;
        int nsim = std::min(left, cfg.max_batch > 0 ? cfg.max_batch : left);
        while (nsim > 0 && used_bytes + request_footprint(r->grid, nsim) > budget) nsim /= 2;
        if (nsim <= 0) {
            ++it;  // does not fit yet; later, smaller requests may (backfill)
            continue;
        }
        std::unique_ptr<Batch> b(new Batch());
        b->req = r;
        b->src0 = r->next_src;
        b->nsim = nsim;
        b->bytes = request_footprint(r->grid, nsim);
        used_bytes += b->bytes;
        if (!r->started) {
            r->started = true;
            r->t_start = Clock::now();
        }
        r->next_src += nsim;
        if (r->next_src >= r->nsrc) it = queue.erase(it);
        setup_queue.push_back(b.get());
        cv_setup.notify_one();
        active.push_back(std::move(b));
        any_started = true;
    }
    return any_started;
}

void sesnt_server::finish_batch(Batch *b) {
    Request *r = b->req;
    const sesnt_grid_t &g = r->grid;
    std::vector<float> seis((size_t)b->nsim * r->nrec * 3 * g.nt);
    int rc = r->nrec ? sesnt_get_seismograms(b->h, seis.data()) : 0;
    if (rc) {
        r->failed = true;
        r->error = sesnt_last_error(b->h);
    } else {
        std::memcpy(r->seis.data() + (size_t)b->src0 * r->nrec * 3 * g.nt, seis.data(), seis.size() * sizeof(float));
    }
    sesnt_destroy(b->h);
    cudaEventDestroy(b->ev);
    b->h = nullptr;
    used_bytes -= b->bytes;
    r->batches_done++;
    request_settled_locked(r, b);
}

void sesnt_server::remove_active_locked(const Batch *b) {
    for (size_t q = 0; q < active.size(); ++q)
        if (active[q].get() == b) {
            active.erase(active.begin() + q);
            return;
        }
}

// A batch of r is gone (finished or failed): r is done when all its sources
// have been handed to batches (or it failed) and none is left.
void sesnt_server::request_settled_locked(Request *r, const Batch *gone) {
    if (r->next_src >= r->nsrc || r->failed) {
        bool pending = false;
        for (auto &x : active)
            if (x.get() != gone && x->req == r) pending = true;
        if (!pending && !r->done) {
            r->done = true;
            r->t_done = Clock::now();
            if (r->failed) {
                ++failed;
            } else {
                ++completed;
                total_updates += r->updates;
                latencies.push_back(std::chrono::duration<double>(r->t_done - r->t_submit).count());
                queue_waits.push_back(std::chrono::duration<double>(r->t_start - r->t_submit).count());
                if (!any || r->t_submit < t_first) t_first = r->t_submit;
                any = true;
                t_last = r->t_done;
            }
            cv_done.notify_all();
        }
    }
}

// Creates and loads the handles of admitted batches, outside the scheduler.
void sesnt_server::run_setup() {
    cudaSetDevice(device);
    for (;;) {
        Batch *b = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_setup.wait(lk, [&] { return stop.load() || !setup_queue.empty(); });
            if (stop.load()) return;
            b = setup_queue.front();
            setup_queue.pop_front();
        }
        Request *r = b->req;
        sesnt_grid_t g = r->grid;
        g.batch = b->nsim;
        sesnt_t *h = nullptr;
        int rc = sesnt_create(&g, &h);
        auto ptr = [&](int q) -> const float * { return r->model[q].empty() ? nullptr : r->model[q].data(); };
        if (!rc) rc = sesnt_set_model(h, ptr(0), ptr(1), ptr(2), ptr(3), ptr(4), ptr(5), ptr(6));
        const int NP = (g.lpd + 1) * (g.lpd + 1) * (g.lpd + 1);
        for (int s = 0; !rc && s < b->nsim; ++s) {
            const int q = b->src0 + s;
            rc = sesnt_add_source(h, s, r->src_elem[3 * q], r->src_elem[3 * q + 1], r->src_elem[3 * q + 2],
                                  &r->src_vm[(size_t)q * NP], r->src_kind[q], &r->src_comp[(size_t)q * 6],
                                  &r->src_stf[(size_t)q * g.nt], g.nt);
        }
        for (int k = 0; !rc && k < r->nrec; ++k) {
            const int idx = sesnt_add_receiver(h, r->rec_elem[3 * k], r->rec_elem[3 * k + 1], r->rec_elem[3 * k + 2],
                                               &r->rec_vm[(size_t)k * NP], r->rec_mask[k]);
            if (idx < 0) rc = idx;
        }
        cudaEvent_t ev = nullptr;
        if (!rc && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) rc = SESNT_ECUDA;
        std::lock_guard<std::mutex> lk(mu);
        if (rc) {
            if (!r->failed) r->error = h ? sesnt_last_error(h) : sesnt_last_error(nullptr);
            r->failed = true;
            if (h) sesnt_destroy(h);
            used_bytes -= b->bytes;
            request_settled_locked(r, b);
            remove_active_locked(b);
        } else {
            b->h = h;
            b->ev = ev;
            b->ready = true;
        }
        cv_work.notify_all();
    }
}

void sesnt_server::run() {
    cudaSetDevice(device);
    auto busy_since = Clock::now();
    bool was_busy = false;
    while (!stop.load()) {
        std::vector<Batch *> finished;
        {
            std::unique_lock<std::mutex> lk(mu);
            admit_locked();
            // launch the next chunk of every idle batch
            for (auto &b : active) {
                if (b->in_flight || !b->ready) continue;
                const int nt = b->req->grid.nt;
                const int n = std::min(cfg.chunk_steps, nt - b->it + 1);
                int rc = sesnt_run(b->h, b->it, n);
                if (!rc) rc = cudaEventRecord(b->ev, (cudaStream_t)sesnt_stream(b->h)) == cudaSuccess ? 0 : SESNT_ECUDA;
                if (rc) {
                    b->req->failed = true;
                    b->req->error = sesnt_last_error(b->h);
                    b->it = nt + 1;
                } else {
                    b->it += n;
                }
                b->in_flight = true;
            }
            if (active.empty() && queue.empty()) {
                if (was_busy) {
                    busy_seconds += std::chrono::duration<double>(Clock::now() - busy_since).count();
                    was_busy = false;
                }
                cv_work.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
            if (!was_busy) {
                busy_since = Clock::now();
                was_busy = true;
            }
        }
        // poll completions outside the lock
        bool progressed = false;
        for (auto &b : active)
            if (b->in_flight && cudaEventQuery(b->ev) == cudaSuccess) {
                b->in_flight = false;
                progressed = true;
                if (b->it > b->req->grid.nt) finished.push_back(b.get());
            }
        if (!finished.empty()) {
            std::lock_guard<std::mutex> lk(mu);
            for (Batch *b : finished) {
                finish_batch(b);
                remove_active_locked(b);
            }
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

extern "C" {

int sesnt_server_create(const sesnt_server_config_t *cfg, sesnt_server_t **out) {
    if (!out) return SESNT_EINVAL;
    *out = nullptr;
    std::unique_ptr<sesnt_server> s(new sesnt_server());
    if (cfg) s->cfg = *cfg;
    if (s->cfg.max_active <= 0) s->cfg.max_active = 16;
    if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 64;
    cudaGetDevice(&s->device);
    if (s->cfg.device_bytes <= 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return SESNT_ECUDA;
        s->budget = (long long)(0.85 * (double)fr);
    } else {
        s->budget = s->cfg.device_bytes;
    }
    sesnt_server *p = s.get();
    s->worker = std::thread([p] { p->run(); });
    s->setup = std::thread([p] { p->run_setup(); });
    *out = s.release();
    return SESNT_OK;
}

int sesnt_server_destroy(sesnt_server_t *s) {
    if (!s) return SESNT_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop.store(true);
    }
    s->cv_work.notify_all();
    s->cv_setup.notify_all();
    if (s->setup.joinable()) s->setup.join();
    if (s->worker.joinable()) s->worker.join();
    // drain: wait for in-flight work, free handles
    for (auto &b : s->active) {
        if (b->h) {
            sesnt_synchronize(b->h);
            sesnt_destroy(b->h);
        }
        if (b->ev) cudaEventDestroy(b->ev);
    }
    s->active.clear();
    delete s;
    return SESNT_OK;
}

int sesnt_server_submit(sesnt_server_t *s, const sesnt_request_t *q, long long *id) {
    if (!s || !q || !id) return SESNT_EINVAL;
    const sesnt_grid_t &g = q->grid;
    sesnt_grid_t one = g;
    one.batch = 1;
    auto reject = [&](int code, const std::string &why) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = why;
        return code;
    };
    if (sesnt_footprint_bytes(&one) < 0) {
        sesnt_t *probe = nullptr;
        sesnt_create(&one, &probe);  // fails at the grid checks and leaves the reason
        if (probe) sesnt_destroy(probe);
        return reject(SESNT_EINVAL, std::string("invalid grid: ") + sesnt_last_error(nullptr));
    }
    if (q->n_sources < 1 || !q->rhoinv || !q->lambda || !q->mu)
        return reject(SESNT_EINVAL, "a request needs a model (rhoinv, lambda, mu) and at least one source");
    if (request_footprint(g, 1) > s->budget)
        return reject(SESNT_ENOMEM, "one simulation of this request needs more device memory than the budget");
    std::unique_ptr<Request> r(new Request());
    r->grid = g;
    r->grid.batch = 1;
    const size_t P = g.lpd + 1, NP = P * P * P, nloc = (size_t)g.nx * g.ny * g.nz * NP;
    const float *m[7] = {q->rhoinv, q->lambda, q->mu, q->a, q->b, q->c, q->q};
    for (int k = 0; k < 7; ++k)
        if (m[k]) r->model[k].assign(m[k], m[k] + nloc);
    r->nsrc = q->n_sources;
    r->nrec = q->n_receivers;
    r->src_elem.assign(q->src_elem, q->src_elem + 3 * r->nsrc);
    r->src_kind.assign(q->src_kind, q->src_kind + r->nsrc);
    r->src_vm.assign(q->src_vanderm, q->src_vanderm + r->nsrc * NP);
    r->src_comp.assign(q->src_comp, q->src_comp + 6 * r->nsrc);
    r->src_stf.assign(q->src_stf, q->src_stf + (size_t)r->nsrc * g.nt);
    if (r->nrec) {
        r->rec_elem.assign(q->rec_elem, q->rec_elem + 3 * r->nrec);
        r->rec_vm.assign(q->rec_vanderm, q->rec_vanderm + r->nrec * NP);
        r->rec_mask.assign(r->nrec, 7u);
        if (q->rec_mask) r->rec_mask.assign(q->rec_mask, q->rec_mask + r->nrec);
    }
    r->seis.assign((size_t)r->nsrc * r->nrec * 3 * g.nt, 0.0f);
    r->updates = (long long)nloc * g.nt * r->nsrc;
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    *id = r->id;
    s->queue.push_back(r.get());
    s->requests[r->id] = std::move(r);
    s->cv_work.notify_all();
    return SESNT_OK;
}

int sesnt_server_wait(sesnt_server_t *s, long long id, double timeout_s) {
    if (!s) return SESNT_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return SESNT_ENOTFOUND;
    Request *r = it->second.get();
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (!r->done) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->done) return SESNT_ETIMEOUT;
    }
    return r->failed ? SESNT_ECUDA : SESNT_OK;
}

int sesnt_server_result(sesnt_server_t *s, long long id, float *seis, double times[2]) {
    if (!s) return SESNT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return SESNT_ENOTFOUND;
    Request *r = it->second.get();
    if (!r->done) return SESNT_ESTATE;
    if (r->failed) {
        s->err = r->error;
        return SESNT_ECUDA;
    }
    if (seis) std::memcpy(seis, r->seis.data(), r->seis.size() * sizeof(float));
    if (times) {
        times[0] = std::chrono::duration<double>(r->t_done - r->t_submit).count();
        times[1] = std::chrono::duration<double>(r->t_start - r->t_submit).count();
    }
    return SESNT_OK;
}

int sesnt_server_release(sesnt_server_t *s, long long id) {
    if (!s) return SESNT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return SESNT_ENOTFOUND;
    if (!it->second->done) return SESNT_ESTATE;
    s->requests.erase(it);
    return SESNT_OK;
}

int sesnt_server_cancel(sesnt_server_t *s, long long id) {
    if (!s) return SESNT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return SESNT_ENOTFOUND;
    Request *r = it->second.get();
    if (r->started) return SESNT_ESTATE;  // running work is not interrupted
    r->cancelled = true;
    r->failed = true;
    r->error = "cancelled";
    r->done = true;
    r->t_done = Clock::now();
    s->cv_done.notify_all();
    return SESNT_OK;
}

int sesnt_server_stats(sesnt_server_t *s, sesnt_server_stats_t *st) {
    if (!s || !st) return SESNT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof *st);
    st->completed = s->completed;
    st->failed = s->failed;
    st->queued = (long long)s->queue.size();
    st->active = (long long)s->active.size();
    st->device_bytes_used = s->used_bytes;
    st->device_bytes_budget = s->budget;
    st->total_updates = s->total_updates;
    std::vector<double> l = s->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5))]; };
        st->latency_p50 = pct(0.50);
        st->latency_p99 = pct(0.99);
        st->latency_max = l.back();
        const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
        st->wall_seconds = span;
        st->updates_per_second = span > 0 ? (double)s->total_updates / span : 0.0;
    }
    std::vector<double> w = s->queue_waits;
    if (!w.empty()) {
        std::sort(w.begin(), w.end());
        st->queue_wait_p50 = w[w.size() / 2];
    }
    return SESNT_OK;
}

const char *sesnt_server_last_error(const sesnt_server_t *s) { return s ? s->err.c_str() : ""; }

}  // extern "C"
