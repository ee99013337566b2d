// serve.cpp -- the scan service of include/blamm_serve.h.
//
// One GPU context per slot (its own CUDA stream and device buffers), one host
// thread per slot.  Slot threads take requests from a FIFO queue as soon as
// they are free and the request's device-memory estimate fits the budget left
// by the requests in flight and the buffers the slots' contexts keep from earlier
// requests (measured after each request); when the queue's head cannot fit and
// nothing is in flight, every slot releases its kept buffers.  A request runs as
// blamm_set_thresholds (when its
// set differs from the slot's) + blamm_set_columns + blamm_scan on its slot.
// Work of different slots overlaps on the device: host<->device copies of one
// request run beside the kernels of another, and a small request's persistent
// scan occupies only the SMs its jobs need.
#include "blamm_serve.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    std::vector<char> bases;
    std::vector<int64_t> runs;
    std::vector<int32_t> cols;
    int set = 0;
    int64_t need = 0;  // device bytes (estimate)
    Clock::time_point t_submit, t_admit, t_done;
    std::vector<blamm_hit> hits;
    int status = BLAMM_OK;
    std::string err;
    bool done = false;
};

struct Slot {
    blamm_ctx *ctx = nullptr;
    int set = -1;
    int64_t held = 0;  // device bytes the context keeps between requests (measured)
    int64_t need = 0;  // estimate of the request in flight on the slot (0: idle)
    std::thread th;
};

}  // namespace

struct blamm_server {
    blamm_server_config cfg{};
    int ncols = 0, p_rows = 0;
    std::vector<float> thr_sets;  // nsets x ncols
    int nsets = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<int64_t, std::shared_ptr<Request>> reqs;
    int64_t next_id = 1;
    int64_t in_flight_bytes = 0;
    int64_t held_bytes = 0;  // sum of the slots' held bytes
    bool release = false;    // the queue's head waits for the slots' kept buffers
    int64_t budget = 0;
    bool stop = false;
    blamm_server_stats st{};
    std::string err;
};

namespace {

int fail(blamm_server *s, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (s) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = buf;
    }
    return code;
}

// Device bytes committed by the slots other than `except` (-1: all): a slot in flight holds
// the larger of its kept buffers and its request's estimate (the request reuses them), an idle
// slot its kept buffers.  The caller holds the server's lock.
int64_t committed(const blamm_server *s, int except)
{
    int64_t c = 0;
    for (size_t k = 0; k < s->slots.size(); ++k)
        if ((int)k != except) c += std::max(s->slots[k].held, s->slots[k].need);
    return c;
}

// Device bytes a request holds while it runs: raw and packed stream, the one-hot entries
// of one scan window (16 B per position, at most 4 Mi positions), run table, candidate
// records (16 B; at least the context's initial 1 Mi, plus the blocks the scan's warps
// reserve), hits, tile plan.
int64_t request_bytes(int64_t n, int64_t nruns, int64_t cols, int p_rows)
{
    const int64_t stream =
        n + (n + 2048) / 32 * 12 + 16 * (std::min<int64_t>(n, int64_t(4) << 20) + 2048) + 8 * nruns;
    const int64_t cand = 16 * std::max<int64_t>(int64_t(1) << 20, n * cols / 1000 + 152 * 16 * 2 * 128);
    const int64_t hits = 16 * std::max<int64_t>(int64_t(1) << 16, n * cols / 2000);
    const int64_t plan = cols * (int64_t)p_rows * 2 * 2 * 2 + (int64_t(1) << 20);
    return stream + cand + hits + plan;
}

void run_request(blamm_server *s, Slot &slot, Request &r)
{
    blamm_ctx *ctx = slot.ctx;
    int rc = BLAMM_OK;
    if (slot.set != r.set) {
        rc = blamm_set_thresholds(ctx, s->thr_sets.data() + (size_t)r.set * s->ncols);
        slot.set = rc == BLAMM_OK ? r.set : -1;
    }
    if (rc == BLAMM_OK) rc = blamm_set_columns(ctx, r.cols.empty() ? nullptr : r.cols.data(), (int)r.cols.size());
    if (rc == BLAMM_OK && !r.bases.empty()) {
        const int64_t cols = r.cols.empty() ? s->ncols : (int64_t)r.cols.size();
        int64_t cap = std::max<int64_t>(1024, (int64_t)r.bases.size() * cols / 4000);
        for (int attempt = 0; attempt < 3; ++attempt) {
            r.hits.resize((size_t)cap);
            int64_t nh = 0;
            rc = blamm_scan(ctx, r.bases.data(), (int64_t)r.bases.size(), r.runs.data(), (int64_t)r.runs.size(),
                            r.hits.data(), cap, &nh);
            if (rc == BLAMM_ERR_OVERFLOW) {
                cap = nh + nh / 8 + 1024;
                continue;
            }
            r.hits.resize(rc == BLAMM_OK ? (size_t)nh : 0);
            break;
        }
    } else {
        r.hits.clear();
    }
    if (rc != BLAMM_OK) {  // a failed request carries no hits
        std::vector<blamm_hit>().swap(r.hits);
        r.status = rc;
        r.err = blamm_last_error(ctx);
    }
}

void slot_loop(blamm_server *s, int k)
{
    Slot &slot = s->slots[(size_t)k];
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (s->stop) return true;
                if (s->release && slot.held > 0) return true;  // give the kept buffers back
                if (s->queue.empty()) return false;
                // first in, first out: the head is admitted when it fits beside what the other
                // slots commit (this slot's kept buffers are reused by it)
                const int64_t need = s->queue.front()->need;
                if (committed(s, k) + std::max(slot.held, need) <= s->budget) return true;
                if (s->in_flight_bytes == 0 && !s->release) {
                    s->release = true;  // nothing runs: the slots release what they keep
                    s->cv_work.notify_all();
                }
                return s->in_flight_bytes == 0 && committed(s, k) == 0;  // every other slot released
            });
            if (s->stop) return;
            if (s->release && slot.held > 0 &&
                (s->queue.empty() || committed(s, k) + std::max(slot.held, s->queue.front()->need) > s->budget)) {
                const int64_t had = slot.held;
                lk.unlock();
                blamm_release_buffers(slot.ctx);
                int64_t now = 0;
                blamm_ctx_call_bytes(slot.ctx, &now);
                lk.lock();
                slot.held = now;
                s->held_bytes += now - had;
                if (s->held_bytes == 0 || s->in_flight_bytes > 0) s->release = false;
                s->cv_work.notify_all();
                continue;
            }
            if (s->queue.empty()) continue;
            s->release = false;
            r = s->queue.front();
            s->queue.pop_front();
            s->in_flight_bytes += r->need;
            slot.need = r->need;
            s->st.peak_committed = std::max(s->st.peak_committed, committed(s, -1));
            r->t_admit = Clock::now();
        }
        s->cv_work.notify_all();  // the next request may fit too
        run_request(s, slot, *r);
        int64_t kept = 0;
        blamm_ctx_call_bytes(slot.ctx, &kept);
        bool over = false;
        {
            // the slot now holds what its context keeps, which may exceed the request's estimate:
            // if the slots' commitments no longer fit, this (now idle) slot gives its buffers back
            std::lock_guard<std::mutex> lk(s->mu);
            s->held_bytes += kept - slot.held;
            slot.held = kept;
            slot.need = 0;
            over = committed(s, -1) > s->budget;
        }
        if (over) {
            blamm_release_buffers(slot.ctx);
            blamm_ctx_call_bytes(slot.ctx, &kept);
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->t_done = Clock::now();
            r->done = true;
            s->in_flight_bytes -= r->need;
            s->held_bytes += kept - slot.held;
            slot.held = kept;
            if (r->status == BLAMM_OK) {
                s->st.completed += 1;
                s->st.bases += (int64_t)r->bases.size();
                s->st.bp_columns += (double)r->bases.size() * (double)(r->cols.empty() ? s->ncols : r->cols.size());
            } else {
                s->st.failed += 1;
                s->err = r->err;
            }
            // the inputs are no longer needed
            std::vector<char>().swap(r->bases);
            std::vector<int64_t>().swap(r->runs);
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" {

int blamm_server_create(const blamm_server_config *cfg, const float *P, int p_rows, int ncols,
                        const int32_t *col_len, const float *thr_sets, int nsets, blamm_server **out)
{
    if (!cfg || !P || !col_len || !thr_sets || !out || nsets <= 0 || ncols <= 0) return BLAMM_ERR_ARG;
    if (cfg->slots < 1 || cfg->slots > 64) return BLAMM_ERR_ARG;
    *out = nullptr;
    auto s = std::make_unique<blamm_server>();
    s->cfg = *cfg;
    s->ncols = ncols;
    s->p_rows = p_rows;
    s->nsets = nsets;
    s->thr_sets.assign(thr_sets, thr_sets + (size_t)nsets * ncols);
    int64_t free_b = 0, total_b = 0;
    int rc = blamm_device_memory(cfg->device, &free_b, &total_b);
    if (rc != BLAMM_OK) return rc;
    s->budget = cfg->hbm_budget > 0 ? cfg->hbm_budget : free_b / 5 * 4;
    s->st.budget = s->budget;
    s->slots.resize((size_t)cfg->slots);
    for (auto &slot : s->slots) {
        rc = blamm_ctx_create(cfg->device, &slot.ctx);
        if (rc == BLAMM_OK) rc = blamm_set_mode(slot.ctx, cfg->mode);
        if (rc == BLAMM_OK) rc = blamm_set_motifs(slot.ctx, P, p_rows, ncols, col_len, thr_sets);
        if (rc != BLAMM_OK) {
            for (auto &o : s->slots)
                if (o.ctx) blamm_ctx_destroy(o.ctx);
            return rc;
        }
        slot.set = 0;
    }
    blamm_server *sp = s.release();
    for (int k = 0; k < cfg->slots; ++k) sp->slots[(size_t)k].th = std::thread(slot_loop, sp, k);
    *out = sp;
    return BLAMM_OK;
}

int blamm_server_submit(blamm_server *s, const char *bases, int64_t n, const int64_t *run_start, int64_t nruns,
                        const int32_t *cols, int ncols_sel, int thr_set, int64_t *id)
{
    if (!s || !id || n < 0 || ncols_sel < 0 || ncols_sel > s->ncols) return BLAMM_ERR_ARG;
    if (thr_set < 0 || thr_set >= s->nsets) return fail(s, BLAMM_ERR_ARG, "no threshold set %d", thr_set);
    if (n > 0 && (!bases || !run_start || nruns <= 0)) return fail(s, BLAMM_ERR_ARG, "null buffer");
    if (ncols_sel > 0 && !cols) return fail(s, BLAMM_ERR_ARG, "null column list");
    auto r = std::make_shared<Request>();
    r->bases.assign(bases, bases + n);
    if (n > 0) r->runs.assign(run_start, run_start + nruns);
    if (ncols_sel > 0) r->cols.assign(cols, cols + ncols_sel);
    r->set = thr_set;
    r->need = request_bytes(n, nruns, ncols_sel > 0 ? ncols_sel : s->ncols, s->p_rows);
    if (r->need > s->budget)
        return fail(s, BLAMM_ERR_NOMEM, "request needs %lld device bytes > budget %lld", (long long)r->need,
                    (long long)s->budget);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->t_submit = Clock::now();
        s->reqs[r->id] = r;
        s->queue.push_back(r);
        s->st.submitted += 1;
        *id = r->id;
    }
    s->cv_work.notify_one();
    return BLAMM_OK;
}

int blamm_server_wait(blamm_server *s, int64_t id, int64_t timeout_ms, int64_t *n_hits, double *latency_ms,
                      double *queue_ms)
{
    if (!s) return BLAMM_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return BLAMM_ERR_ARG;
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return BLAMM_ERR_TIMEOUT;
    }
    if (n_hits) *n_hits = (int64_t)r->hits.size();
    if (latency_ms) *latency_ms = ms_between(r->t_submit, r->t_done);
    if (queue_ms) *queue_ms = ms_between(r->t_submit, r->t_admit);
    if (r->status != BLAMM_OK) s->err = r->err;
    return r->status;
}

int blamm_server_take(blamm_server *s, int64_t id, blamm_hit *hits, int64_t cap, int64_t *n_hits)
{
    if (!s || cap < 0 || (cap > 0 && !hits)) return BLAMM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return BLAMM_ERR_ARG;
    Request &r = *it->second;
    if (!r.done) return BLAMM_ERR_STATE;
    const int64_t nh = (int64_t)r.hits.size();
    if (n_hits) *n_hits = nh;
    if (nh > cap) return BLAMM_ERR_OVERFLOW;
    if (nh > 0) std::memcpy(hits, r.hits.data(), sizeof(blamm_hit) * (size_t)nh);
    s->reqs.erase(it);
    return BLAMM_OK;
}

int blamm_server_stats_get(blamm_server *s, blamm_server_stats *out)
{
    if (!s || !out) return BLAMM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->queued = (int64_t)s->queue.size();
    out->bytes_in_flight = s->in_flight_bytes;
    out->bytes_held = s->held_bytes;
    out->budget = s->budget;
    return BLAMM_OK;
}

const char *blamm_server_last_error(blamm_server *s)
{
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    thread_local std::string copy;
    copy = s->err;
    return copy.c_str();
}

void blamm_server_destroy(blamm_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->queue.clear();  // callers wait for their requests before destroying the server
    }
    s->cv_work.notify_all();
    for (auto &slot : s->slots)
        if (slot.th.joinable()) slot.th.join();
    for (auto &slot : s->slots)
        if (slot.ctx) blamm_ctx_destroy(slot.ctx);
    delete s;
}

}  // extern "C"
