// ltp_serve.cpp -- continuous-batching request loop over the pipelined C ABI.
//
// The reference runs one pre-generated batch per epoch, synchronously
// (src/scheduler.cpp:44-59).  This loop admits transactions as they arrive on
// client streams, forms batches on the fly and keeps up to `depth` of them in
// flight through ltp_pipe, so arrivals are admitted while earlier batches
// execute.  Rules:
//  * a batch closes when its oldest transaction has waited deadline_us, when
//    the pending work reaches the slot capacity or the read/write-set budget
//    (12 bytes of key + opword per op), or -- work-conserving -- as soon as no
//    batch is queued on the device;
//  * transactions re-queued after a priority-rule abort go to the head of the
//    next batch and keep their arrival time;
//  * a stream always maps to one admission lane, so its transactions enter
//    batches in submission order.
#include <time.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "../../include/ltpmg_gb300.h"

namespace {

uint64_t now_ns() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

// Ops of admitted transactions live in chunks; a chunk stays alive while any
// of its transactions is pending or in flight.
struct Chunk {
    std::vector<uint64_t> keys;
    std::vector<uint32_t> opw;
};

struct Txn {
    uint64_t tag, arrival;
    uint32_t stream, n_ops, attempts, off;
    std::shared_ptr<Chunk> chunk;
};

struct Lane {
    std::mutex mu;
    std::shared_ptr<Chunk> chunk = std::make_shared<Chunk>();
    std::vector<Txn> txns;
};

struct Slot {
    uint64_t *keys = nullptr;
    uint32_t *opw = nullptr, *txn_first = nullptr;
    uint8_t *commit = nullptr;
    int32_t *vals = nullptr;
    std::vector<Txn> txns;
    uint64_t ticket = 0, seq = 0;
    bool busy = false;
};

// Log-scale latency histogram: 1% wide buckets from 100 ns to ~30 s.
struct Histo {
    static constexpr double kBase = 100.0, kStep = 1.01;
    static constexpr int kN = 2000;
    std::vector<uint64_t> h = std::vector<uint64_t>(kN + 1, 0);
    uint64_t n = 0;
    double sum = 0, mx = 0;
    void add(double ns) {
        int b = ns <= kBase ? 0 : (int)(std::log(ns / kBase) / std::log(kStep)) + 1;
        if (b > kN) b = kN;
        h[b]++;
        n++;
        sum += ns;
        mx = std::max(mx, ns);
    }
    double pct(double p) const {
        if (!n) return 0;
        const uint64_t want = (uint64_t)std::ceil(p * (double)n);
        uint64_t acc = 0;
        for (int b = 0; b <= kN; b++) {
            acc += h[b];
            if (acc >= want) return b == 0 ? kBase : kBase * std::pow(kStep, b);
        }
        return mx;
    }
};

}  // namespace

struct ltp_server {
    ltp_ctx *ctx = nullptr;
    ltp_serve_config cfg;
    ltp_pipe *pipe = nullptr;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::vector<Slot> slots;
    std::deque<Txn> pending, requeued;
    uint64_t pending_ops = 0;
    std::deque<uint32_t> inflight;  // slot indices in submission order
    std::thread dispatcher;
    std::atomic<bool> stop{false};
    std::atomic<int> status{0};
    std::mutex res_mu;
    std::vector<ltp_serve_result> results;
    Histo histo;
    std::atomic<uint64_t> submitted{0};
    uint64_t completed = 0, committed = 0, aborted_attempts = 0, batches = 0, ops = 0;
    uint64_t closed_deadline = 0, closed_budget = 0, closed_idle = 0;
    uint64_t t_start = 0, t_last = 0;
    uint64_t seq = 0;
};

namespace {

void drain_lanes(ltp_server *s) {
    for (auto &lp : s->lanes) {
        std::vector<Txn> got;
        {
            std::lock_guard<std::mutex> g(lp->mu);
            if (lp->txns.empty()) continue;
            got.swap(lp->txns);
            lp->chunk = std::make_shared<Chunk>();
        }
        for (auto &t : got) {
            s->pending_ops += t.n_ops;
            s->pending.push_back(std::move(t));
        }
    }
}

void complete_batch(ltp_server *s, Slot &sl) {
    ltp_stats st;
    const int rc = ltp_pipe_wait(s->pipe, sl.ticket, &st);
    if (rc) {
        s->status = rc;
        return;
    }
    const uint64_t done = now_ns();
    std::vector<ltp_serve_result> out;
    out.reserve(sl.txns.size());
    for (uint32_t i = 0; i < sl.txns.size(); i++) {
        Txn &t = sl.txns[i];
        const bool ok = sl.commit[i] != 0;
        if (!ok && t.attempts + 1 < s->cfg.max_attempts) {
            s->aborted_attempts++;
            t.attempts++;
            s->requeued.push_back(std::move(t));
            continue;
        }
        if (!ok) s->aborted_attempts++;
        ltp_serve_result r;
        memset(&r, 0, sizeof(r));
        r.tag = t.tag;
        r.arrival_ns = t.arrival;
        r.done_ns = done;
        r.batch_seq = sl.seq;
        r.pos = i;
        r.stream = t.stream;
        r.n_ops = t.n_ops;
        r.attempts = t.attempts + 1;
        r.committed = ok ? 1u : 0u;
        memcpy(r.vals, sl.vals + sl.txn_first[i], t.n_ops * sizeof(int32_t));
        s->completed++;
        if (ok) {
            s->committed++;
            s->histo.add((double)(done - t.arrival));
        }
        out.push_back(r);
    }
    s->t_last = done;
    sl.txns.clear();
    sl.busy = false;
    std::lock_guard<std::mutex> g(s->res_mu);
    s->results.insert(s->results.end(), out.begin(), out.end());
}

bool close_batch(ltp_server *s, uint64_t now) {
    if (s->inflight.size() >= s->cfg.depth) return false;
    if (s->pending.empty() && s->requeued.empty()) return false;
    const uint64_t oldest = std::min(s->requeued.empty() ? UINT64_MAX : s->requeued.front().arrival,
                                     s->pending.empty() ? UINT64_MAX : s->pending.front().arrival);
    const uint64_t cap_ops = std::min<uint64_t>(s->cfg.max_ops, s->cfg.budget_bytes / 12);
    const bool deadline = now >= oldest + (uint64_t)s->cfg.deadline_us * 1000ull;
    const bool full = s->pending_ops >= cap_ops || s->pending.size() + s->requeued.size() >= s->cfg.max_txns;
    const bool idle = s->cfg.eager && s->inflight.empty();
    if (!deadline && !full && !idle) return false;
    if (deadline) s->closed_deadline++;
    else if (full) s->closed_budget++;
    else s->closed_idle++;
    // find a free slot
    uint32_t si = 0;
    while (si < s->slots.size() && s->slots[si].busy) si++;
    if (si == s->slots.size()) return false;
    Slot &sl = s->slots[si];
    uint64_t nops = 0;
    uint32_t nt = 0;
    sl.txn_first[0] = 0;
    auto take = [&](std::deque<Txn> &q) {
        while (!q.empty() && nt < s->cfg.max_txns && nops + q.front().n_ops <= cap_ops) {
            Txn &t = q.front();
            memcpy(sl.keys + nops, t.chunk->keys.data() + t.off, t.n_ops * sizeof(uint64_t));
            memcpy(sl.opw + nops, t.chunk->opw.data() + t.off, t.n_ops * sizeof(uint32_t));
            nops += t.n_ops;
            sl.txn_first[++nt] = (uint32_t)nops;
            sl.txns.push_back(std::move(t));
            q.pop_front();
        }
    };
    take(s->requeued);  // aborted transactions first: they keep their arrival time
    const uint64_t before = nops;
    take(s->pending);
    s->pending_ops -= (nops - before);
    if (nt == 0) return false;
    uint64_t ticket = 0;
    const int rc = ltp_pipe_submit(s->pipe, nt, sl.txn_first, 0, nops, sl.keys, sl.opw, nullptr, 0, sl.commit, sl.vals,
                                   &ticket);
    if (rc) {
        s->status = rc;
        return false;
    }
    sl.ticket = ticket;
    sl.seq = s->seq++;
    sl.busy = true;
    s->inflight.push_back(si);
    s->batches++;
    s->ops += nops;
    return true;
}

void dispatch_loop(ltp_server *s) {
    for (;;) {
        drain_lanes(s);
        bool progressed = false;
        while (!s->inflight.empty() && ltp_pipe_poll(s->pipe, s->slots[s->inflight.front()].ticket) == 0) {
            complete_batch(s, s->slots[s->inflight.front()]);
            s->inflight.pop_front();
            progressed = true;
        }
        if (s->status) break;
        if (close_batch(s, now_ns())) progressed = true;
        if (s->stop && s->pending.empty() && s->requeued.empty() && s->inflight.empty()) {
            drain_lanes(s);
            if (s->pending.empty()) break;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(2));
    }
}

}  // namespace

extern "C" {

uint64_t ltp_now_ns(void) { return now_ns(); }

int ltp_serve_open(ltp_ctx *ctx, const ltp_serve_config *cfg, ltp_server **out) {
    if (!ctx || !cfg || !out || cfg->depth < 2 || cfg->max_txns == 0 || cfg->max_ops == 0) return LTP_E_BADARG;
    *out = nullptr;
    ltp_server *s = new ltp_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    if (s->cfg.max_attempts == 0) s->cfg.max_attempts = 1;
    int rc = ltp_pipe_create(ctx, cfg->depth, cfg->max_txns, cfg->max_ops, &s->pipe);
    if (rc) {
        delete s;
        return rc;
    }
    const unsigned n_lanes = 64;
    for (unsigned i = 0; i < n_lanes; i++) s->lanes.emplace_back(new Lane());
    s->slots.resize(cfg->depth);
    for (auto &sl : s->slots) {
        sl.keys = (uint64_t *)ltp_host_alloc(cfg->max_ops * 8);
        sl.opw = (uint32_t *)ltp_host_alloc(cfg->max_ops * 4);
        sl.vals = (int32_t *)ltp_host_alloc(cfg->max_ops * 4);
        sl.txn_first = (uint32_t *)ltp_host_alloc((cfg->max_txns + 1) * 4);
        sl.commit = (uint8_t *)ltp_host_alloc(cfg->max_txns);
        if (!sl.keys || !sl.opw || !sl.vals || !sl.txn_first || !sl.commit) {
            ltp_serve_close(s, nullptr);
            return LTP_E_NOMEM;
        }
    }
    s->t_start = s->t_last = now_ns();
    s->dispatcher = std::thread(dispatch_loop, s);
    *out = s;
    return LTP_OK;
}

int ltp_serve_submit(ltp_server *s, uint32_t stream, uint32_t n_ops, const uint64_t *keys, const uint32_t *opw,
                     uint64_t tag, uint64_t arrival_ns) {
    if (!s || (n_ops && (!keys || !opw))) return LTP_E_BADARG;
    if (n_ops > LTP_SERVE_MAX_OPS || n_ops > s->cfg.max_ops) return LTP_E_CAPACITY;
    if (s->status) return s->status;
    Lane &ln = *s->lanes[stream % s->lanes.size()];
    Txn t;
    t.tag = tag;
    t.arrival = arrival_ns ? arrival_ns : now_ns();
    t.stream = stream;
    t.n_ops = n_ops;
    t.attempts = 0;
    {
        std::lock_guard<std::mutex> g(ln.mu);
        t.off = (uint32_t)ln.chunk->keys.size();
        ln.chunk->keys.insert(ln.chunk->keys.end(), keys, keys + n_ops);
        ln.chunk->opw.insert(ln.chunk->opw.end(), opw, opw + n_ops);
        t.chunk = ln.chunk;
        ln.txns.push_back(std::move(t));
    }
    s->submitted++;
    return LTP_OK;
}

int ltp_serve_poll(ltp_server *s, ltp_serve_result *out, uint32_t max, uint32_t *n) {
    if (!s || !n || (max && !out)) return LTP_E_BADARG;
    std::lock_guard<std::mutex> g(s->res_mu);
    const uint32_t k = (uint32_t)std::min<size_t>(max, s->results.size());
    if (k) memcpy(out, s->results.data(), k * sizeof(ltp_serve_result));
    s->results.erase(s->results.begin(), s->results.begin() + k);
    *n = k;
    return s->status;
}

int ltp_serve_loadgen(ltp_server *s, double rate, double seconds, uint32_t n_streams, uint64_t seed,
                      const uint32_t *txn_first, uint64_t n_pool, const uint64_t *keys, const uint32_t *opw,
                      uint32_t n_threads) {
    if (!s || rate <= 0 || seconds <= 0 || !n_streams || !txn_first || !n_pool || !keys || !opw) return LTP_E_BADARG;
    if (!n_threads) n_threads = 1;
    const uint64_t t0 = now_ns() + 1000000;  // start 1 ms from now
    const uint64_t t_end = t0 + (uint64_t)(seconds * 1e9);
    std::vector<std::thread> th;
    std::atomic<uint64_t> next_pool{0};
    for (uint32_t g = 0; g < n_threads; g++) {
        th.emplace_back([=, &next_pool]() {
            // this thread's share of the streams: s = g, g + n_threads, ...
            const uint32_t my_streams = (n_streams - g + n_threads - 1) / n_threads;
            if (!my_streams) return;
            const double my_rate = rate * (double)my_streams / (double)n_streams;
            std::mt19937_64 rng(seed * 0x9E3779B97F4A7C15ULL + g + 1);
            std::exponential_distribution<double> gap(my_rate / 1e9);
            double t = (double)t0;
            while (true) {
                t += gap(rng);
                const uint64_t at = (uint64_t)t;
                if (at >= t_end || s->status) break;
                while (now_ns() < at) {
                }
                const uint64_t k = next_pool.fetch_add(1) % n_pool;
                const uint32_t st = g + n_threads * (uint32_t)(rng() % my_streams);
                const uint32_t a = txn_first[k], n = txn_first[k + 1] - txn_first[k];
                if (ltp_serve_submit(s, st, n, keys + a, opw + a, k, at)) break;
            }
        });
    }
    for (auto &x : th) x.join();
    return s->status;
}

int ltp_serve_stats_now(ltp_server *s, ltp_serve_stats *st) {
    if (!s || !st) return LTP_E_BADARG;
    memset(st, 0, sizeof(*st));
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->committed = s->committed;
    st->aborted_attempts = s->aborted_attempts;
    st->batches = s->batches;
    st->closed_deadline = s->closed_deadline;
    st->closed_budget = s->closed_budget;
    st->closed_idle = s->closed_idle;
    st->ops = s->ops;
    st->p50_us = s->histo.pct(0.50) / 1e3;
    st->p99_us = s->histo.pct(0.99) / 1e3;
    st->p999_us = s->histo.pct(0.999) / 1e3;
    st->mean_us = s->histo.n ? s->histo.sum / (double)s->histo.n / 1e3 : 0;
    st->max_us = s->histo.mx / 1e3;
    st->elapsed_s = (double)(s->t_last - s->t_start) / 1e9;
    st->committed_per_s = st->elapsed_s > 0 ? (double)s->committed / st->elapsed_s : 0;
    return s->status;
}

int ltp_serve_close(ltp_server *s, ltp_serve_stats *st) {
    if (!s) return LTP_E_BADARG;
    s->stop = true;
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (st) ltp_serve_stats_now(s, st);
    const int status = s->status;
    if (s->pipe) ltp_pipe_free(s->pipe);
    for (auto &sl : s->slots) {
        ltp_host_free(sl.keys);
        ltp_host_free(sl.opw);
        ltp_host_free(sl.vals);
        ltp_host_free(sl.txn_first);
        ltp_host_free(sl.commit);
    }
    delete s;
    return status;
}

}  // extern "C"
