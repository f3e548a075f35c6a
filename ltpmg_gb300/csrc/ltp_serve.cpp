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
//
// Admission is in bulk: a lane accumulates transactions (headers and ops in
// flat arrays) until the dispatcher swaps the whole lane out as a segment;
// batches copy runs of consecutive transactions with one memcpy per run, and
// completion walks runs, so the per-transaction cost is a few nanoseconds.
// Two threads drive the loop: the dispatcher admits and submits, the
// completer waits for finished batches in order, records latencies and hands
// aborted transactions back to the dispatcher.
#include <time.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "../../include/ltpmg_gb300.h"
#include "ltp_histo.h"
#include "ltp_trace.h"

namespace {

uint64_t now_ns() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

inline bool is_insert(uint32_t w) { return (w & 3u) == LTP_OP_INSERT; }

// Transactions of one lane between two drains, in arrival order.  An insert
// op's key is an offset into the segment's payload array.
struct Seg {
    std::vector<uint64_t> arrival, tag;
    std::vector<uint32_t> stream, off, attempts;  // off: first op; txn i's ops are [off[i], off[i+1])
    std::vector<uint64_t> keys;
    std::vector<uint32_t> opw;
    std::vector<uint32_t> poff;  // txn i's payload is [poff[i], poff[i+1])
    std::vector<int32_t> payload;
    size_t head = 0;  // next transaction to batch
    size_t n() const { return arrival.size(); }
    void clear() {
        arrival.clear();
        tag.clear();
        stream.clear();
        off.assign(1, 0);
        poff.assign(1, 0);
        attempts.clear();
        keys.clear();
        opw.clear();
        payload.clear();
        head = 0;
    }
    // key_base: what the caller's insert keys are relative to
    void push(uint64_t arr, uint64_t tg, uint32_t st, uint32_t att, uint32_t n_ops, const uint64_t *k,
              const uint32_t *w, uint32_t n_pay, const int32_t *pay, uint64_t key_base) {
        arrival.push_back(arr);
        tag.push_back(tg);
        stream.push_back(st);
        attempts.push_back(att);
        const size_t k0 = keys.size();
        keys.insert(keys.end(), k, k + n_ops);
        opw.insert(opw.end(), w, w + n_ops);
        off.push_back((uint32_t)keys.size());
        if (n_pay) {
            const uint64_t p0 = payload.size();
            payload.insert(payload.end(), pay, pay + n_pay);
            for (size_t j = k0; j < keys.size(); j++)
                if (is_insert(opw[j])) keys[j] = keys[j] - key_base + p0;
        }
        poff.push_back((uint32_t)payload.size());
    }
};

// Lock for sections of a few dozen nanoseconds (a lane's append or swap):
// waiting threads spin, then yield, instead of sleeping in the kernel.
struct SpinLock {
    std::atomic<bool> f{false};
    void lock() {
        for (unsigned n = 0; f.exchange(true, std::memory_order_acquire);)
            while (f.load(std::memory_order_relaxed))
                if (++n > 64) std::this_thread::yield();
    }
    void unlock() { f.store(false, std::memory_order_release); }
};

// An admission lane.  The dispatcher reads the counters without the lock to
// decide whether a batch is due, and takes the segment only when it closes
// one, so segments hold a batch's worth of a lane's arrivals.
struct alignas(64) Lane {
    SpinLock mu;
    std::shared_ptr<Seg> seg;
    std::atomic<uint64_t> oldest{UINT64_MAX};  // earliest arrival in seg
    std::atomic<uint64_t> n_txns{0}, n_ops{0};  // what seg holds
    std::atomic<uint64_t> submitted{0};         // written under mu only
};

struct Run {  // transactions [first, first+count) of a segment inside a batch
    std::shared_ptr<Seg> seg;
    size_t first, count;
};

// Part of a batch: transactions [i0, i1) of a segment, placed at transaction
// t0, op o0 and payload slot p0 of the slot's arrays.
struct Piece {
    Seg *g;
    size_t i0, i1;
    uint64_t t0, o0, p0;
};

struct Slot {
    uint64_t *keys = nullptr;
    uint32_t *opw = nullptr, *txn_first = nullptr;
    uint8_t *commit = nullptr;
    int32_t *vals = nullptr;
    int64_t *vals64 = nullptr;  // when the context has int64 columns
    int32_t *payload = nullptr;
    std::vector<Run> runs;
    uint64_t ticket = 0, seq = 0;
    std::atomic<bool> busy{false};  // set by the dispatcher, cleared by the completer
};

}  // namespace

struct ltp_server {
    ltp_ctx *ctx = nullptr;
    ltp_serve_config cfg;
    bool keep_results = true;
    bool wide = false;
    uint64_t max_payload = 0;
    ltp_pipe *pipe = nullptr;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::unique_ptr<Slot[]> slots;  // [n_slots]
    uint32_t n_slots = 0;
    std::deque<std::shared_ptr<Seg>> pending;  // requeued segments go to the front
    uint64_t pending_txns = 0, pending_ops = 0;
    // submitted batches, oldest first: the dispatcher appends, the completer
    // takes the front; aborted transactions come back through `requeued`
    std::mutex fl_mu;
    std::condition_variable fl_cv;
    std::deque<uint32_t> inflight;
    std::vector<std::shared_ptr<Seg>> requeued;
    std::atomic<uint32_t> n_inflight{0};
    std::atomic<bool> dispatcher_done{false};
    std::thread dispatcher, completer;
    std::mutex histo_mu;
    std::atomic<bool> stop{false};
    std::atomic<int> status{0};
    std::mutex res_mu;
    std::vector<ltp_serve_result> results;
    ltp::Histo histo;
    std::atomic<bool> started{false};
    std::atomic<uint64_t> completed{0}, committed{0};
    std::atomic<uint64_t> dispatch_ns{0}, complete_ns{0}, lg_total{0}, lg_late{0};
    uint64_t aborted_attempts = 0, batches = 0, ops = 0;
    uint64_t closed_deadline = 0, closed_budget = 0, closed_idle = 0;
    std::atomic<uint64_t> t_first{0};
    uint64_t t_last = 0, seq = 0;
    std::mutex free_mu;
    std::vector<std::shared_ptr<Seg>> free_segs;
    // batch assembly: the dispatcher cuts the batch into pieces and copies
    // them together with the helper threads.  claim = generation << 40 |
    // piece count << 20 | next piece; a helper claims a piece only while the
    // generation it saw is current and pieces remain, so a late helper never
    // reads the list while the dispatcher rebuilds it for the next batch.
    std::vector<Piece> pieces;
    Slot *asm_slot = nullptr;
    std::atomic<uint64_t> claim{0};
    std::atomic<uint64_t> pieces_done{0};
    std::atomic<bool> helpers_stop{false};
    std::mutex asm_mu;
    std::condition_variable asm_cv;  // a new generation was published
    std::vector<std::thread> helpers;
};

namespace {

std::shared_ptr<Seg> new_seg(ltp_server *s) {
    std::lock_guard<std::mutex> g(s->free_mu);
    if (!s->free_segs.empty()) {
        auto p = s->free_segs.back();
        s->free_segs.pop_back();
        return p;
    }
    auto p = std::make_shared<Seg>();
    p->clear();
    return p;
}

void recycle(ltp_server *s, std::shared_ptr<Seg> &p) {
    if (p && p.use_count() == 1) {
        p->clear();
        std::lock_guard<std::mutex> g(s->free_mu);
        if (s->free_segs.size() < 256) s->free_segs.push_back(p);
    }
    p.reset();
}

void drain_lanes(ltp_server *s) {
    for (auto &lp : s->lanes) {
        if (lp->n_txns.load(std::memory_order_relaxed) == 0) continue;
        std::shared_ptr<Seg> got;
        {
            std::lock_guard<SpinLock> g(lp->mu);
            if (!lp->seg || lp->seg->n() == 0) continue;
            got = std::move(lp->seg);
            lp->seg = nullptr;
            lp->oldest.store(UINT64_MAX, std::memory_order_relaxed);
            lp->n_txns.store(0, std::memory_order_relaxed);
            lp->n_ops.store(0, std::memory_order_relaxed);
        }
        s->pending_txns += got->n();
        s->pending_ops += got->keys.size();
        s->pending.push_back(std::move(got));
    }
}

void complete_batch(ltp_server *s, Slot &sl) {
    ltp::TraceRange tr("serve: complete batch");
    ltp_stats st;
    const int rc = ltp_pipe_wait(s->pipe, sl.ticket, &st);
    if (rc) {
        s->status = rc;
        return;
    }
    const uint64_t done = now_ns();
    std::shared_ptr<Seg> again;  // aborted transactions to re-queue
    std::vector<ltp_serve_result> out;
    std::vector<uint64_t> lat;
    lat.reserve(sl.runs.empty() ? 0 : 4096);
    uint32_t pos = 0;
    uint64_t n_ok = 0, n_done = 0;
    for (Run &r : sl.runs) {
        Seg &g = *r.seg;
        for (size_t i = r.first; i < r.first + r.count; i++, pos++) {
            const bool ok = sl.commit[pos] != 0;
            if (!ok && g.attempts[i] + 1 < s->cfg.max_attempts) {
                s->aborted_attempts++;
                if (!again) again = new_seg(s);
                again->push(g.arrival[i], g.tag[i], g.stream[i], g.attempts[i] + 1, g.off[i + 1] - g.off[i],
                            g.keys.data() + g.off[i], g.opw.data() + g.off[i], g.poff[i + 1] - g.poff[i],
                            g.payload.data() + g.poff[i], g.poff[i]);
                continue;
            }
            if (!ok) s->aborted_attempts++;
            n_done++;
            if (ok) {
                n_ok++;
                lat.push_back(done - g.arrival[i]);
            }
            if (s->keep_results) {
                ltp_serve_result res;
                memset(&res, 0, sizeof(res));
                res.tag = g.tag[i];
                res.arrival_ns = g.arrival[i];
                res.done_ns = done;
                res.batch_seq = sl.seq;
                res.pos = pos;
                res.stream = g.stream[i];
                res.n_ops = g.off[i + 1] - g.off[i];
                res.attempts = g.attempts[i] + 1;
                res.committed = ok ? 1u : 0u;
                if (s->wide) {
                    memcpy(res.vals, sl.vals64 + sl.txn_first[pos], res.n_ops * sizeof(int64_t));
                } else {
                    for (uint32_t j = 0; j < res.n_ops; j++) res.vals[j] = sl.vals[sl.txn_first[pos] + j];
                }
                out.push_back(res);
            }
        }
    }
    for (Run &r : sl.runs) recycle(s, r.seg);
    sl.runs.clear();
    if (again) {  // the dispatcher puts them ahead of everything pending
        std::lock_guard<std::mutex> g(s->fl_mu);
        s->requeued.push_back(std::move(again));
    }
    {
        std::lock_guard<std::mutex> g(s->histo_mu);
        for (uint64_t ns : lat) s->histo.add(ns);
    }
    s->completed += n_done;
    s->committed += n_ok;
    s->t_last = done;
    sl.busy.store(false, std::memory_order_release);
    if (!out.empty()) {
        std::lock_guard<std::mutex> g(s->res_mu);
        s->results.insert(s->results.end(), out.begin(), out.end());
    }
}

uint64_t oldest_pending(const ltp_server *s) {
    uint64_t o = UINT64_MAX;
    for (const auto &p : s->pending)
        if (p->head < p->n()) o = std::min(o, p->arrival[p->head]);
    return o;
}

// Copies one piece into the slot: keys, opwords, payload (with insert keys
// rebased onto the batch payload) and the transactions' op offsets.
void copy_piece(Slot &sl, const Piece &pc) {
    const Seg &g = *pc.g;
    const uint32_t a = g.off[pc.i0], b = g.off[pc.i1];
    memcpy(sl.keys + pc.o0, g.keys.data() + a, (size_t)(b - a) * sizeof(uint64_t));
    memcpy(sl.opw + pc.o0, g.opw.data() + a, (size_t)(b - a) * sizeof(uint32_t));
    const uint32_t pa = g.poff[pc.i0], pb = g.poff[pc.i1];
    if (pb > pa) {
        memcpy(sl.payload + pc.p0, g.payload.data() + pa, (size_t)(pb - pa) * sizeof(int32_t));
        const uint64_t delta = pc.p0 - pa;
        for (uint64_t j = pc.o0; j < pc.o0 + (b - a); j++)
            if (is_insert(sl.opw[j])) sl.keys[j] += delta;
    }
    for (size_t i = pc.i0; i < pc.i1; i++) sl.txn_first[pc.t0 + (i - pc.i0) + 1] = (uint32_t)(pc.o0 + g.off[i + 1] - a);
}

constexpr uint64_t kClaimMask = (1u << 20) - 1;
inline uint64_t claim_gen(uint64_t c) { return c >> 40; }

// Copies pieces of the current generation until none is left unclaimed.
void copy_pieces(ltp_server *s, uint64_t gen) {
    for (;;) {
        uint64_t c = s->claim.load(std::memory_order_acquire);
        if (claim_gen(c) != gen) return;
        const uint32_t i = (uint32_t)(c & kClaimMask);
        if (i >= ((c >> 20) & kClaimMask)) return;
        if (!s->claim.compare_exchange_weak(c, c + 1, std::memory_order_acq_rel)) continue;
        copy_piece(*s->asm_slot, s->pieces[i]);
        s->pieces_done.fetch_add(1, std::memory_order_acq_rel);
    }
}

// Sleeps until a batch is published, then helps copy it (the dispatcher
// starts copying at once, so a helper that wakes late only helps less).
void helper_loop(ltp_server *s) {
    uint64_t seen = claim_gen(s->claim.load());
    for (;;) {
        uint64_t gen;
        {
            std::unique_lock<std::mutex> lk(s->asm_mu);
            s->asm_cv.wait(lk, [&] {
                return s->helpers_stop.load() || claim_gen(s->claim.load(std::memory_order_acquire)) != seen;
            });
            if (s->helpers_stop.load()) return;
            gen = claim_gen(s->claim.load(std::memory_order_acquire));
        }
        seen = gen;
        copy_pieces(s, gen);
    }
}

constexpr unsigned kHelpers = 3;          // batch-assembly threads besides the dispatcher
constexpr size_t kPieceTxns = 2048;  // transactions per piece at most
constexpr uint64_t kParallelOps = 16384;  // smaller batches are copied by the dispatcher alone

bool close_batch(ltp_server *s, uint64_t now) {
    if (s->n_inflight.load() >= s->cfg.depth) return false;
    // what is waiting, pending or still in the lanes (read without locking)
    uint64_t oldest = oldest_pending(s), w_txns = s->pending_txns, w_ops = s->pending_ops;
    for (const auto &lp : s->lanes) {
        oldest = std::min(oldest, lp->oldest.load(std::memory_order_relaxed));
        w_txns += lp->n_txns.load(std::memory_order_relaxed);
        w_ops += lp->n_ops.load(std::memory_order_relaxed);
    }
    if (w_txns == 0) return false;
    const uint64_t cap_ops = std::min<uint64_t>(s->cfg.max_ops, s->cfg.budget_bytes / 12);
    const bool deadline = oldest != UINT64_MAX && now >= oldest + (uint64_t)s->cfg.deadline_us * 1000ull;
    const bool full = w_ops >= cap_ops || w_txns >= s->cfg.max_txns;
    const bool idle = (s->cfg.flags & LTP_SERVE_EAGER) && s->n_inflight.load() == 0;
    if (!deadline && !full && !idle) return false;
    uint32_t si = 0;
    while (si < s->n_slots && s->slots[si].busy.load(std::memory_order_acquire)) si++;
    if (si == s->n_slots) return false;
    ltp::TraceRange tr("serve: close batch");
    drain_lanes(s);
    if (s->pending_txns == 0) return false;
    if (deadline) s->closed_deadline++;
    else if (full) s->closed_budget++;
    else s->closed_idle++;
    Slot &sl = s->slots[si];
    uint64_t nops = 0, npay = 0;
    uint32_t nt = 0;
    sl.txn_first[0] = 0;
    s->pieces.clear();
    while (!s->pending.empty() && nt < s->cfg.max_txns) {
        std::shared_ptr<Seg> &p = s->pending.front();
        Seg &g = *p;
        // largest run of this segment that fits (offsets are non-decreasing)
        const size_t h = g.head;
        size_t k = std::min<size_t>(g.n(), h + (s->cfg.max_txns - nt));
        k = (size_t)(std::upper_bound(g.off.begin() + h, g.off.begin() + k + 1, g.off[h] + (cap_ops - nops)) -
                     g.off.begin()) - 1;
        k = (size_t)(std::upper_bound(g.poff.begin() + h, g.poff.begin() + k + 1,
                                      g.poff[h] + (s->max_payload - npay)) - g.poff.begin()) - 1;
        const size_t cnt = k - h;
        if (cnt) {
            for (size_t i0 = h; i0 < k; i0 += kPieceTxns) {
                const size_t i1 = std::min(k, i0 + kPieceTxns);
                s->pieces.push_back(Piece{&g, i0, i1, nt + (i0 - h), nops + (g.off[i0] - g.off[h]),
                                          npay + (g.poff[i0] - g.poff[h])});
            }
            const uint32_t ops = g.off[k] - g.off[h];
            nt += (uint32_t)cnt;
            nops += ops;
            npay += g.poff[k] - g.poff[h];
            sl.runs.push_back(Run{p, h, cnt});
            s->pending_txns -= cnt;
            s->pending_ops -= ops;
            g.head = k;
        }
        if (g.head == g.n()) {
            s->pending.pop_front();
        } else {
            break;  // the batch is full
        }
    }
    if (nops < kParallelOps || s->helpers.empty() || s->pieces.size() > kClaimMask) {
        for (const Piece &pc : s->pieces) copy_piece(sl, pc);
    } else {
        s->asm_slot = &sl;
        s->pieces_done.store(0, std::memory_order_relaxed);
        const uint64_t gen = (claim_gen(s->claim.load()) + 1) & ((1u << 24) - 1);
        {
            std::lock_guard<std::mutex> g(s->asm_mu);
            s->claim.store(gen << 40 | (uint64_t)s->pieces.size() << 20, std::memory_order_release);
        }
        s->asm_cv.notify_all();
        copy_pieces(s, gen);
        while (s->pieces_done.load(std::memory_order_acquire) < s->pieces.size()) {
        }
    }
    if (nt == 0) return false;
    uint64_t ticket = 0;
    const int rc = s->wide ? ltp_pipe_submit64(s->pipe, nt, sl.txn_first, 0, nops, sl.keys, sl.opw, sl.payload, npay,
                                               sl.commit, sl.vals64, &ticket)
                           : ltp_pipe_submit(s->pipe, nt, sl.txn_first, 0, nops, sl.keys, sl.opw, sl.payload, npay,
                                             sl.commit, sl.vals, &ticket);
    if (rc) {
        s->status = rc;
        return false;
    }
    sl.ticket = ticket;
    sl.seq = s->seq++;
    sl.busy.store(true, std::memory_order_release);
    {
        std::lock_guard<std::mutex> g(s->fl_mu);
        s->inflight.push_back(si);
        s->n_inflight++;
    }
    s->fl_cv.notify_one();
    s->batches++;
    s->ops += nops;
    return true;
}

// Puts transactions re-queued by the completer ahead of everything pending.
void take_requeued(ltp_server *s) {
    std::vector<std::shared_ptr<Seg>> got;
    {
        std::lock_guard<std::mutex> g(s->fl_mu);
        got.swap(s->requeued);
    }
    for (auto it = got.rbegin(); it != got.rend(); ++it) {
        s->pending_txns += (*it)->n();
        s->pending_ops += (*it)->keys.size();
        s->pending.push_front(std::move(*it));
    }
}

// Admission and submission; completion runs on its own thread.
void dispatch_loop(ltp_server *s) {
    for (;;) {
        take_requeued(s);
        const uint64_t t0 = now_ns();
        const bool progressed = close_batch(s, t0);
        if (progressed) s->dispatch_ns += now_ns() - t0;
        if (s->status) break;
        if (s->stop && s->pending_txns == 0 && s->n_inflight.load() == 0) {
            drain_lanes(s);
            take_requeued(s);
            if (s->pending_txns == 0 && s->n_inflight.load() == 0) break;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(2));
    }
    s->dispatcher_done = true;
    s->fl_cv.notify_all();
}

// Waits for submitted batches in order and hands their results back.
void complete_loop(ltp_server *s) {
    for (;;) {
        uint32_t si;
        {
            std::unique_lock<std::mutex> lk(s->fl_mu);
            s->fl_cv.wait_for(lk, std::chrono::milliseconds(1),
                              [&] { return !s->inflight.empty() || s->dispatcher_done.load(); });
            if (s->inflight.empty()) {
                if (s->dispatcher_done.load()) break;
                continue;
            }
            si = s->inflight.front();
        }
        while (ltp_pipe_poll(s->pipe, s->slots[si].ticket) == 1) std::this_thread::sleep_for(std::chrono::microseconds(2));
        const uint64_t c0 = now_ns();
        complete_batch(s, s->slots[si]);  // the batch's results are in host memory
        s->complete_ns += now_ns() - c0;
        {
            std::lock_guard<std::mutex> g(s->fl_mu);
            s->inflight.pop_front();
            s->n_inflight--;
        }
        if (s->status) {
            // the dispatcher stops on the status; drop what is still in flight
            std::lock_guard<std::mutex> g(s->fl_mu);
            if (s->dispatcher_done.load() && s->inflight.empty()) break;
        }
    }
}

// Appends a checked transaction to its stream's lane.  key_base: what the
// insert ops' keys are relative to (the start of `payload`).
void admit(ltp_server *s, uint32_t stream, uint64_t at, uint64_t tag, uint32_t n_ops, const uint64_t *keys,
           const uint32_t *opw, uint32_t n_payload, const int32_t *payload, uint64_t key_base) {
    Lane &ln = *s->lanes[stream % s->lanes.size()];
    {
        std::lock_guard<SpinLock> g(ln.mu);
        if (!ln.seg) ln.seg = new_seg(s);
        ln.seg->push(at, tag, stream, 0, n_ops, keys, opw, n_payload, payload, key_base);
        if (at < ln.oldest.load(std::memory_order_relaxed)) ln.oldest.store(at, std::memory_order_relaxed);
        ln.n_txns.store(ln.n_txns.load(std::memory_order_relaxed) + 1, std::memory_order_relaxed);
        ln.n_ops.store(ln.n_ops.load(std::memory_order_relaxed) + n_ops, std::memory_order_relaxed);
        ln.submitted.store(ln.submitted.load(std::memory_order_relaxed) + 1, std::memory_order_relaxed);
    }
    if (!s->started.load(std::memory_order_relaxed) && !s->started.exchange(true)) s->t_first = at;
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
    s->keep_results = (cfg->flags & LTP_SERVE_KEEP_RESULTS) != 0;
    s->wide = ltp_ctx_wide(ctx) != 0;
    s->max_payload = cfg->max_ops * 6;  // int32 slots of insert payload per batch
    if (s->cfg.max_attempts == 0) s->cfg.max_attempts = 1;
    int rc = ltp_pipe_create2(ctx, cfg->depth, cfg->max_txns, cfg->max_ops,
                              (cfg->flags & LTP_SERVE_PERSISTENT) ? LTP_PIPE_PERSISTENT : 0u, &s->pipe);
    if (rc) {
        delete s;
        return rc;
    }
    const unsigned n_lanes = 64;
    for (unsigned i = 0; i < n_lanes; i++) s->lanes.emplace_back(new Lane());
    s->slots.reset(new Slot[cfg->depth]);
    s->n_slots = cfg->depth;
    for (uint32_t i = 0; i < s->n_slots; i++) {
        Slot &sl = s->slots[i];
        sl.keys = (uint64_t *)ltp_host_alloc(cfg->max_ops * 8);
        sl.opw = (uint32_t *)ltp_host_alloc(cfg->max_ops * 4);
        sl.vals = (int32_t *)ltp_host_alloc(cfg->max_ops * 4);
        sl.vals64 = s->wide ? (int64_t *)ltp_host_alloc(cfg->max_ops * 8) : nullptr;
        sl.payload = (int32_t *)ltp_host_alloc(s->max_payload * 4);
        sl.txn_first = (uint32_t *)ltp_host_alloc((cfg->max_txns + 1) * 4);
        sl.commit = (uint8_t *)ltp_host_alloc(cfg->max_txns);
        if (!sl.keys || !sl.opw || !sl.vals || !sl.txn_first || !sl.commit || !sl.payload || (s->wide && !sl.vals64)) {
            ltp_serve_close(s, nullptr);
            return LTP_E_NOMEM;
        }
    }
    s->dispatcher = std::thread(dispatch_loop, s);
    s->completer = std::thread(complete_loop, s);
    for (unsigned i = 0; i < kHelpers; i++) s->helpers.emplace_back(helper_loop, s);
    *out = s;
    return LTP_OK;
}

int ltp_serve_submit_rows(ltp_server *s, uint32_t stream, uint32_t n_ops, const uint64_t *keys, const uint32_t *opw,
                          uint32_t n_payload, const int32_t *payload, uint64_t tag, uint64_t arrival_ns) {
    if (!s || (n_ops && (!keys || !opw)) || (n_payload && !payload)) return LTP_E_BADARG;
    if (n_ops > LTP_SERVE_MAX_OPS || n_ops > s->cfg.max_ops || n_payload > s->max_payload) return LTP_E_CAPACITY;
    for (uint32_t j = 0; j < n_ops; j++)  // an insert's payload row must start inside this transaction's payload
        if (is_insert(opw[j]) && keys[j] >= n_payload) return LTP_E_BADARG;
    if (s->status) return s->status;
    admit(s, stream, arrival_ns ? arrival_ns : now_ns(), tag, n_ops, keys, opw, n_payload, payload, 0);
    return LTP_OK;
}

int ltp_serve_submit(ltp_server *s, uint32_t stream, uint32_t n_ops, const uint64_t *keys, const uint32_t *opw,
                     uint64_t tag, uint64_t arrival_ns) {
    return ltp_serve_submit_rows(s, stream, n_ops, keys, opw, 0, nullptr, tag, arrival_ns);
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
    return ltp_serve_loadgen_rows(s, rate, seconds, n_streams, seed, txn_first, n_pool, keys, opw, nullptr, nullptr,
                                  n_threads);
}

int ltp_serve_loadgen_rows(ltp_server *s, double rate, double seconds, uint32_t n_streams, uint64_t seed,
                           const uint32_t *txn_first, uint64_t n_pool, const uint64_t *keys, const uint32_t *opw,
                           const uint64_t *pay_first, const int32_t *payload, uint32_t n_threads) {
    if (!s || rate <= 0 || seconds <= 0 || !n_streams || !txn_first || !n_pool || !keys || !opw) return LTP_E_BADARG;
    if ((pay_first == nullptr) != (payload == nullptr)) return LTP_E_BADARG;
    if (!n_threads) n_threads = 1;
    // the pool is checked once, as ltp_serve_submit_rows checks a transaction
    for (uint64_t k = 0; k < n_pool; k++) {
        const uint32_t a = txn_first[k], n = txn_first[k + 1] - txn_first[k];
        const uint64_t p0 = pay_first ? pay_first[k] : 0, np = pay_first ? pay_first[k + 1] - p0 : 0;
        if (txn_first[k + 1] < a || (pay_first && pay_first[k + 1] < p0)) return LTP_E_BADARG;
        if (n > LTP_SERVE_MAX_OPS || n > s->cfg.max_ops || np > s->max_payload) return LTP_E_CAPACITY;
        for (uint32_t j = 0; j < n; j++)
            if (is_insert(opw[a + j]) && (keys[a + j] < p0 || keys[a + j] - p0 >= np)) return LTP_E_BADARG;
    }
    const uint32_t n_lanes = (uint32_t)s->lanes.size();
    const uint64_t t0 = now_ns() + 1000000;  // start 1 ms from now
    const uint64_t t_end = t0 + (uint64_t)(seconds * 1e9);
    std::vector<std::thread> th;
    for (uint32_t g = 0; g < n_threads; g++) {
        th.emplace_back([=]() {
            // this thread's streams: those whose lane no other generator
            // thread uses (lane = stream mod lanes); its own slice of the pool
            std::vector<uint32_t> mine;
            for (uint32_t st = 0; st < n_streams; st++)
                if ((st % n_lanes) % n_threads == g) mine.push_back(st);
            const uint32_t my_streams = (uint32_t)mine.size();
            if (!my_streams) return;
            const double my_rate = rate * (double)my_streams / (double)n_streams;
            std::mt19937_64 rng(seed * 0x9E3779B97F4A7C15ULL + g + 1);
            std::exponential_distribution<double> gap(my_rate / 1e9);
            double t = (double)t0;
            uint64_t k = (n_pool * g) / n_threads;
            uint64_t local_total = 0, local_late = 0, tn = 0;
            while (true) {
                t += gap(rng);
                const uint64_t at = (uint64_t)t;
                if (at >= t_end || s->status) break;
                if (tn < at)  // not due yet (a generator running behind skips the clock read)
                    while ((tn = now_ns()) < at) {
                    }
                local_total++;
                if (tn - at > 100000ull) local_late++;
                const uint32_t st = mine[rng() % my_streams];
                const uint32_t a = txn_first[k], n = txn_first[k + 1] - txn_first[k];
                if (s->status) break;
                if (pay_first)  // the pool's insert keys are offsets into the whole payload
                    admit(s, st, at, k, n, keys + a, opw + a, (uint32_t)(pay_first[k + 1] - pay_first[k]),
                          payload + pay_first[k], pay_first[k]);
                else
                    admit(s, st, at, k, n, keys + a, opw + a, 0, nullptr, 0);
                if (++k == n_pool) k = 0;
            }
            s->lg_total += local_total;
            s->lg_late += local_late;
        });
    }
    for (auto &x : th) x.join();
    return s->status;
}

int ltp_poisson_arrivals(uint64_t n, double rate, uint64_t seed, uint64_t *arrival_ns, int n_threads) {
    if (!arrival_ns || !(rate > 0)) return n ? LTP_E_BADARG : LTP_OK;
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    const uint64_t chunks = std::min<uint64_t>((uint64_t)n_threads, std::max<uint64_t>(1, n / 65536));
    const double mean_gap_ns = 1e9 / rate;
    // each chunk draws its own gaps (its own seeded stream) and sums them;
    // the chunks' totals then shift every later chunk
    std::vector<double> total(chunks, 0.0);
    auto body = [&](uint64_t c, bool shift, double base) {
        const uint64_t lo = n * c / chunks, hi = n * (c + 1) / chunks;
        if (shift) {
            for (uint64_t i = lo; i < hi; i++) arrival_ns[i] += (uint64_t)base;
            return;
        }
        std::mt19937_64 rng(seed * 0x9E3779B97F4A7C15ULL + c * 0xD1B54A32D192ED03ULL + 1);
        std::exponential_distribution<double> gap(1.0 / mean_gap_ns);
        double t = 0.0;
        for (uint64_t i = lo; i < hi; i++) {
            t += gap(rng);
            arrival_ns[i] = (uint64_t)t;
        }
        total[c] = t;
    };
    std::vector<std::thread> th;
    for (uint64_t c = 0; c < chunks; c++) th.emplace_back(body, c, false, 0.0);
    for (auto &x : th) x.join();
    th.clear();
    double base = 0.0;
    for (uint64_t c = 1; c < chunks; c++) {
        base += total[c - 1];
        th.emplace_back(body, c, true, base);
    }
    for (auto &x : th) x.join();
    return LTP_OK;
}

int ltp_serve_stats_now(ltp_server *s, ltp_serve_stats *st) {
    if (!s || !st) return LTP_E_BADARG;
    memset(st, 0, sizeof(*st));
    for (const auto &lp : s->lanes) st->submitted += lp->submitted.load(std::memory_order_relaxed);
    st->completed = s->completed;
    st->committed = s->committed;
    st->aborted_attempts = s->aborted_attempts;
    st->batches = s->batches;
    st->closed_deadline = s->closed_deadline;
    st->closed_budget = s->closed_budget;
    st->closed_idle = s->closed_idle;
    st->ops = s->ops;
    {
        std::lock_guard<std::mutex> g(s->histo_mu);
        st->p50_us = s->histo.pct(0.50) / 1e3;
        st->p99_us = s->histo.pct(0.99) / 1e3;
        st->p999_us = s->histo.pct(0.999) / 1e3;
        st->mean_us = s->histo.n ? s->histo.sum / (double)s->histo.n / 1e3 : 0;
        st->max_us = (double)s->histo.mx / 1e3;
    }
    const uint64_t t_first = s->t_first.load();
    st->elapsed_s = s->t_last > t_first ? (double)(s->t_last - t_first) / 1e9 : 0;
    st->dispatch_busy_s = (double)s->dispatch_ns.load() / 1e9;
    st->complete_busy_s = (double)s->complete_ns.load() / 1e9;
    st->loadgen_late_frac = s->lg_total.load() ? (double)s->lg_late.load() / (double)s->lg_total.load() : 0.0;
    st->committed_per_s = st->elapsed_s > 0 ? (double)s->committed / st->elapsed_s : 0;
    return s->status;
}

int ltp_serve_close(ltp_server *s, ltp_serve_stats *st) {
    if (!s) return LTP_E_BADARG;
    s->stop = true;
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (s->completer.joinable()) s->completer.join();
    {
        std::lock_guard<std::mutex> g(s->asm_mu);
        s->helpers_stop = true;
    }
    s->asm_cv.notify_all();
    for (auto &h : s->helpers) h.join();
    if (st) ltp_serve_stats_now(s, st);
    const int status = s->status;
    if (s->pipe) ltp_pipe_free(s->pipe);
    for (uint32_t i = 0; i < s->n_slots; i++) {
        Slot &sl = s->slots[i];
        ltp_host_free(sl.keys);
        ltp_host_free(sl.opw);
        ltp_host_free(sl.vals);
        ltp_host_free(sl.vals64);
        ltp_host_free(sl.payload);
        ltp_host_free(sl.txn_first);
        ltp_host_free(sl.commit);
    }
    delete s;
    return status;
}

}  // extern "C"
