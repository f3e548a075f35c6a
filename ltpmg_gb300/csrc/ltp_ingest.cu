// ltp_ingest.cu -- serving from a device-resident request log.
//
// The host-API server (ltp_serve.cpp) pays per transaction on the host: a
// client thread appends it to a lane, the dispatcher copies it into a pinned
// batch, the copy engine moves it to HBM.  Here requests are already in HBM
// when they arrive (as a NIC writing by GPUDirect RDMA would place them) and
// carry arrival times, so the host loop only moves log indices:
//   * admission: every request whose arrival time has passed is pending; a
//     batch closes on the rules of the host server (deadline after the
//     oldest pending arrival, slot capacity / read-write-set budget, or --
//     with LTP_SERVE_EAGER -- when the device has nothing in flight);
//   * a batch is a list of log runs: re-queued aborts first (the priority
//     rule's losers, oldest batch first, in their batch order), then the
//     newly arrived requests in arrival order.  The log's keys and opwords
//     are stored twice back to back, so any window of at most n_pool
//     consecutive requests is contiguous: a batch of new requests only
//     executes in place from the log (its transaction offsets are rebased;
//     a pool of equal-length transactions needs not even that).  Other
//     batches are gathered from the log by kernels.  Keys are stored as
//     32-bit keys when every key of the pool fits;
//   * just-in-time queueing (LTP_SERVE_JIT): with a batch executing, the
//     next one is closed only once the executing batch has passed a late
//     stage (its radix sort, or classify for small batches), so requests
//     arriving meanwhile still join it instead of waiting a whole batch
//     behind a queued one;
//   * completion: the batch's counters (and, under the priority rule, its
//     commit vector) come back; latencies of a run of requests are added to
//     the histogram with one binary search per bucket, because arrivals
//     within a run are sorted.
// The per-batch host work is a few kernel launches plus O(runs + aborts),
// independent of how many requests a batch holds.
#include <string.h>
#include <time.h>

#include <algorithm>
#include <deque>
#include <unordered_map>
#include <vector>

#include "ltp_histo.h"
#include "ltp_host.cuh"
#include "ltp_trace.h"

using namespace ltp;

namespace {

uint64_t mono_ns() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

// Requests [log0, log0 + n) = pool transactions [pool0, pool0 + n), placed
// at transaction t0, op o0 and payload slot p0 of the batch.  Runs are in
// batch order: t0, o0 and p0 never decrease from one run to the next.
struct LogRun {
    u64 pool0, log0, o0, p0;
    u32 n, t0;
};

// last run with t0 <= t
__device__ __forceinline__ u32 run_of_txn(const LogRun *runs, u32 n_runs, u32 t) {
    u32 lo = 0, hi = n_runs;
    while (hi - lo > 1) {
        const u32 mid = (lo + hi) >> 1;
        if (runs[mid].t0 <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

// last run with p0 <= s: runs without payload share p0 with the run after
// them, so the last one is the run whose payload holds slot s
__device__ __forceinline__ u32 run_of_slot(const LogRun *runs, u32 n_runs, u64 s) {
    u32 lo = 0, hi = n_runs;
    while (hi - lo > 1) {
        const u32 mid = (lo + hi) >> 1;
        if (runs[mid].p0 <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Transaction offsets of the batch (rebased onto its op array) and the log
// index of each of its transactions.
__global__ void k_log_txns(const LogRun *runs, u32 n_runs, u32 n_txns, u64 n_ops, const u32 *p_tf, u32 *txn_first,
                           u64 *txn_log) {
    for (u32 t = blockIdx.x * blockDim.x + threadIdx.x; t < n_txns; t += gridDim.x * blockDim.x) {
        const LogRun R = runs[run_of_txn(runs, n_runs, t)];
        const u64 pt = R.pool0 + (t - R.t0);
        txn_first[t] = (u32)(R.o0 + (p_tf[pt] - p_tf[R.pool0]));
        txn_log[t] = R.log0 + (t - R.t0);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) txn_first[n_txns] = (u32)n_ops;
}

// Keys (u64 or u32) and opwords of the batch; an insert's key (a payload
// offset in the pool) is moved onto the batch payload.  opt > 0: every
// transaction has opt ops (txn_first and op_txn are not built).
template <typename K>
__global__ void k_log_ops(const LogRun *runs, u32 n_runs, u64 n_ops, u32 opt, const u32 *txn_first,
                          const u32 *op_txn, const u32 *p_tf, const K *p_keys, const u32 *p_opw, const u64 *p_pf,
                          K *keys, u32 *opw) {
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < n_ops; j += (u64)gridDim.x * blockDim.x) {
        const u32 t = opt ? (u32)(j / opt) : op_txn[j];
        const LogRun R = runs[run_of_txn(runs, n_runs, t)];
        const u64 src = p_tf[R.pool0 + (t - R.t0)] + (j - (opt ? (u64)t * opt : (u64)txn_first[t]));
        K k = p_keys[src];
        const u32 w = p_opw[src];
        if (p_pf && opw_kind(w) == LTP_OP_INSERT) k = (K)(k - p_pf[R.pool0] + R.p0);
        keys[j] = k;
        opw[j] = w;
    }
}

__global__ void k_log_payload(const LogRun *runs, u32 n_runs, u64 n_slots, const u64 *p_pf, const int32_t *p_pay,
                              int32_t *pay) {
    for (u64 s = (u64)blockIdx.x * blockDim.x + threadIdx.x; s < n_slots; s += (u64)gridDim.x * blockDim.x) {
        const LogRun R = runs[run_of_slot(runs, n_runs, s)];
        pay[s] = p_pay[p_pf[R.pool0] + (s - R.p0)];
    }
}

// Op values of the batch into the log's value array (log index < pool size);
// ops on int64 cells have theirs in out64, the others in out.
__global__ void k_log_vals(u64 n_ops, u32 opt, const u32 *txn_first, const u32 *op_txn, const u64 *txn_log,
                           const u32 *p_tf, const u32 *opw, const TablesDev T, const int32_t *out,
                           const long long *out64, long long *vals) {
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < n_ops; j += (u64)gridDim.x * blockDim.x) {
        const u32 t = opt ? (u32)(j / opt) : op_txn[j], w = opw[j], tb = opw_table(w);
        const bool wide = out64 && opw_kind(w) <= LTP_OP_ADD && tb < T.n && col_wide(T.t[tb], opw_col(w));
        vals[p_tf[txn_log[t]] + (j - (opt ? (u64)t * opt : (u64)txn_first[t]))] = wide ? out64[j] : (long long)out[j];
    }
}

unsigned grid_for(u64 n, int num_sms) {
    const u64 want = (n + 255) / 256, cap = (u64)num_sms * 8;
    return (unsigned)std::max<u64>(1, std::min(want, cap));
}

struct IngestSlot {
    ltp_batch *b = nullptr;
    uint64_t *own_keys = nullptr;  // the batch's own arrays (gathered batches; 32-bit keys use own_keys' storage)
    uint32_t *own_keys32 = nullptr;
    uint32_t *own_opw = nullptr;
    int32_t *own_pay = nullptr;
    LogRun *h_runs = nullptr, *d_runs = nullptr;  // pinned staging, device copy
    u64 *d_txn_log = nullptr;
    Counters *host_ctr = nullptr;
    uint8_t *h_commit = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t progress = nullptr;  // the batch is past its sort (LTP_SERVE_JIT)
    std::vector<LogRun> runs;
    uint64_t seq = 0;
};

struct BatchRecord {  // which requests a batch held, for ltp_ingest_results
    uint64_t seq;
    std::vector<LogRun> runs;
};

}  // namespace

struct ltp_ingest {
    ltp_ctx *ctx = nullptr;
    ltp_serve_config cfg;
    uint64_t cap_ops = 0, max_payload = 0;
    bool keep = false;
    // the pool, on the device and its offsets on the host; keys and opwords
    // are stored twice back to back ([2 * pool_ops]), keys as u32 when k32
    uint64_t n_pool = 0, pool_ops = 0, pool_pay = 0;
    bool k32 = false;
    uint32_t fixed_ops = 0;  // > 0: every pool transaction has this many ops
    u32 *p_tf = nullptr;
    void *p_keys = nullptr;
    u64 *p_pf = nullptr;
    u32 *p_opw = nullptr;
    int32_t *p_pay = nullptr;
    std::vector<uint32_t> tf;
    std::vector<uint64_t> pf;
    std::vector<IngestSlot> slots;
    long long *d_vals = nullptr;  // [pool_ops] op values of the last run (LTP_SERVE_KEEP_RESULTS)
    // the last run
    uint64_t n_run = 0;
    std::vector<BatchRecord> history;
    std::unordered_map<uint64_t, uint32_t> aborts;  // request -> tries that aborted
    std::vector<uint64_t> given_up;
    uint64_t seq = 0;

    uint64_t log_ops(uint64_t i) const { return (i / n_pool) * pool_ops + tf[i % n_pool]; }
    uint64_t log_pay(uint64_t i) const { return pf.empty() ? 0 : (i / n_pool) * pool_pay + pf[i % n_pool]; }
    uint64_t txn_ops(uint64_t li) const { return tf[li % n_pool + 1] - tf[li % n_pool]; }
    uint64_t txn_pay(uint64_t li) const { return pf.empty() ? 0 : pf[li % n_pool + 1] - pf[li % n_pool]; }
};

namespace {

#define IK(call)                                                           \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) return host_cuda_fail(g->ctx, _e, #call);   \
    } while (0)

void free_slot(IngestSlot &sl, ltp_ctx *ctx) {
    if (sl.done) cudaEventSynchronize(sl.done);
    if (sl.b) {
        sl.b->keys = sl.own_keys;
        sl.b->keys32 = sl.own_keys32;
        sl.b->opw = sl.own_opw;
        sl.b->payload = sl.own_pay;
        ltp_batch_free(ctx, sl.b);
    }
    if (sl.h_runs) cudaFreeHost(sl.h_runs);
    cudaFree(sl.d_runs);
    cudaFree(sl.d_txn_log);
    if (sl.host_ctr) cudaFreeHost(sl.host_ctr);
    if (sl.h_commit) cudaFreeHost(sl.h_commit);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.progress) cudaEventDestroy(sl.progress);
    sl = IngestSlot();
}

// Launches one batch of the given runs (t txns, o ops, p payload slots) in
// slot sl.  `view`: new requests only (at most n_pool, so at most two runs,
// contiguous in the doubled log), executed in place from the log.
int submit(ltp_ingest *g, IngestSlot &sl, uint32_t t, uint64_t o, uint64_t p, bool view) {
    ltp_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    ltp_batch *b = sl.b;
    const uint32_t nr = (uint32_t)sl.runs.size();
    const uint32_t opt = g->fixed_ops;
    memcpy(sl.h_runs, sl.runs.data(), nr * sizeof(LogRun));
    IK(cudaMemcpyAsync(sl.d_runs, sl.h_runs, nr * sizeof(LogRun), cudaMemcpyHostToDevice, st));
    if (!opt || g->keep) {  // fixed-length batches need neither offsets nor op -> transaction map
        k_log_txns<<<grid_for(t, ctx->num_sms), 256, 0, st>>>(sl.d_runs, nr, t, o, g->p_tf, b->txn_first,
                                                             sl.d_txn_log);
        IK(cudaGetLastError());
    }
    if (!opt) IK(launch_expand_op_txn(st, b->txn_first, t, b->op_txn));
    b->key32 = g->k32;
    if (view) {
        const uint64_t first = g->tf[sl.runs[0].pool0];
        if (g->k32) b->keys32 = (uint32_t *)g->p_keys + first;
        else b->keys = (uint64_t *)g->p_keys + first;
        b->opw = g->p_opw + first;
        b->payload = g->p_pay;  // insert keys index the whole pool payload
        b->payload_len = g->pool_pay;
    } else {
        b->keys = sl.own_keys;
        b->keys32 = (uint32_t *)sl.own_keys;
        b->opw = sl.own_opw;
        b->payload = sl.own_pay;
        b->payload_len = p;
        if (g->k32)
            k_log_ops<u32><<<grid_for(o, ctx->num_sms), 256, 0, st>>>(sl.d_runs, nr, o, opt, b->txn_first, b->op_txn,
                                                                     g->p_tf, (const u32 *)g->p_keys, g->p_opw,
                                                                     g->p_pf, b->keys32, b->opw);
        else
            k_log_ops<u64><<<grid_for(o, ctx->num_sms), 256, 0, st>>>(sl.d_runs, nr, o, opt, b->txn_first, b->op_txn,
                                                                     g->p_tf, (const u64 *)g->p_keys, g->p_opw,
                                                                     g->p_pf, (u64 *)b->keys, b->opw);
        IK(cudaGetLastError());
        if (p) {
            k_log_payload<<<grid_for(p, ctx->num_sms), 256, 0, st>>>(sl.d_runs, nr, p, g->p_pf, g->p_pay, b->payload);
            IK(cudaGetLastError());
        }
    }
    b->n_txns = t;
    b->n_ops = o;
    b->ops_per_txn = opt;
    // the "nearly done" mark: after apply in a large batch (inserts and
    // clean-up left), after the radix sort in a mid-sized one, after
    // classify in a small one -- what is left must cover the host's close
    // and first launches of the next batch (~40 us)
    b->progress = (g->cfg.flags & LTP_SERVE_JIT) ? sl.progress : nullptr;
    b->progress_stage = o >= (1ull << 22) ? 8 : o >= (1ull << 20) ? 7 : 3;
    b->loaded = true;
    b->executed = false;
    int rc = host_prepare(ctx, &b, 1, st);
    if (!rc) rc = host_execute(ctx, b, st);
    // the launches hold the pointers they were given: the batch owns its arrays again
    b->keys = sl.own_keys;
    b->keys32 = sl.own_keys32;
    b->key32 = false;
    b->opw = sl.own_opw;
    b->payload = sl.own_pay;
    b->progress = nullptr;
    if (rc) return rc;
    if (g->keep) {
        const u32 *opw = view ? g->p_opw + g->tf[sl.runs[0].pool0] : sl.own_opw;
        k_log_vals<<<grid_for(o, ctx->num_sms), 256, 0, st>>>(o, opt, b->txn_first, b->op_txn, sl.d_txn_log, g->p_tf,
                                                             opw, host_tables(ctx), b->out, b->out64, g->d_vals);
        IK(cudaGetLastError());
    }
    IK(cudaMemcpyAsync(sl.host_ctr, b->snap, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    if (ctx->rule == LTP_RULE_PRIORITY) IK(cudaMemcpyAsync(sl.h_commit, b->commit, t, cudaMemcpyDeviceToHost, st));
    IK(cudaEventRecord(sl.done, st));
    return LTP_OK;
}

struct RunState {
    const uint64_t *arr = nullptr;
    uint64_t n = 0, head = 0, arrived = 0;
    std::deque<uint64_t> requeue;
    uint64_t rq_ops = 0, rq_pay = 0;
    std::deque<uint32_t> inflight;  // slot indices, oldest first
    Histo histo;
    uint64_t completed = 0, committed = 0, aborted_attempts = 0, batches = 0, ops = 0;
    uint64_t closed_deadline = 0, closed_budget = 0, closed_idle = 0;
    uint64_t t_last = 0;
    uint64_t dispatch_ns = 0, complete_ns = 0;
};

// Folds a finished batch into the run: latencies, commits, re-queued aborts.
int complete(ltp_ingest *g, RunState &R, IngestSlot &sl, uint64_t done) {
    TraceRange tr("ingest: complete batch");
    if (sl.host_ctr->err) {
        g->ctx->dirty = true;
        return host_fail(g->ctx, sl.host_ctr->err, "a served batch failed on the device");
    }
    const uint32_t t = sl.b->n_txns;
    for (const LogRun &r : sl.runs) R.histo.add_sorted(done, R.arr, r.log0, r.log0 + r.n);
    uint64_t n_abort = 0;
    if (g->ctx->rule == LTP_RULE_PRIORITY) {
        const uint8_t *c = sl.h_commit;
        for (const uint8_t *z = (const uint8_t *)memchr(c, 0, t); z; z = (const uint8_t *)memchr(z + 1, 0, c + t - z - 1)) {
            const uint32_t pos = (uint32_t)(z - c);
            size_t k = 0;  // run holding this position
            for (size_t lo = 0, hi = sl.runs.size(); hi - lo > 1;) {
                const size_t mid = (lo + hi) / 2;
                if (sl.runs[mid].t0 <= pos) lo = mid;
                else hi = mid;
                k = lo;
            }
            const uint64_t li = sl.runs[k].log0 + (pos - sl.runs[k].t0);
            R.histo.remove(done - R.arr[li]);
            n_abort++;
            R.aborted_attempts++;
            const uint32_t tries = ++g->aborts[li];
            if (tries < g->cfg.max_attempts) {
                R.requeue.push_back(li);
                R.rq_ops += g->txn_ops(li);
                R.rq_pay += g->txn_pay(li);
            } else {
                g->given_up.push_back(li);
                R.completed++;
            }
            if (z + 1 >= c + t) break;
        }
    }
    R.committed += t - n_abort;
    R.completed += t - n_abort;
    R.t_last = done;
    g->history.push_back(BatchRecord{sl.seq, sl.runs});
    return LTP_OK;
}

// Closes a batch from the re-queued and the arrived requests if a rule says
// so.
int maybe_close(ltp_ingest *g, RunState &R, uint64_t now) {
    const uint64_t rq = R.requeue.size(), fresh = R.arrived - R.head;
    if (rq + fresh == 0 || R.inflight.size() >= g->cfg.depth) return LTP_OK;
    const uint64_t oldest = rq ? R.arr[R.requeue.front()] : R.arr[R.head];
    const uint64_t p_ops = R.rq_ops + g->log_ops(R.arrived) - g->log_ops(R.head);
    const uint64_t p_pay = R.rq_pay + g->log_pay(R.arrived) - g->log_pay(R.head);
    const bool deadline = now >= oldest + (uint64_t)g->cfg.deadline_us * 1000ull;
    const bool full = p_ops >= g->cap_ops || rq + fresh >= g->cfg.max_txns || p_pay >= g->max_payload;
    // just in time: the batch ahead (the last one launched) is past its sort
    const bool jit = (g->cfg.flags & LTP_SERVE_JIT) != 0;
    const bool ahead_ending =
        R.inflight.empty() || (jit && cudaEventQuery(g->slots[R.inflight.back()].progress) != cudaErrorNotReady);
    if (jit && !ahead_ending && !full) return LTP_OK;
    const bool idle = (g->cfg.flags & LTP_SERVE_EAGER) && ahead_ending;
    if (!deadline && !full && !idle) return LTP_OK;
    TraceRange tr("ingest: close batch");
    const uint64_t t0 = mono_ns();
    const uint32_t si = (uint32_t)(g->seq % g->slots.size());
    IngestSlot &sl = g->slots[si];
    sl.runs.clear();
    uint32_t t = 0;
    uint64_t o = 0, p = 0;
    while (!R.requeue.empty()) {  // re-queued transactions first
        const uint64_t li = R.requeue.front(), no = g->txn_ops(li), np = g->txn_pay(li);
        if (t + 1 > g->cfg.max_txns || o + no > g->cap_ops || p + np > g->max_payload) break;
        const uint64_t pt = li % g->n_pool;
        if (!sl.runs.empty() && sl.runs.back().log0 + sl.runs.back().n == li && sl.runs.back().pool0 + sl.runs.back().n == pt)
            sl.runs.back().n++;
        else
            sl.runs.push_back(LogRun{pt, li, o, p, 1u, t});
        t++;
        o += no;
        p += np;
        R.requeue.pop_front();
        R.rq_ops -= no;
        R.rq_pay -= np;
    }
    const bool had_requeue = t > 0;
    if (R.requeue.empty() && R.arrived > R.head) {  // then the arrived requests, as many as fit
        uint64_t e = std::min<uint64_t>(R.arrived, R.head + (g->cfg.max_txns - t));
        const uint64_t ob = g->log_ops(R.head), pb = g->log_pay(R.head);
        uint64_t lo = R.head, hi = e;  // largest e' in [head, e] within the op and payload room
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo + 1) / 2;
            if (g->log_ops(mid) - ob <= g->cap_ops - o && g->log_pay(mid) - pb <= g->max_payload - p) lo = mid;
            else hi = mid - 1;
        }
        e = lo;
        for (uint64_t i = R.head; i < e;) {  // one run per stretch that does not wrap the pool
            const uint64_t pt = i % g->n_pool, m = std::min<uint64_t>(e - i, g->n_pool - pt);
            sl.runs.push_back(LogRun{pt, i, o + (g->log_ops(i) - ob), p + (g->log_pay(i) - pb), (u32)m,
                                     (u32)(t + (i - R.head))});
            i += m;
        }
        t += (uint32_t)(e - R.head);
        o += g->log_ops(e) - ob;
        p += g->log_pay(e) - pb;
        R.head = e;
    }
    if (t == 0) return host_fail(g->ctx, LTP_E_CAPACITY, "a request does not fit an empty batch");
    if (deadline) R.closed_deadline++;
    else if (full) R.closed_budget++;
    else R.closed_idle++;
    const bool view = !had_requeue && t <= g->n_pool;
    sl.seq = g->seq++;
    const int rc = submit(g, sl, t, o, p, view);
    if (rc) return rc;
    R.inflight.push_back(si);
    R.batches++;
    R.ops += o;
    R.dispatch_ns += mono_ns() - t0;
    return LTP_OK;
}

}  // namespace

extern "C" {

int ltp_ingest_open(ltp_ctx *ctx, const ltp_serve_config *cfg, uint64_t n_pool, const uint32_t *txn_first,
                    const uint64_t *keys, const uint32_t *opw, const uint64_t *pay_first, const int32_t *payload,
                    ltp_ingest **out) {
    if (!ctx || !cfg || !out || !n_pool || !txn_first || !keys || !opw) return LTP_E_BADARG;
    if ((pay_first == nullptr) != (payload == nullptr)) return LTP_E_BADARG;
    if (cfg->depth < 2 || cfg->depth > 64 || cfg->max_txns == 0 || cfg->max_ops == 0) return LTP_E_BADARG;
    *out = nullptr;
    const uint64_t cap_ops = std::min<uint64_t>(cfg->max_ops, cfg->budget_bytes / 12);
    const uint64_t max_payload = cfg->max_ops * 6;
    if (txn_first[0] != 0 || (pay_first && pay_first[0] != 0)) return host_fail(ctx, LTP_E_BADARG, "pool offsets must start at 0");
    for (uint64_t k = 0; k < n_pool; k++) {  // every request must fit an empty batch and name its own payload
        if (txn_first[k + 1] < txn_first[k] || (pay_first && pay_first[k + 1] < pay_first[k]))
            return host_fail(ctx, LTP_E_BADARG, "pool offsets must be non-decreasing");
        const uint64_t no = txn_first[k + 1] - txn_first[k], p0 = pay_first ? pay_first[k] : 0;
        const uint64_t np = pay_first ? pay_first[k + 1] - p0 : 0;
        if (no > cap_ops || np > max_payload) return host_fail(ctx, LTP_E_CAPACITY, "a pool transaction exceeds a batch");
        for (uint64_t j = txn_first[k]; j < txn_first[k + 1]; j++)
            if ((opw[j] & 3u) == LTP_OP_INSERT && (keys[j] < p0 || keys[j] - p0 >= np))
                return host_fail(ctx, LTP_E_BADARG, "an insert's payload row lies outside its transaction's payload");
    }
    const uint64_t pool_ops = txn_first[n_pool], pool_pay = pay_first ? pay_first[n_pool] : 0;
    if (pool_pay >= (1ull << 32)) return host_fail(ctx, LTP_E_CAPACITY, "pool payload must be below 2^32 slots");
    bool k32 = !(cfg->flags & LTP_SERVE_KEYS64);
    for (uint64_t j = 0; j < pool_ops && k32; j++) k32 = keys[j] < (1ull << 32);
    uint32_t fixed_ops = txn_first[1];
    for (uint64_t k = 1; k < n_pool && fixed_ops; k++)
        if (txn_first[k + 1] - txn_first[k] != fixed_ops) fixed_ops = 0;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return LTP_E_CUDA;
    ltp_ingest *g = new ltp_ingest();
    g->ctx = ctx;
    g->cfg = *cfg;
    if (g->cfg.max_attempts == 0) g->cfg.max_attempts = 1;
    g->cap_ops = cap_ops;
    g->max_payload = max_payload;
    g->keep = (cfg->flags & LTP_SERVE_KEEP_RESULTS) != 0;
    g->n_pool = n_pool;
    g->pool_ops = pool_ops;
    g->pool_pay = pool_pay;
    g->k32 = k32;
    g->fixed_ops = fixed_ops;
    g->tf.assign(txn_first, txn_first + n_pool + 1);
    if (pay_first) g->pf.assign(pay_first, pay_first + n_pool + 1);
    auto up = [&](void **dst, const void *src, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(dst, bytes ? bytes : 4);
        if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        return e;
    };
    // the log's keys and opwords twice, back to back
    auto up2 = [&](void **dst, const void *src, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(dst, bytes ? 2 * bytes : 4);
        if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && bytes) e = cudaMemcpy((char *)*dst + bytes, src, bytes, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up((void **)&g->p_tf, txn_first, (n_pool + 1) * 4);
    if (e == cudaSuccess) {
        if (k32) {
            std::vector<uint32_t> k4(keys, keys + pool_ops);
            e = up2(&g->p_keys, k4.data(), pool_ops * 4);
        } else {
            e = up2(&g->p_keys, keys, pool_ops * 8);
        }
    }
    if (e == cudaSuccess) e = up2((void **)&g->p_opw, opw, pool_ops * 4);
    if (e == cudaSuccess && pay_first) e = up((void **)&g->p_pf, pay_first, (n_pool + 1) * 8);
    if (e == cudaSuccess && pay_first) e = up((void **)&g->p_pay, payload, pool_pay * 4);
    if (e == cudaSuccess && g->keep) e = cudaMalloc((void **)&g->d_vals, std::max<uint64_t>(pool_ops, 1) * 8);
    int rc = LTP_OK;
    g->slots.resize(cfg->depth);
    for (auto &sl : g->slots) {
        if (e != cudaSuccess || rc) break;
        if ((rc = ltp_batch_create(ctx, cfg->max_txns, cap_ops, &sl.b))) break;
        sl.own_keys = sl.b->keys;
        sl.own_keys32 = sl.b->keys32;
        sl.own_opw = sl.b->opw;
        e = cudaMalloc((void **)&sl.own_pay, std::max<uint64_t>(max_payload, 1) * 4);
        sl.b->payload = sl.own_pay;
        sl.b->payload_cap = max_payload;
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.h_runs, (cfg->max_txns + 2) * sizeof(LogRun));
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.d_runs, (cfg->max_txns + 2) * sizeof(LogRun));
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.d_txn_log, cfg->max_txns * sizeof(u64));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.host_ctr, sizeof(Counters));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.h_commit, cfg->max_txns);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.progress, cudaEventDisableTiming);
    }
    if (rc || e != cudaSuccess) {
        if (!rc) rc = host_cuda_fail(ctx, e, "ltp_ingest_open");
        ltp_ingest_close(g);
        return rc;
    }
    *out = g;
    return LTP_OK;
}

int ltp_ingest_run(ltp_ingest *g, uint64_t n_txns, const uint64_t *arrival_ns, ltp_serve_stats *st) {
    if (!g || (n_txns && !arrival_ns)) return LTP_E_BADARG;
    for (uint64_t i = 1; i < n_txns; i++)
        if (arrival_ns[i] < arrival_ns[i - 1]) return host_fail(g->ctx, LTP_E_BADARG, "arrival times must not decrease");
    if (g->keep && n_txns > g->n_pool)
        return host_fail(g->ctx, LTP_E_BADARG, "kept results need n_txns <= the pool size");
    ltp_ctx *ctx = g->ctx;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return LTP_E_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return host_fail(ctx, LTP_E_CUDA, "device error before the run");
    g->n_run = n_txns;
    g->history.clear();
    g->aborts.clear();
    g->given_up.clear();
    RunState R;
    R.arr = arrival_ns;
    R.n = n_txns;
    const uint64_t base = mono_ns() + 200000;  // the run starts 200 us from now
    int rc = LTP_OK;
    for (;;) {
        while (!R.inflight.empty()) {  // finished batches, in order
            IngestSlot &sl = g->slots[R.inflight.front()];
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess) {
                rc = host_cuda_fail(ctx, q, "served batch");
                break;
            }
            const uint64_t c0 = mono_ns();
            const uint64_t now = c0 > base ? c0 - base : 0;
            if ((rc = complete(g, R, sl, now))) break;
            R.inflight.pop_front();
            R.complete_ns += mono_ns() - c0;
        }
        if (rc) break;
        if (R.head == R.n && R.requeue.empty() && R.inflight.empty()) break;
        const uint64_t c = mono_ns();
        const uint64_t now = c > base ? c - base : 0;
        if (R.arrived < R.n && R.arr[R.arrived] <= now)
            R.arrived = (uint64_t)(std::upper_bound(R.arr + R.arrived, R.arr + R.n, now) - R.arr);
        if ((rc = maybe_close(g, R, now))) break;
    }
    if (rc) {  // let what was launched finish before the caller touches the tables
        cudaStreamSynchronize(ctx->stream);
        return rc;
    }
    if (st) {
        memset(st, 0, sizeof(*st));
        st->submitted = n_txns;
        st->completed = R.completed;
        st->committed = R.committed;
        st->aborted_attempts = R.aborted_attempts;
        st->batches = R.batches;
        st->closed_deadline = R.closed_deadline;
        st->closed_budget = R.closed_budget;
        st->closed_idle = R.closed_idle;
        st->ops = R.ops;
        st->p50_us = R.histo.pct(0.50) / 1e3;
        st->p99_us = R.histo.pct(0.99) / 1e3;
        st->p999_us = R.histo.pct(0.999) / 1e3;
        st->mean_us = R.histo.n ? R.histo.sum / (double)R.histo.n / 1e3 : 0;
        st->max_us = (double)R.histo.mx / 1e3;
        const uint64_t first = n_txns ? arrival_ns[0] : 0;
        st->elapsed_s = R.t_last > first ? (double)(R.t_last - first) / 1e9 : 0;
        st->committed_per_s = st->elapsed_s > 0 ? (double)R.committed / st->elapsed_s : 0;
        st->dispatch_busy_s = (double)R.dispatch_ns / 1e9;
        st->complete_busy_s = (double)R.complete_ns / 1e9;
    }
    return LTP_OK;
}

int ltp_ingest_results(ltp_ingest *g, uint8_t *committed, uint64_t *batch_seq, uint32_t *pos, uint32_t *attempts,
                       int64_t *vals) {
    if (!g) return LTP_E_BADARG;
    const uint64_t n = g->n_run;
    if (committed) {
        memset(committed, 1, n);
        for (uint64_t li : g->given_up) committed[li] = 0;
    }
    if (batch_seq || pos) {  // later tries overwrite earlier ones
        for (const BatchRecord &br : g->history)
            for (const LogRun &r : br.runs)
                for (uint32_t k = 0; k < r.n; k++) {
                    if (batch_seq) batch_seq[r.log0 + k] = br.seq;
                    if (pos) pos[r.log0 + k] = r.t0 + k;
                }
    }
    if (attempts) {
        for (uint64_t i = 0; i < n; i++) attempts[i] = 1;
        for (const auto &kv : g->aborts) attempts[kv.first] += kv.second;
        for (uint64_t li : g->given_up) attempts[li] -= 1;  // its last abort was its last try
    }
    if (vals) {
        if (!g->keep) return host_fail(g->ctx, LTP_E_STATE, "values need LTP_SERVE_KEEP_RESULTS");
        if (cudaSetDevice(g->ctx->device) != cudaSuccess) return LTP_E_CUDA;
        const uint64_t ops = g->log_ops(n);
        if (ops) IK(cudaMemcpy(vals, g->d_vals, ops * 8, cudaMemcpyDeviceToHost));
    }
    return LTP_OK;
}

int ltp_ingest_close(ltp_ingest *g) {
    if (!g) return LTP_E_BADARG;
    cudaSetDevice(g->ctx->device);
    for (auto &sl : g->slots) free_slot(sl, g->ctx);
    cudaFree(g->p_tf);
    cudaFree(g->p_keys);
    cudaFree(g->p_opw);
    cudaFree(g->p_pf);
    cudaFree(g->p_pay);
    cudaFree(g->d_vals);
    delete g;
    return LTP_OK;
}

}  // extern "C"
