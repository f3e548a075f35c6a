// ltp_api.cu -- C ABI of the hot path: context, column-store tables, batches,
// execution and results.  Replaces the reference's GPUScheduler singleton
// (cuda/include/gpuscheduler.cuh:54) with an explicit context handle; every
// call returns a status instead of exiting the process.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <unordered_map>
#include <vector>

#include "ltp_host.cuh"
#include "ltp_trace.h"

using namespace ltp;

namespace {

int fail(ltp_ctx *ctx, int status, const char *fmt, const char *detail = "") {
    if (ctx) {
        char buf[512];
        snprintf(buf, sizeof(buf), fmt, detail);
        ctx->last_error = buf;
    }
    return status;
}

int cuda_fail(ltp_ctx *ctx, cudaError_t e, const char *where) {
    std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
    if (ctx) ctx->last_error = msg;
    return (e == cudaErrorMemoryAllocation) ? LTP_E_NOMEM : LTP_E_CUDA;
}

#define CK(call)                                                \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call); \
    } while (0)

#define CK_CTX(c, call)                                          \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return cuda_fail((c), _e, #call); \
    } while (0)

cudaStream_t pick_stream(ltp_ctx *ctx, void *stream) { return stream ? (cudaStream_t)stream : ctx->stream; }

template <typename T>
cudaError_t dalloc(T **p, uint64_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, count * sizeof(T));
}

void free_scratch_ops(Scratch &s) {
    cudaFree(s.tw_list);
    cudaFree(s.list[0]);
    cudaFree(s.list[1]);
    cudaFree(s.dcell);
    cudaFree(s.dbase);
    cudaFree(s.dminw);
    cudaFree(s.st_sort[0]);
    cudaFree(s.st_sort[1]);
    cudaFree(s.st_cls);
    cudaFree(s.st_apply);
    cudaFree(s.st_ins);
    cudaFree(s.ins_pre);
    s.st_ins = nullptr;
    s.ins_pre = nullptr;
    s.tw_list = nullptr;
    s.list[0] = s.list[1] = nullptr;
    s.dcell = nullptr;
    s.dbase = nullptr;
    s.dminw = nullptr;
    s.st_sort[0] = s.st_sort[1] = nullptr;
    s.st_cls = s.st_apply = nullptr;
    s.cap_ops = 0;
}

void free_scratch_words(Scratch &s) {
    cudaFree(s.words);
    cudaFree(s.cview);
    s.words = nullptr;
    s.cview = nullptr;
}

// Sizes the bitmaps to the cell space and the per-op scratch to n_ops.
int ensure_scratch(ltp_ctx *ctx, uint64_t n_ops) {
    Scratch &s = ctx->s;
    const uint64_t words = (ctx->total_cells + 31) / 32 + 1;
    if (words > ctx->alloc_words) {
        CK(cudaStreamSynchronize(ctx->stream));
        free_scratch_words(s);
        // one spare entry: the 64-cell layout of the same buffer rounds up
        CK(dalloc(&s.words, words + 1));
        CK(cudaMemset(s.words, 0, (words + 1) * sizeof(WordState)));
        CK(dalloc(&s.cview, words + 1));  // 8 B per 32 cells; the 64-cell view takes 16 B per word
        CK(cudaMemset(s.cview, 0, (words + 1) * sizeof(uint2)));
        ctx->alloc_words = words;
    }
    s.n_words = words;
    if (n_ops > s.cap_ops) {
        CK(cudaStreamSynchronize(ctx->stream));
        free_scratch_ops(s);
        uint64_t cap = 1024;
        while (cap < n_ops) cap <<= 1;
        const uint64_t tiles = cap / kMinTile + 2;
        const uint64_t stiles = cap / kSortTile + 2;
        CK(dalloc(&s.tw_list, cap));
        CK(dalloc(&s.list[0], cap));
        CK(dalloc(&s.list[1], cap));
        CK(dalloc(&s.dcell, cap));
        CK(dalloc(&s.dbase, cap));
        CK(dalloc(&s.dminw, cap));
        CK(dalloc(&s.st_sort[0], stiles * 256));
        CK(dalloc(&s.st_sort[1], stiles * 256));
        CK(dalloc(&s.st_cls, tiles));
        CK(dalloc(&s.st_apply, tiles));
        CK(dalloc(&s.st_ins, tiles * LTP_MAX_TABLES));
        CK(dalloc(&s.ins_pre, tiles * LTP_MAX_TABLES));
        s.cap_ops = cap;
        s.cap_tiles = tiles;
        s.cap_sort_tiles = stiles;
        CK(launch_reset_scratch(ctx->stream, s));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return LTP_OK;
}

TablesDev tables_dev(const ltp_ctx *ctx) {
    TablesDev T;
    memset(&T, 0, sizeof(T));
    T.n = (uint32_t)ctx->tables.size();
    T.rows_now = ctx->rows_now;
    T.any_wide = ctx->any_wide ? 1u : 0u;
    for (size_t i = 0; i < ctx->tables.size(); i++) T.t[i] = ctx->tables[i].dev;
    return T;
}

uint32_t bucket_of(uint64_t n) {
    uint32_t b = 0;
    while (b < 63 && (2ull << b) <= n) b++;
    return b;
}

}  // namespace

extern "C" {

const char *ltp_version(void) { return "ltpmg_gb300 0.1 (sm_103a)"; }

const char *ltp_status_string(int status) {
    switch (status) {
    case LTP_OK: return "ok";
    case LTP_E_CUDA: return "CUDA runtime error";
    case LTP_E_CAPACITY: return "capacity exceeded";
    case LTP_E_TIMEOUT: return "device-side wait timed out";
    case LTP_E_BADARG: return "invalid argument or malformed operation";
    case LTP_E_DEVICE_ASSERT: return "device consistency check failed";
    case LTP_E_NOMEM: return "out of memory";
    case LTP_E_STATE: return "call out of order";
    default: return "unknown status";
    }
}

const char *ltp_last_error(const ltp_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int ltp_init(const ltp_config *cfg, ltp_ctx **out) {
    if (!cfg || !out) return LTP_E_BADARG;
    *out = nullptr;
    if (cfg->rule != LTP_RULE_ORDERED && cfg->rule != LTP_RULE_PRIORITY) return LTP_E_BADARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return LTP_E_CUDA;
    if (cfg->device < 0 || cfg->device >= ndev) return LTP_E_BADARG;
    ltp_ctx *ctx = new ltp_ctx();
    ctx->device = cfg->device;
    ctx->rule = cfg->rule;
    ctx->flags = cfg->flags;
    memset(&ctx->s, 0, sizeof(ctx->s));
    for (int i = 0; i < 64; i++) ctx->tuning[i] = Tuning{512, 4, 32, 0};
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, cfg->device);
    // random 4-16 byte gathers dominate: fetch 32-byte sectors, not 64-byte pairs
    // (a limit of this process's context only)
    if (e == cudaSuccess) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, 32);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->ctr, sizeof(Counters));
    if (e == cudaSuccess) e = cudaMemset(ctx->ctr, 0, sizeof(Counters));
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->rows_now, LTP_MAX_TABLES * sizeof(u64));
    if (e == cudaSuccess) e = cudaMemset(ctx->rows_now, 0, LTP_MAX_TABLES * sizeof(u64));
    if (e != cudaSuccess) {
        ltp_shutdown(ctx);
        return e == cudaErrorMemoryAllocation ? LTP_E_NOMEM : LTP_E_CUDA;
    }
    if (cfg->reserve_ops) {
        int rc = ensure_scratch(ctx, cfg->reserve_ops);
        if (rc) {
            ltp_shutdown(ctx);
            return rc;
        }
    }
    *out = ctx;
    return LTP_OK;
}

int ltp_shutdown(ltp_ctx *ctx) {
    if (!ctx) return LTP_E_BADARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &t : ctx->tables) cudaFree(t.dev.data);
    free_scratch_ops(ctx->s);
    free_scratch_words(ctx->s);
    cudaFree(ctx->ctr);
    cudaFree(ctx->rows_now);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->p_exec) cudaGraphExecDestroy(ctx->p_exec);
    cudaFree(ctx->p_batches);
    cudaFree(ctx->p_snaps);
    cudaFree(ctx->p_bar);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LTP_OK;
}

void *ltp_default_stream(ltp_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int ltp_sync(ltp_ctx *ctx, void *stream) {
    if (!ctx) return LTP_E_BADARG;
    CK(cudaStreamSynchronize(pick_stream(ctx, stream)));
    return LTP_OK;
}

int ltp_table_create(ltp_ctx *ctx, const ltp_schema *schema, uint64_t rows, uint32_t *table_id) {
    return ltp_table_create_cap(ctx, schema, rows, rows, table_id);
}

int ltp_table_create_cap(ltp_ctx *ctx, const ltp_schema *schema, uint64_t rows, uint64_t rows_cap,
                         uint32_t *table_id) {
    if (!ctx || !schema || !table_id) return LTP_E_BADARG;
    if (rows_cap < rows) return fail(ctx, LTP_E_BADARG, "rows_cap must be >= rows");
    if (schema->n_cols == 0 || schema->n_cols > LTP_MAX_COLS) return fail(ctx, LTP_E_BADARG, "n_cols must be 1..64");
    if (rows_cap == 0 || rows_cap > (1ull << 31)) return fail(ctx, LTP_E_BADARG, "rows_cap must be 1..2^31");
    if (schema->n_cols < 64 && (schema->wide_cols >> schema->n_cols))
        return fail(ctx, LTP_E_BADARG, "wide_cols names a column beyond n_cols");
    if (ctx->tables.size() >= LTP_MAX_TABLES) return fail(ctx, LTP_E_CAPACITY, "at most 16 tables");
    const uint64_t cells = rows_cap * schema->n_cols;
    if ((ctx->total_cells + cells + 31) / 32 >= (1ull << 32))
        return fail(ctx, LTP_E_CAPACITY, "cell space exceeds 2^37 cells");
    CK(cudaSetDevice(ctx->device));
    TableHost t;
    memset(&t, 0, sizeof(t));
    t.n_cols = schema->n_cols;
    t.dev.rows_cap = (rows_cap + 63) & ~63ull;  // 256-byte aligned columns
    t.dev.row_limit = rows_cap;
    t.dev.n_rows = rows;
    t.dev.n_cols = schema->n_cols;
    t.dev.cell_base = ctx->total_cells;
    t.dev.wide = schema->wide_cols;
    t.bytes = col_off(t.dev, schema->n_cols);  // offset one past the last column
    CK(cudaMalloc((void **)&t.dev.data, t.bytes));
    CK(cudaMemset(t.dev.data, 0, t.bytes));
    if (t.dev.wide) ctx->any_wide = true;
    // keep the next table's cells in a fresh bitmap word
    ctx->total_cells += (cells + 31) & ~31ull;
    *table_id = (uint32_t)ctx->tables.size();
    const u64 r = rows;
    CK(cudaMemcpy(ctx->rows_now + *table_id, &r, sizeof(u64), cudaMemcpyHostToDevice));
    ctx->tables.push_back(t);
    return LTP_OK;
}

static int check_table(ltp_ctx *ctx, uint32_t table, uint32_t col, uint64_t row0, uint64_t n) {
    if (!ctx) return LTP_E_BADARG;
    if (table >= ctx->tables.size()) return fail(ctx, LTP_E_BADARG, "no such table");
    const TableHost &t = ctx->tables[table];
    if (col >= t.n_cols) return fail(ctx, LTP_E_BADARG, "no such column");
    u64 rows = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&rows, ctx->rows_now + table, sizeof(u64), cudaMemcpyDeviceToHost));
    if (row0 > rows || n > rows - row0) return fail(ctx, LTP_E_BADARG, "row range out of bounds");
    return LTP_OK;
}

int ltp_table_upload(ltp_ctx *ctx, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, const void *src) {
    int rc = check_table(ctx, table, col, row0, n);
    if (rc) return rc;
    if (!src && n) return LTP_E_BADARG;
    const TableHost &t = ctx->tables[table];
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(t.col_ptr(col, row0), src, n * t.width(col), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return LTP_OK;
}

int ltp_table_download(ltp_ctx *ctx, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, void *dst) {
    int rc = check_table(ctx, table, col, row0, n);
    if (rc) return rc;
    if (!dst && n) return LTP_E_BADARG;
    const TableHost &t = ctx->tables[table];
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpyAsync(dst, t.col_ptr(col, row0), n * t.width(col), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return LTP_OK;
}

int ltp_table_fill_seeded(ltp_ctx *ctx, uint32_t table, uint64_t seed, void *stream) {
    if (!ctx || table >= ctx->tables.size()) return LTP_E_BADARG;
    CK(cudaSetDevice(ctx->device));
    CK(launch_fill_seeded(pick_stream(ctx, stream), ctx->tables[table].dev, seed));
    return LTP_OK;
}

int ltp_table_truncate(ltp_ctx *ctx, uint32_t table, uint64_t rows) {
    uint64_t cur = 0;
    int rc = ltp_table_rows(ctx, table, &cur);
    if (rc) return rc;
    if (rows > cur) return fail(ctx, LTP_E_BADARG, "truncate cannot grow a table");
    const u64 r = rows;
    CK(cudaMemcpy(ctx->rows_now + table, &r, sizeof(u64), cudaMemcpyHostToDevice));
    return LTP_OK;
}

int ltp_ctx_wide(ltp_ctx *ctx) { return ctx && ctx->any_wide ? 1 : 0; }

int ltp_table_rows(ltp_ctx *ctx, uint32_t table, uint64_t *rows) {
    if (!ctx || !rows || table >= ctx->tables.size()) return LTP_E_BADARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    u64 r = 0;
    CK(cudaMemcpy(&r, ctx->rows_now + table, sizeof(u64), cudaMemcpyDeviceToHost));
    *rows = r;
    return LTP_OK;
}

int ltp_table_fingerprint(ltp_ctx *ctx, uint32_t table, uint64_t *out) {
    if (!ctx || !out || table >= ctx->tables.size()) return LTP_E_BADARG;
    const TableHost &t = ctx->tables[table];
    uint64_t nrows = 0;
    int rc0 = ltp_table_rows(ctx, table, &nrows);
    if (rc0) return rc0;
    std::vector<int64_t> buf(nrows);
    uint64_t h = 0xCBF29CE484222325ull;
    for (uint32_t c = 0; c < t.n_cols; c++) {
        int rc = ltp_table_download(ctx, table, c, 0, nrows, buf.data());
        if (rc) return rc;
        const uint8_t *p = (const uint8_t *)buf.data();
        for (uint64_t i = 0; i < nrows * t.width(c); i++) {
            h ^= p[i];
            h *= 0x100000001B3ull;
        }
    }
    *out = h;
    return LTP_OK;
}

int ltp_batch_create(ltp_ctx *ctx, uint64_t max_txns, uint64_t max_ops, ltp_batch **out) {
    if (!ctx || !out) return LTP_E_BADARG;
    *out = nullptr;
    if (max_ops >= (1ull << 30)) return fail(ctx, LTP_E_CAPACITY, "a batch holds fewer than 2^30 ops");
    if (max_txns >= (1ull << 32)) return fail(ctx, LTP_E_CAPACITY, "a batch holds fewer than 2^32 transactions");
    CK(cudaSetDevice(ctx->device));
    ltp_batch *b = new ltp_batch();
    b->cap_txns = max_txns;
    b->cap_ops = max_ops;
    cudaError_t e = dalloc(&b->keys, max_ops);
    if (e == cudaSuccess) e = dalloc(&b->opw, max_ops);
    if (e == cudaSuccess) e = dalloc(&b->op_txn, max_ops);
    if (e == cudaSuccess) e = dalloc(&b->out, max_ops);
    if (e == cudaSuccess && ctx->any_wide) e = dalloc(&b->out64, max_ops);
    if (e == cudaSuccess) e = dalloc(&b->txn_first, max_txns + 1);
    if (e == cudaSuccess) e = dalloc(&b->commit, max_txns);
    if (e == cudaSuccess) e = dalloc(&b->snap, 1);
    if (e == cudaSuccess && (ctx->flags & LTP_FLAG_STAGE_TIMING)) {
        for (int i = 0; e == cudaSuccess && i < LTP_N_STAGES; i++) e = cudaEventCreate(&b->ev[i]);
        b->have_events = e == cudaSuccess;
    }
    if (e != cudaSuccess) {
        ltp_batch_free(ctx, b);
        return cuda_fail(ctx, e, "ltp_batch_create");
    }
    int rc = ensure_scratch(ctx, max_ops);
    if (rc) {
        ltp_batch_free(ctx, b);
        return rc;
    }
    *out = b;
    return LTP_OK;
}

int ltp_batch_free(ltp_ctx *ctx, ltp_batch *b) {
    if (!b) return LTP_E_BADARG;
    if (ctx) cudaSetDevice(ctx->device);
    cudaFree(b->keys);
    cudaFree(b->keys32);
    cudaFree(b->opw);
    cudaFree(b->op_txn);
    cudaFree(b->out);
    cudaFree(b->out64);
    cudaFree(b->txn_first);
    cudaFree(b->commit);
    cudaFree(b->snap);
    cudaFree(b->payload);
    if (b->have_events)
        for (int i = 0; i < LTP_N_STAGES; i++) cudaEventDestroy(b->ev[i]);
    delete b;
    return LTP_OK;
}

static int batch_load(ltp_ctx *ctx, ltp_batch *b, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                      uint64_t n_ops, const void *keys, bool k32, const uint32_t *opw, void *stream) {
    TraceRange tr("ltp_batch_load");
    if (!ctx || !b) return LTP_E_BADARG;
    if (n_txns > b->cap_txns || n_ops > b->cap_ops) return fail(ctx, LTP_E_CAPACITY, "batch larger than its capacity");
    if (n_ops && (!keys || !opw)) return fail(ctx, LTP_E_BADARG, "null op arrays");
    if (txn_first) {
        if (txn_first[0] != 0 || txn_first[n_txns] != n_ops)
            return fail(ctx, LTP_E_BADARG, "txn_first must start at 0 and end at n_ops");
        for (uint64_t t = 0; t < n_txns; t++)
            if (txn_first[t + 1] < txn_first[t]) return fail(ctx, LTP_E_BADARG, "txn_first must be non-decreasing");
    } else if ((uint64_t)ops_per_txn * n_txns != n_ops || (n_txns && ops_per_txn == 0)) {
        return fail(ctx, LTP_E_BADARG, "n_ops must equal n_txns * ops_per_txn");
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    if (ctx->any_wide && !b->out64) {  // an int64 column appeared after the batch was made
        CK(cudaStreamSynchronize(st));
        CK(dalloc(&b->out64, b->cap_ops));
    }
    if (k32 && !b->keys32) {
        CK(cudaStreamSynchronize(st));
        CK(dalloc(&b->keys32, b->cap_ops));
    }
    b->key32 = k32;
    if (n_ops) {
        if (k32) CK(cudaMemcpyAsync(b->keys32, keys, n_ops * 4, cudaMemcpyHostToDevice, st));
        else CK(cudaMemcpyAsync(b->keys, keys, n_ops * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(b->opw, opw, n_ops * 4, cudaMemcpyHostToDevice, st));
    }
    b->n_txns = n_txns;
    b->n_ops = n_ops;
    b->ops_per_txn = txn_first ? 0u : ops_per_txn;
    b->payload_len = 0;
    if (txn_first) {
        CK(cudaMemcpyAsync(b->txn_first, txn_first, (n_txns + 1) * 4, cudaMemcpyHostToDevice, st));
        CK(launch_expand_op_txn(st, b->txn_first, n_txns, b->op_txn));
    }
    b->loaded = true;
    b->executed = false;
    return LTP_OK;
}

int ltp_batch_load(ltp_ctx *ctx, ltp_batch *b, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                   uint64_t n_ops, const uint64_t *keys, const uint32_t *opw, void *stream) {
    return batch_load(ctx, b, n_txns, txn_first, ops_per_txn, n_ops, keys, false, opw, stream);
}

int ltp_batch_load32(ltp_ctx *ctx, ltp_batch *b, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                     uint64_t n_ops, const uint32_t *keys, const uint32_t *opw, void *stream) {
    return batch_load(ctx, b, n_txns, txn_first, ops_per_txn, n_ops, keys, true, opw, stream);
}

int ltp_batch_load_payload(ltp_ctx *ctx, ltp_batch *b, const int32_t *payload, uint64_t n, void *stream) {
    if (!ctx || !b || (n && !payload)) return LTP_E_BADARG;
    if (!b->loaded) return fail(ctx, LTP_E_STATE, "load the batch before its payload");
    if (n >= (1ull << 32)) return fail(ctx, LTP_E_CAPACITY, "a payload holds fewer than 2^32 slots");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    if (n > b->payload_cap) {
        CK(cudaStreamSynchronize(st));
        cudaFree(b->payload);
        b->payload = nullptr;
        b->payload_cap = 0;
        uint64_t cap = 1024;
        while (cap < n) cap <<= 1;
        CK(dalloc(&b->payload, cap));
        b->payload_cap = cap;
    }
    if (n) CK(cudaMemcpyAsync(b->payload, payload, n * 4, cudaMemcpyHostToDevice, st));
    b->payload_len = n;
    return LTP_OK;
}

namespace {

BatchDev batch_dev(const ltp_batch *b) {
    BatchDev bd;
    bd.keys = b->key32 ? nullptr : (const u64 *)b->keys;
    bd.keys32 = b->key32 ? b->keys32 : nullptr;
    bd.opw = b->opw;
    bd.txn_first = b->txn_first;
    bd.op_txn = b->op_txn;
    bd.out = b->out;
    bd.out64 = b->out64;
    bd.commit = b->commit;
    bd.n_ops = b->n_ops;
    bd.n_txns = b->n_txns;
    bd.ops_per_txn = b->ops_per_txn;
    bd.flags = 0;
    bd.payload = b->payload;
    bd.payload_len = b->payload_len;
    return bd;
}

// Stream-ordered launches of one batch (scratch already sized and clean).
int execute_one(ltp_ctx *ctx, ltp_batch *b, cudaStream_t st, bool allow_stall) {
    CK(cudaMemsetAsync(ctx->ctr, 0, sizeof(Counters), st));
    if (b->n_txns) CK(cudaMemsetAsync(b->commit, 1, b->n_txns, st));
    Launch L;
    L.stream = st;
    L.num_sms = ctx->num_sms;
    L.rule = ctx->rule;
    L.tune = ctx->tuning[bucket_of(b->n_ops)];
    L.stall = allow_stall && ctx->stall_ms_next != 0;
    L.stall_ms = ctx->stall_ms_next;
    if (allow_stall) ctx->stall_ms_next = 0;
    L.timing = b->have_events && (ctx->flags & LTP_FLAG_STAGE_TIMING);
    L.ev = b->ev;
    L.progress = b->progress;
    L.progress_stage = b->progress_stage;
    if (b->n_ops) CK(launch_execute(L, batch_dev(b), tables_dev(ctx), ctx->s, ctx->ctr));
    CK(cudaMemcpyAsync(b->snap, ctx->ctr, sizeof(Counters), cudaMemcpyDeviceToDevice, st));
    b->rule = ctx->rule;
    b->executed = true;
    return LTP_OK;
}

int prepare(ltp_ctx *ctx, ltp_batch *const *bs, uint32_t n, cudaStream_t st) {
    uint64_t max_ops = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (!bs[i]) return fail(ctx, LTP_E_BADARG, "null batch");
        if (!bs[i]->loaded) return fail(ctx, LTP_E_STATE, "batch not loaded");
        if (bs[i]->n_ops > max_ops) max_ops = bs[i]->n_ops;
    }
    if (ctx->tables.empty()) return fail(ctx, LTP_E_STATE, "no tables");
    int rc = ensure_scratch(ctx, max_ops);
    if (rc) return rc;
    if (ctx->dirty) {
        CK(launch_reset_scratch(st, ctx->s));
        ctx->dirty = false;
    }
    return LTP_OK;
}

}  // namespace

}  // extern "C"

namespace ltp {
int host_fail(ltp_ctx *ctx, int status, const char *msg) { return fail(ctx, status, "%s", msg); }
int host_cuda_fail(ltp_ctx *ctx, cudaError_t e, const char *where) { return cuda_fail(ctx, e, where); }
int host_prepare(ltp_ctx *ctx, ltp_batch *const *bs, uint32_t n, cudaStream_t st) { return prepare(ctx, bs, n, st); }
int host_execute(ltp_ctx *ctx, ltp_batch *b, cudaStream_t st) { return execute_one(ctx, b, st, false); }
TablesDev host_tables(const ltp_ctx *ctx) { return tables_dev(ctx); }
}  // namespace ltp

extern "C" {

int ltp_batch_execute(ltp_ctx *ctx, ltp_batch *b, void *stream) {
    if (!ctx || !b) return LTP_E_BADARG;
    TraceRange tr("ltp_batch_execute");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    int rc = prepare(ctx, &b, 1, st);
    if (rc) return rc;
    return execute_one(ctx, b, st, true);
}

int ltp_batches_execute(ltp_ctx *ctx, ltp_batch *const *batches, uint32_t n, int32_t mode, void *stream) {
    if (!ctx || (n && !batches)) return LTP_E_BADARG;
    TraceRange tr("ltp_batches_execute");
    if (mode != LTP_MODE_STREAM && mode != LTP_MODE_GRAPH && mode != LTP_MODE_PERSISTENT)
        return fail(ctx, LTP_E_BADARG, "unknown execution mode");
    if (n == 0) return LTP_OK;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    int rc = prepare(ctx, batches, n, st);
    if (rc) return rc;
    if (mode == LTP_MODE_STREAM) {
        for (uint32_t i = 0; i < n; i++)
            if ((rc = execute_one(ctx, batches[i], st, false))) return rc;
        return LTP_OK;
    }
    if (mode == LTP_MODE_GRAPH) {
        // the captured launch sequence bakes in pointers, sizes and tuning
        std::vector<uint64_t> key;
        key.push_back((uint64_t)ctx->rule);
        key.push_back((uint64_t)(uintptr_t)st);
        for (uint32_t i = 0; i < n; i++) {
            const ltp_batch *b = batches[i];
            const Tuning &t = ctx->tuning[bucket_of(b->n_ops)];
            key.insert(key.end(), {(uint64_t)(uintptr_t)b, b->n_ops, b->n_txns, b->ops_per_txn,
                                   (uint64_t)(uintptr_t)b->payload, b->payload_len,
                                   ((uint64_t)t.block << 32) | t.ipt, ((uint64_t)t.word_bits << 32) | t.flags,
                                   (uint64_t)(b->have_events && (ctx->flags & LTP_FLAG_STAGE_TIMING)),
                                   (uint64_t)b->key32});
        }
        key.push_back(ctx->tables.size());
        key.push_back(ctx->any_wide ? 1u : 0u);
        if (!ctx->graph_exec || key != ctx->graph_key) {
            if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            for (uint32_t i = 0; i < n && !rc; i++) rc = execute_one(ctx, batches[i], st, false);
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                ctx->graph_exec = nullptr;
                return cuda_fail(ctx, e, "cudaGraphInstantiate");
            }
            ctx->graph_key = key;
        }
        CK(cudaGraphLaunch(ctx->graph_exec, st));
        for (uint32_t i = 0; i < n; i++) {
            batches[i]->rule = ctx->rule;
            batches[i]->executed = true;
        }
        return LTP_OK;
    }
    // persistent: one cooperative kernel over all batches.  The batch
    // descriptors stay on the device while the list is unchanged, and the
    // launch (counter reset + cooperative kernel) is a captured CUDA graph.
    std::vector<uint64_t> key = {(uint64_t)ctx->rule, ctx->tables.size(), ctx->any_wide ? 1u : 0u};
    for (uint32_t i = 0; i < n; i++) {
        const ltp_batch *b = batches[i];
        key.insert(key.end(), {(uint64_t)(uintptr_t)b, b->n_ops, b->n_txns, b->ops_per_txn,
                               (uint64_t)(uintptr_t)b->payload, b->payload_len,
                               (uint64_t)ctx->tuning[bucket_of(b->n_ops)].flags, (uint64_t)b->key32});
    }
    if (key != ctx->p_key) {
        CK(cudaStreamSynchronize(st));
        if (ctx->p_exec) cudaGraphExecDestroy(ctx->p_exec);
        ctx->p_exec = nullptr;
        ctx->p_key.clear();
        if (n > ctx->p_cap) {
            cudaFree(ctx->p_batches);
            cudaFree(ctx->p_snaps);
            ctx->p_batches = nullptr;
            ctx->p_snaps = nullptr;
            ctx->p_cap = 0;
            CK(dalloc(&ctx->p_batches, n));
            CK(dalloc(&ctx->p_snaps, n));
            ctx->p_cap = n;
        }
        if (!ctx->p_bar) CK(dalloc(&ctx->p_bar, 2));
        std::vector<BatchDev> hb(n);
        std::vector<Counters *> hs(n);
        for (uint32_t i = 0; i < n; i++) {
            hb[i] = batch_dev(batches[i]);
            hb[i].flags = ctx->tuning[bucket_of(batches[i]->n_ops)].flags;
            hs[i] = batches[i]->snap;
        }
        CK(cudaMemcpy(ctx->p_batches, hb.data(), n * sizeof(BatchDev), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->p_snaps, hs.data(), n * sizeof(Counters *), cudaMemcpyHostToDevice));
        ctx->p_key = key;
    }
    if (ctx->p_exec && ctx->p_stream != st) {
        cudaGraphExecDestroy(ctx->p_exec);
        ctx->p_exec = nullptr;
    }
    if (!ctx->p_exec) {
        persistent_grid(ctx->num_sms);  // kernel attributes, outside the capture
        cudaGraph_t graph = nullptr;
        cudaError_t e = ctx->p_no_graph ? cudaErrorNotSupported : cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            cudaMemsetAsync(ctx->ctr, 0, sizeof(Counters), st);
            launch_persistent(st, ctx->num_sms, ctx->rule, ctx->p_batches, ctx->p_snaps, n, tables_dev(ctx), ctx->s,
                              ctx->ctr, ctx->p_bar);
            e = cudaStreamEndCapture(st, &graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->p_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {  // a driver without captured cooperative launches: launch directly
            (void)cudaGetLastError();
            ctx->p_exec = nullptr;
            ctx->p_no_graph = true;
            CK(cudaMemsetAsync(ctx->ctr, 0, sizeof(Counters), st));
            CK(launch_persistent(st, ctx->num_sms, ctx->rule, ctx->p_batches, ctx->p_snaps, n, tables_dev(ctx),
                                 ctx->s, ctx->ctr, ctx->p_bar));
        }
        ctx->p_stream = st;
    }
    if (ctx->p_exec) CK(cudaGraphLaunch(ctx->p_exec, st));
    for (uint32_t i = 0; i < n; i++) {
        batches[i]->rule = ctx->rule;
        batches[i]->executed = true;
    }
    return LTP_OK;
}

int ltp_batch_fetch(ltp_ctx *ctx, ltp_batch *b, uint8_t *commit, int32_t *vals, void *stream) {
    if (!ctx || !b) return LTP_E_BADARG;
    if (!b->executed) return fail(ctx, LTP_E_STATE, "batch not executed");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    if (commit && b->n_txns) CK(cudaMemcpyAsync(commit, b->commit, b->n_txns, cudaMemcpyDeviceToHost, st));
    if (vals && b->n_ops) CK(cudaMemcpyAsync(vals, b->out, b->n_ops * 4, cudaMemcpyDeviceToHost, st));
    return LTP_OK;
}

int ltp_batch_fetch64(ltp_ctx *ctx, ltp_batch *b, int64_t *vals, void *stream) {
    if (!ctx || !b) return LTP_E_BADARG;
    if (!b->executed) return fail(ctx, LTP_E_STATE, "batch not executed");
    if (!b->out64) return fail(ctx, LTP_E_STATE, "the context has no int64 column");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    if (vals && b->n_ops) {
        CK(launch_widen_out(st, batch_dev(b), tables_dev(ctx)));
        CK(cudaMemcpyAsync(vals, b->out64, b->n_ops * 8, cudaMemcpyDeviceToHost, st));
    }
    return LTP_OK;
}

int ltp_batch_finish(ltp_ctx *ctx, ltp_batch *b, ltp_stats *stats, void *stream) {
    if (!ctx || !b) return LTP_E_BADARG;
    if (!b->executed) return fail(ctx, LTP_E_STATE, "batch not executed");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = pick_stream(ctx, stream);
    Counters c;
    CK(cudaMemcpyAsync(&c, b->snap, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->txns = b->n_txns;
        stats->ops = b->n_ops;
        stats->committed = b->rule == LTP_RULE_PRIORITY ? c.committed : b->n_txns;
        stats->aborted = b->n_txns - stats->committed;
        stats->contended_ops = c.n_c;
        stats->contended_cells = c.M;
        stats->touched_words = c.n_tw;
        stats->bytes_algorithmic = 28ull * b->n_ops + 4ull * b->n_txns;
        if (b->have_events && (ctx->flags & LTP_FLAG_STAGE_TIMING) && b->n_ops) {
            // stage events are absent for batches run by the persistent kernel
            for (int i = 0; i < 10; i++) {
                float ms = 0;
                if (cudaEventElapsedTime(&ms, b->ev[i], b->ev[i + 1]) != cudaSuccess) {
                    (void)cudaGetLastError();
                    ms = -1.0f;
                }
                stats->ms_stage[i] = ms;
            }
            float total = 0;
            if (cudaEventElapsedTime(&total, b->ev[0], b->ev[10]) != cudaSuccess) {
                (void)cudaGetLastError();
                total = -1.0f;
            }
            stats->ms_stage[11] = total;
        }
    }
    if (c.err) {
        ctx->dirty = true;
        if (c.err == LTP_E_BADARG && c.bad_op) {
            char buf[128];
            snprintf(buf, sizeof(buf), "malformed op at index %llu (key/column/table/kind out of range)",
                     (unsigned long long)~c.bad_op);
            ctx->last_error = buf;
        } else {
            ctx->last_error = ltp_status_string(c.err);
        }
        return c.err;
    }
    return LTP_OK;
}

int ltp_batch_results(ltp_ctx *ctx, ltp_batch *b, uint8_t *commit, int32_t *vals, ltp_stats *stats) {
    int rc = ltp_batch_fetch(ctx, b, commit, vals, nullptr);
    if (rc) return rc;
    return ltp_batch_finish(ctx, b, stats, nullptr);
}

int ltp_batch_device_ptrs(ltp_batch *b, uint64_t **keys, uint32_t **opw, uint32_t **txn_first, int32_t **vals,
                          uint8_t **commit) {
    if (!b) return LTP_E_BADARG;
    if (keys) *keys = b->key32 ? nullptr : b->keys;
    if (opw) *opw = b->opw;
    if (txn_first) *txn_first = b->txn_first;
    if (vals) *vals = b->out;
    if (commit) *commit = b->commit;
    return LTP_OK;
}

void *ltp_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
    return p;
}

void ltp_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

int ltp_set_tuning(ltp_ctx *ctx, uint32_t bucket, const ltp_tuning *t) {
    if (!ctx || !t || bucket >= 64) return LTP_E_BADARG;
    if (t->block != 128 && t->block != 256 && t->block != 512) return fail(ctx, LTP_E_BADARG, "block must be 128/256/512");
    if (t->ipt != 1 && t->ipt != 2 && t->ipt != 4 && t->ipt != 8) return fail(ctx, LTP_E_BADARG, "ipt must be 1/2/4/8");
    if (t->word_bits != 32 && t->word_bits != 64) return fail(ctx, LTP_E_BADARG, "word_bits must be 32 or 64");
    if (!tiling_supported((int)t->block, (int)t->ipt, (int)t->word_bits))
        return fail(ctx, LTP_E_BADARG, "64-cell conflict words need block x ipt <= 2048");
    if (t->flags & ~LTP_TUNE_MARK_PRECHECK) return fail(ctx, LTP_E_BADARG, "unknown tuning flag");
    ctx->tuning[bucket] = Tuning{t->block, t->ipt, t->word_bits, t->flags};
    return LTP_OK;
}

int ltp_get_tuning(ltp_ctx *ctx, uint32_t bucket, ltp_tuning *t) {
    if (!ctx || !t || bucket >= 64) return LTP_E_BADARG;
    t->block = ctx->tuning[bucket].block;
    t->ipt = ctx->tuning[bucket].ipt;
    t->word_bits = ctx->tuning[bucket].word_bits;
    t->flags = ctx->tuning[bucket].flags;
    return LTP_OK;
}

int ltp_set_stage_timing(ltp_ctx *ctx, int32_t on) {
    if (!ctx) return LTP_E_BADARG;
    if (on) ctx->flags |= LTP_FLAG_STAGE_TIMING;
    else ctx->flags &= ~LTP_FLAG_STAGE_TIMING;
    return LTP_OK;
}

int ltp_debug_stall_next(ltp_ctx *ctx, uint32_t ms) {
    if (!ctx || ms == 0 || ms > 10000) return LTP_E_BADARG;
    ctx->stall_ms_next = ms;
    return LTP_OK;
}

}  // extern "C"

// ============================================================================
// pipelined submission
// ============================================================================
namespace {

struct PipeSlot {
    ltp_batch *b = nullptr;
    cudaEvent_t in = nullptr, exec = nullptr, out = nullptr;
    cudaGraphExec_t gexec = nullptr;   // this slot's captured launch sequence ...
    std::vector<uint64_t> gkey;        // ... for batches of this shape
    std::vector<uint64_t> last_key;    // shape of the slot's previous batch
    BatchDev *h_desc = nullptr;    // pinned staging of the batch descriptor (persistent execution)
    BatchDev *d_desc = nullptr;    // device copy the persistent kernel reads
    Counters **d_snap = nullptr;   // device array holding b->snap
    Counters *host_ctr = nullptr;  // pinned copy of the batch's counters
    uint64_t ticket = UINT64_MAX;
    bool waited = true;
    int status = LTP_OK;
};

}  // namespace

struct PipeDone {
    int status;
    ltp_stats stats;
};

struct ltp_pipe {
    ltp_ctx *ctx = nullptr;
    bool persistent = false;  // each batch runs as one persistent-kernel launch
    std::vector<PipeSlot> slots;
    cudaStream_t s_in = nullptr, s_out = nullptr;
    uint64_t next = 0;
    std::unordered_map<uint64_t, PipeDone> done;  // finished tickets whose slot was reused
};

static void pipe_stats(const PipeSlot &sl, ltp_stats *stats) {
    memset(stats, 0, sizeof(*stats));
    const Counters &c = *sl.host_ctr;
    stats->txns = sl.b->n_txns;
    stats->ops = sl.b->n_ops;
    stats->committed = sl.b->rule == LTP_RULE_PRIORITY ? c.committed : sl.b->n_txns;
    stats->aborted = sl.b->n_txns - stats->committed;
    stats->contended_ops = c.n_c;
    stats->contended_cells = c.M;
    stats->touched_words = c.n_tw;
    stats->bytes_algorithmic = 28ull * sl.b->n_ops + 4ull * sl.b->n_txns;
}

// Executes the slot's batch on sx.  A slot that sees two batches of the same
// shape in a row captures their launch sequence as a CUDA graph and replays
// it while the shape stays (one launch call instead of a dozen).
static int pipe_execute(ltp_ctx *ctx, PipeSlot &sl, cudaStream_t sx) {
    const ltp_batch *b = sl.b;
    const Tuning &t = ctx->tuning[bucket_of(b->n_ops)];
    const std::vector<uint64_t> key = {b->n_ops, b->n_txns, b->ops_per_txn, (uint64_t)(uintptr_t)b->payload,
                                       b->payload_len, ((uint64_t)t.block << 32) | t.ipt,
                                       ((uint64_t)t.word_bits << 32) | t.flags, (uint64_t)b->key32,
                                       (uint64_t)ctx->rule,
                                       (uint64_t)(b->have_events && (ctx->flags & LTP_FLAG_STAGE_TIMING)),
                                       ctx->tables.size(), ctx->any_wide ? 1u : 0u};
    if (sl.gexec && key == sl.gkey) {
        CK(cudaGraphLaunch(sl.gexec, sx));
        sl.b->rule = ctx->rule;
        sl.b->executed = true;
        return LTP_OK;
    }
    if (key != sl.last_key) {
        sl.last_key = key;
        return execute_one(ctx, sl.b, sx, false);
    }
    if (sl.gexec) cudaGraphExecDestroy(sl.gexec);
    sl.gexec = nullptr;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(sx, cudaStreamCaptureModeRelaxed));
    int rc = execute_one(ctx, sl.b, sx, false);
    cudaError_t e = cudaStreamEndCapture(sx, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&sl.gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        sl.gexec = nullptr;
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    sl.gkey = key;
    CK(cudaGraphLaunch(sl.gexec, sx));
    return LTP_OK;
}

static int pipe_finalize(ltp_pipe *p, PipeSlot &sl) {
    ltp_ctx *ctx = p->ctx;
    CK(cudaEventSynchronize(sl.out));
    if (!sl.waited) {
        sl.status = sl.host_ctr->err;
        if (sl.status) ctx->dirty = true;
        sl.waited = true;
    }
    return LTP_OK;
}

extern "C" {

int ltp_pipe_create(ltp_ctx *ctx, uint32_t depth, uint64_t max_txns, uint64_t max_ops, ltp_pipe **out) {
    return ltp_pipe_create2(ctx, depth, max_txns, max_ops, 0, out);
}

int ltp_pipe_create2(ltp_ctx *ctx, uint32_t depth, uint64_t max_txns, uint64_t max_ops, uint32_t flags,
                     ltp_pipe **out) {
    if (!ctx || !out || depth < 2 || depth > 64 || (flags & ~LTP_PIPE_PERSISTENT)) return LTP_E_BADARG;
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    int rc = ensure_scratch(ctx, max_ops);
    if (rc) return rc;
    ltp_pipe *p = new ltp_pipe();
    p->ctx = ctx;
    p->persistent = (flags & LTP_PIPE_PERSISTENT) != 0;
    p->slots.resize(depth);
    cudaError_t e = cudaStreamCreateWithFlags(&p->s_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->s_out, cudaStreamNonBlocking);
    for (auto &sl : p->slots) {
        if (e != cudaSuccess) break;
        if ((rc = ltp_batch_create(ctx, max_txns, max_ops, &sl.b))) break;
        e = cudaEventCreateWithFlags(&sl.in, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.exec, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.out, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.host_ctr, sizeof(Counters));
        if (e == cudaSuccess && p->persistent) {
            e = cudaMallocHost((void **)&sl.h_desc, sizeof(BatchDev));
            if (e == cudaSuccess) e = dalloc(&sl.d_desc, 1);
            if (e == cudaSuccess) e = dalloc(&sl.d_snap, 1);
            if (e == cudaSuccess) e = cudaMemcpy(sl.d_snap, &sl.b->snap, sizeof(Counters *), cudaMemcpyHostToDevice);
        }
    }
    if (!rc && e == cudaSuccess && p->persistent && !ctx->p_bar) e = dalloc(&ctx->p_bar, 2);
    if (rc || e != cudaSuccess) {
        ltp_pipe_free(p);
        return rc ? rc : cuda_fail(ctx, e, "ltp_pipe_create");
    }
    *out = p;
    return LTP_OK;
}

int ltp_pipe_free(ltp_pipe *p) {
    if (!p) return LTP_E_BADARG;
    ltp_ctx *ctx = p->ctx;
    cudaSetDevice(ctx->device);
    for (auto &sl : p->slots) {
        if (sl.out) cudaEventSynchronize(sl.out);
        if (sl.b) ltp_batch_free(ctx, sl.b);
        if (sl.in) cudaEventDestroy(sl.in);
        if (sl.exec) cudaEventDestroy(sl.exec);
        if (sl.out) cudaEventDestroy(sl.out);
        if (sl.host_ctr) cudaFreeHost(sl.host_ctr);
        if (sl.h_desc) cudaFreeHost(sl.h_desc);
        if (sl.gexec) cudaGraphExecDestroy(sl.gexec);
        cudaFree(sl.d_desc);
        cudaFree(sl.d_snap);
    }
    if (p->s_in) cudaStreamDestroy(p->s_in);
    if (p->s_out) cudaStreamDestroy(p->s_out);
    delete p;
    return LTP_OK;
}

}  // extern "C"

static int pipe_submit(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                       const void *keys, bool k32, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                       uint8_t *commit_out, int32_t *vals_out, int64_t *vals64_out, uint64_t *ticket) {
    if (!p) return LTP_E_BADARG;
    TraceRange tr("ltp_pipe_submit");
    ltp_ctx *ctx = p->ctx;
    CK(cudaSetDevice(ctx->device));
    const uint64_t t = p->next;
    PipeSlot &sl = p->slots[t % p->slots.size()];
    if (sl.ticket != UINT64_MAX) {  // the slot's previous batch must be out
        const bool unwaited = !sl.waited;
        int rc = pipe_finalize(p, sl);
        if (rc) return rc;
        if (unwaited) {  // keep its status for a later ltp_pipe_wait
            PipeDone d;
            d.status = sl.status;
            pipe_stats(sl, &d.stats);
            p->done[sl.ticket] = d;
        }
    }
    if (ctx->dirty) return fail(ctx, LTP_E_STATE, "an earlier batch of this pipeline failed");
    int rc = batch_load(ctx, sl.b, n_txns, txn_first, ops_per_txn, n_ops, keys, k32, opw, p->s_in);
    if (rc) return rc;
    if (payload && payload_len) {
        if (payload_len > sl.b->payload_cap) CK(cudaStreamSynchronize(p->s_in));
        if ((rc = ltp_batch_load_payload(ctx, sl.b, payload, payload_len, p->s_in))) return rc;
    }
    CK(cudaEventRecord(sl.in, p->s_in));
    cudaStream_t sx = ctx->stream;
    CK(cudaStreamWaitEvent(sx, sl.in, 0));
    if (p->persistent && sl.b->n_ops) {
        // one cooperative launch runs every phase of the batch; its
        // descriptor goes up from pinned staging on the execution stream
        *sl.h_desc = batch_dev(sl.b);
        sl.h_desc->flags = ctx->tuning[bucket_of(sl.b->n_ops)].flags;
        CK(cudaMemcpyAsync(sl.d_desc, sl.h_desc, sizeof(BatchDev), cudaMemcpyHostToDevice, sx));
        CK(cudaMemsetAsync(ctx->ctr, 0, sizeof(Counters), sx));
        CK(launch_persistent(sx, ctx->num_sms, ctx->rule, sl.d_desc, sl.d_snap, 1, tables_dev(ctx), ctx->s, ctx->ctr,
                             ctx->p_bar));
        sl.b->rule = ctx->rule;
        sl.b->executed = true;
    } else if ((rc = pipe_execute(ctx, sl, sx))) {
        return rc;
    }
    CK(cudaMemcpyAsync(sl.host_ctr, sl.b->snap, sizeof(Counters), cudaMemcpyDeviceToHost, sx));
    CK(cudaEventRecord(sl.exec, sx));
    CK(cudaStreamWaitEvent(p->s_out, sl.exec, 0));
    if ((rc = ltp_batch_fetch(ctx, sl.b, commit_out, vals_out, p->s_out))) return rc;
    if (vals64_out && (rc = ltp_batch_fetch64(ctx, sl.b, vals64_out, p->s_out))) return rc;
    CK(cudaEventRecord(sl.out, p->s_out));
    sl.ticket = t;
    sl.waited = false;
    sl.status = LTP_OK;
    p->next = t + 1;
    if (ticket) *ticket = t;
    return LTP_OK;
}

extern "C" {

int ltp_pipe_submit(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                    const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                    uint8_t *commit_out, int32_t *vals_out, uint64_t *ticket) {
    return pipe_submit(p, n_txns, txn_first, ops_per_txn, n_ops, keys, false, opw, payload, payload_len, commit_out,
                       vals_out, nullptr, ticket);
}

int ltp_pipe_submit32(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                      const uint32_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                      uint8_t *commit_out, int32_t *vals_out, uint64_t *ticket) {
    return pipe_submit(p, n_txns, txn_first, ops_per_txn, n_ops, keys, true, opw, payload, payload_len, commit_out,
                       vals_out, nullptr, ticket);
}

int ltp_pipe_submit64(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                      const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                      uint8_t *commit_out, int64_t *vals_out, uint64_t *ticket) {
    return pipe_submit(p, n_txns, txn_first, ops_per_txn, n_ops, keys, false, opw, payload, payload_len, commit_out,
                       nullptr, vals_out, ticket);
}

int ltp_pipe_wait(ltp_pipe *p, uint64_t ticket, ltp_stats *stats) {
    if (!p) return LTP_E_BADARG;
    TraceRange tr("ltp_pipe_wait");
    auto it = p->done.find(ticket);
    if (it != p->done.end()) {
        const PipeDone d = it->second;
        p->done.erase(it);
        if (stats) *stats = d.stats;
        if (d.status) p->ctx->last_error = ltp_status_string(d.status);
        return d.status;
    }
    PipeSlot &sl = p->slots[ticket % p->slots.size()];
    if (sl.ticket != ticket) return fail(p->ctx, LTP_E_STATE, "unknown or already waited ticket");
    CK_CTX(p->ctx, cudaSetDevice(p->ctx->device));
    int rc = pipe_finalize(p, sl);
    if (rc) return rc;
    if (stats) pipe_stats(sl, stats);
    if (sl.status) p->ctx->last_error = ltp_status_string(sl.status);
    return sl.status;
}

int ltp_pipe_poll(ltp_pipe *p, uint64_t ticket) {
    if (!p) return LTP_E_BADARG;
    if (p->done.count(ticket)) return LTP_OK;
    PipeSlot &sl = p->slots[ticket % p->slots.size()];
    if (sl.ticket != ticket) return LTP_E_STATE;
    cudaError_t e = cudaEventQuery(sl.out);
    if (e == cudaErrorNotReady) return 1;
    if (e != cudaSuccess) return cuda_fail(p->ctx, e, "ltp_pipe_poll");
    return LTP_OK;
}

}  // extern "C"
