// ltp_host.cuh -- host-side state shared by the C ABI translation units:
// the context, its tables and the batch object, plus the few entry points
// the request-log server (ltp_ingest.cu) drives a batch through.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "ltp_internal.cuh"

using ltp::TableDev;
using ltp::Scratch;
using ltp::Counters;
using ltp::Tuning;
using ltp::BatchDev;
using ltp::TablesDev;
using ltp::u64;
using ltp::u32;

struct TableHost {
    TableDev dev;
    uint32_t n_cols;
    uint64_t bytes;  // whole allocation (every column over rows_cap rows)

    uint32_t width(uint32_t col) const { return col_wide(dev, col) ? 8u : 4u; }
    char *col_ptr(uint32_t col, uint64_t row) const { return dev.data + col_off(dev, col) + row * width(col); }
};

struct ltp_ctx {
    int device = 0;
    int rule = LTP_RULE_ORDERED;
    uint32_t flags = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<TableHost> tables;
    uint64_t total_cells = 0;
    bool any_wide = false;  // some table has an int64 column
    Scratch s;
    uint64_t alloc_words = 0;  // bitmap words currently allocated
    Counters *ctr = nullptr;
    u64 *rows_now = nullptr;  // [LTP_MAX_TABLES] device row counts
    std::string last_error;
    Tuning tuning[64];
    uint32_t stall_ms_next = 0;
    bool dirty = false;  // scratch must be reset before the next batch
    // multi-batch execution: cached CUDA graph and persistent-kernel buffers
    std::vector<uint64_t> graph_key;
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    BatchDev *p_batches = nullptr;
    Counters **p_snaps = nullptr;
    uint32_t p_cap = 0;
    u32 *p_bar = nullptr;
    std::vector<uint64_t> p_key;          // batch list whose descriptors are on the device
    cudaGraphExec_t p_exec = nullptr;     // captured persistent launch for that list
    cudaStream_t p_stream = nullptr;
    bool p_no_graph = false;              // capture of the cooperative launch failed once: launch directly
};

struct ltp_batch {
    uint64_t cap_txns = 0, cap_ops = 0;
    uint64_t *keys = nullptr;
    uint32_t *keys32 = nullptr;  // 32-bit keys (allocated at the first ltp_batch_load32)
    bool key32 = false;          // the loaded batch carries 32-bit keys
    uint32_t *opw = nullptr, *txn_first = nullptr, *op_txn = nullptr;
    int32_t *out = nullptr;
    long long *out64 = nullptr;  // full outputs, allocated once the context has int64 columns
    uint8_t *commit = nullptr;
    uint64_t n_txns = 0, n_ops = 0;
    uint32_t ops_per_txn = 0;
    bool loaded = false, executed = false;
    int rule = 0;
    Counters *snap = nullptr;  // device copy of the counters after this batch
    int32_t *payload = nullptr;
    uint64_t payload_cap = 0, payload_len = 0;
    cudaEvent_t ev[LTP_N_STAGES];
    bool have_events = false;
    cudaEvent_t progress = nullptr;  // recorded after stage progress_stage of the next execution
    int progress_stage = 0;
};

namespace ltp {

// ctx->last_error = msg; returns status
int host_fail(ltp_ctx *ctx, int status, const char *msg);
int host_cuda_fail(ltp_ctx *ctx, cudaError_t e, const char *where);
// Sizes and, if needed, resets the scratch for these batches.
int host_prepare(ltp_ctx *ctx, ltp_batch *const *bs, uint32_t n, cudaStream_t st);
// Stream-ordered launches of one loaded batch (counters, commit init,
// kernels, counter snapshot).
int host_execute(ltp_ctx *ctx, ltp_batch *b, cudaStream_t st);
// Device view of the context's tables.
TablesDev host_tables(const ltp_ctx *ctx);

}  // namespace ltp
