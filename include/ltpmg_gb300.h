/*
 * ltpmg_gb300.h -- C ABI of the GB300-native batched transaction-processing
 * hot path (one GPU, hand-written sm_103a CUDA).
 *
 * The reference exposes eight C++ entry points between its host program and
 * its CUDA library (cuda/src/gpuscheduler.cu:3-47, declared in
 * include/database.h:66-70, include/query.h:63-70, include/scheduler.h:33-37).
 * This header is the plain-pointer layer those entry points forward to; the
 * reference-compatible C++ shims live in include/ltpmg_compat.h.  Every
 * function returns LTP_OK (0) or a negative LTP_E_* status and never exits
 * the process (the reference's CHECK macro printed and called exit(-1),
 * cuda/include/define.cuh:57-65).
 *
 * Data model
 *  - A context owns one CUDA device, its tables and all scratch memory.
 *  - A table is column-store: one contiguous array per column, int32 or
 *    int64 (ltp_schema.wide_cols).  Cells are addressed by (table, row =
 *    key, column).  Arithmetic on a cell wraps at its own width.
 *  - A batch is a transaction-major list of operations: transaction t owns
 *    ops [txn_first[t], txn_first[t+1]); its TID is t.  Each op is a 64-bit
 *    key (the row id) and a 32-bit opword (LTP_OPW below).
 *  - Outputs per batch: commit[t] (1 committed, 0 aborted) and, per op, the
 *    value of the cell immediately after the op in the serial order (the
 *    value read, or the value the read-modify-write produced; 0 for ops of
 *    aborted transactions).  ltp_batch_fetch returns the low 32 bits of
 *    each value; ltp_batch_fetch64 the full value once the context has an
 *    int64 column.  The table state is read back with ltp_table_download.
 *
 * Rules (ltp_config.rule)
 *  - LTP_RULE_ORDERED: every op on a cell runs in ascending (TID, op) order
 *    and every transaction commits -- the reference's rule (per-row TID
 *    order: cuda/src/gpulauncher.cu:382-418, 2439-2671).
 *  - LTP_RULE_PRIORITY: deterministic TID-priority abort: a transaction
 *    aborts when a smaller TID writes a cell it reads or writes.
 */
#ifndef LTPMG_GB300_H
#define LTPMG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LTP_OK 0
#define LTP_E_CUDA (-1)          /* a CUDA runtime call failed */
#define LTP_E_CAPACITY (-2)      /* a size exceeds what the context or batch holds */
#define LTP_E_TIMEOUT (-3)       /* a bounded device-side wait ran out */
#define LTP_E_BADARG (-4)        /* invalid argument or malformed operation */
#define LTP_E_DEVICE_ASSERT (-5) /* a kernel's own consistency check failed */
#define LTP_E_NOMEM (-6)         /* device or pinned-host allocation failed */
#define LTP_E_STATE (-7)         /* call out of order (e.g. results before execute) */

#define LTP_RULE_ORDERED 0
#define LTP_RULE_PRIORITY 1

#define LTP_MAX_TABLES 16
#define LTP_MAX_COLS 64

/* opword: bits 0-1 kind, 2-7 column, 8-11 table, 12-31 signed immediate */
#define LTP_OP_READ 0u
#define LTP_OP_ADD 1u /* read-modify-write: cell += immediate (two's-complement wrap) */
/* Insert: appends one row to the op's table.  The op's key is an offset into
 * the batch's insert payload (ltp_batch_load_payload) where the new row's
 * values start: one int32 slot per int32 column, two (low word first) per
 * int64 column.  The new row's id is the table's row count at batch start
 * plus the number of committed inserts into that table earlier in (TID, op)
 * order; it is the op's output value.  A new row cannot be named by other
 * ops of its batch.
 * Linked insert: when the low 10 bits of the immediate hold a distance d > 0,
 * column `col` of the new row takes the output of op i - d (a read or
 * read-modify-write of the same transaction) instead of its payload value --
 * e.g. an order row taking the order id its transaction just drew from the
 * district's next-order-id counter.  With d = 0 the column and immediate
 * fields are unused. */
#define LTP_OP_INSERT 2u
#define LTP_INSERT_LINK(col, table, d) LTP_OPW(LTP_OP_INSERT, col, table, (d) & 0x3FF)
#define LTP_OPW(kind, col, table, imm) \
    ((uint32_t)(kind) | ((uint32_t)(col) << 2) | ((uint32_t)(table) << 8) | (((uint32_t)(imm) & 0xFFFFFu) << 12))

#define LTP_FLAG_STAGE_TIMING 1u /* record CUDA events around every stage */

typedef struct ltp_ctx ltp_ctx;
typedef struct ltp_batch ltp_batch;

typedef struct {
    int32_t device;       /* CUDA device ordinal */
    int32_t rule;         /* LTP_RULE_* */
    uint64_t reserve_ops; /* pre-size scratch for batches of this many ops (0: on demand) */
    uint32_t flags;       /* LTP_FLAG_* */
    uint32_t reserved;
} ltp_config;

typedef struct {
    uint32_t n_cols;    /* 1..LTP_MAX_COLS columns */
    uint32_t reserved;
    uint64_t wide_cols; /* bit c set: column c holds int64, else int32 */
} ltp_schema;

#define LTP_N_STAGES 12
typedef struct {
    uint64_t txns, ops, committed, aborted;
    uint64_t contended_ops;   /* ops on cells touched >1 time with >=1 write */
    uint64_t contended_cells;
    uint64_t touched_words;   /* conflict words (32 or 64 cells, ltp_tuning.word_bits) touched by the batch */
    uint64_t bytes_algorithmic;
    /* with LTP_FLAG_STAGE_TIMING, milliseconds per kernel of the batch:
     * ordered rule:  0 mark, 1 ids, 2 classify, 3-6 radix passes, 7 apply,
     *                8 insert, 9 finish
     * priority rule: 0 mark, 1 ids, 2 min-writer, 3 abort, 4 execute,
     *                8 insert, 9 finish
     * and 11 the whole batch */
    float ms_stage[LTP_N_STAGES];
} ltp_stats;

typedef struct {
    uint64_t seed;
    uint64_t n_rows;
    uint32_t n_cols;
    uint32_t ops_min, ops_max; /* ops per transaction, uniform in [ops_min, ops_max] */
    int32_t rmw_delta;         /* immediate of every RMW op */
    double read_frac;          /* probability that an op is a read */
    double theta;              /* 0: uniform keys; else Zipf(theta) over a seeded permutation */
} ltp_ycsb_params;

/* ---- version / errors ------------------------------------------------ */
const char *ltp_version(void);
const char *ltp_status_string(int status);
const char *ltp_last_error(const ltp_ctx *ctx);

/* ---- context --------------------------------------------------------- */
/* Replaces GPUScheduler's global state (cuda/include/gpuscheduler.cuh:54). */
int ltp_init(const ltp_config *cfg, ltp_ctx **out);
int ltp_shutdown(ltp_ctx *ctx);
/* Raw cudaStream_t of the context's own stream (used when a NULL stream is passed). */
void *ltp_default_stream(ltp_ctx *ctx);
int ltp_sync(ltp_ctx *ctx, void *stream);

/* ---- tables (GPUdatabase::malloc_global_row / copy_to_global_row,
 *      cuda/src/gpudatabase.cu:9-238, made column-store) ---------------- */
int ltp_table_create(ltp_ctx *ctx, const ltp_schema *schema, uint64_t rows, uint32_t *table_id);
/* Same with room for inserts: rows_cap >= rows rows are allocated. */
int ltp_table_create_cap(ltp_ctx *ctx, const ltp_schema *schema, uint64_t rows, uint64_t rows_cap,
                         uint32_t *table_id);
/* Copies rows [row0, row0+n) of one column from host memory (n int32 or
 * int64 values, the column's own width). */
int ltp_table_upload(ltp_ctx *ctx, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, const void *src);
/* New: the reference never copies tables back (gpudatabase.cu:240-339). */
int ltp_table_download(ltp_ctx *ctx, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, void *dst);
/* Device-side fill with ltp_table_value(seed, row, col, n_cols); an int64
 * column holds that value sign-extended. */
int ltp_table_fill_seeded(ltp_ctx *ctx, uint32_t table, uint64_t seed, void *stream);
/* FNV-1a 64 of the whole table (column-major bytes), computed on the host
 * from a download; for checkpoints and tests. */
int ltp_table_fingerprint(ltp_ctx *ctx, uint32_t table, uint64_t *out);

/* ---- batches (GPUquery::malloc_global_txn / copy_global_txn,
 *      cuda/src/gpuquery.cu:17-627) -------------------------------------- */
int ltp_batch_create(ltp_ctx *ctx, uint64_t max_txns, uint64_t max_ops, ltp_batch **out);
int ltp_batch_free(ltp_ctx *ctx, ltp_batch *b);
/* Asynchronous host->device copy of a batch.  txn_first has n_txns+1
 * entries; when it is NULL every transaction has ops_per_txn ops. */
int ltp_batch_load(ltp_ctx *ctx, ltp_batch *b, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                   uint64_t n_ops, const uint64_t *keys, const uint32_t *opw, void *stream);
/* The same with 32-bit keys (row ids below 2^32, as the reference's YCSB
 * ROW_ID): a third less to copy per op.  Insert keys (payload offsets) must
 * fit too. */
int ltp_batch_load32(ltp_ctx *ctx, ltp_batch *b, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                     uint64_t n_ops, const uint32_t *keys, const uint32_t *opw, void *stream);
/* Asynchronous host->device copy of the batch's insert payload (n int32
 * values, read by LTP_OP_INSERT ops through their key).  Call after
 * ltp_batch_load; a batch loaded without a payload has none. */
int ltp_batch_load_payload(ltp_ctx *ctx, ltp_batch *b, const int32_t *payload, uint64_t n, void *stream);
/* Current row count of a table (grows with committed inserts); synchronises. */
int ltp_table_rows(ltp_ctx *ctx, uint32_t table, uint64_t *rows);
/* Drops the rows at and above `rows` (<= the current count): later inserts
 * reuse their slots.  Synchronises. */
int ltp_table_truncate(ltp_ctx *ctx, uint32_t table, uint64_t rows);
/* 1 when some table of the context has an int64 column (outputs then have a
 * 64-bit copy, ltp_batch_fetch64), else 0. */
int ltp_ctx_wide(ltp_ctx *ctx);
/* Executes one batch against the context's tables (replaces
 * GPUlauncher::txn_kernel_launcher, cuda/src/gpulauncher.cu:755-1116). */
int ltp_batch_execute(ltp_ctx *ctx, ltp_batch *b, void *stream);
/* Many batches in order, against the context's tables, with no host round
 * trip between them:
 *  LTP_MODE_STREAM     every batch's kernels launched in order on the stream;
 *  LTP_MODE_GRAPH      the same launch sequence captured once into a CUDA
 *                      graph (re-captured when a batch's size, pointers or
 *                      tuning change) and replayed with one graph launch;
 *  LTP_MODE_PERSISTENT one cooperative persistent kernel runs every batch
 *                      through all phases with bounded grid-wide barriers;
 *                      returns after the kernel completes.
 * Per-batch results and status come from ltp_batch_fetch / ltp_batch_finish
 * as for ltp_batch_execute.  Replaces the reference's per-epoch
 * execute_on_GPU loop (src/scheduler.cpp:44-59). */
#define LTP_MODE_STREAM 0
#define LTP_MODE_GRAPH 1
#define LTP_MODE_PERSISTENT 2
int ltp_batches_execute(ltp_ctx *ctx, ltp_batch *const *batches, uint32_t n, int32_t mode, void *stream);
/* Asynchronous device->host copy of the outputs (commit may be NULL, vals
 * may be NULL). */
int ltp_batch_fetch(ltp_ctx *ctx, ltp_batch *b, uint8_t *commit, int32_t *vals, void *stream);
/* The same for the full 64-bit output values (needs an int64 column in the
 * context; LTP_E_STATE otherwise). */
int ltp_batch_fetch64(ltp_ctx *ctx, ltp_batch *b, int64_t *vals, void *stream);
/* Synchronises the stream, then fills stats (may be NULL) and reports any
 * device-side error of the batch. */
int ltp_batch_finish(ltp_ctx *ctx, ltp_batch *b, ltp_stats *stats, void *stream);
/* Convenience: fetch + finish. */
int ltp_batch_results(ltp_ctx *ctx, ltp_batch *b, uint8_t *commit, int32_t *vals, ltp_stats *stats);
/* Device pointers of a loaded batch's arrays (for zero-copy callers); *keys
 * is the 64-bit key array, or NULL while the batch carries 32-bit keys
 * (ltp_batch_load32). */
int ltp_batch_device_ptrs(ltp_batch *b, uint64_t **keys, uint32_t **opw, uint32_t **txn_first, int32_t **vals,
                          uint8_t **commit);

/* ---- pipelined submission ---------------------------------------------- */
/* A pipeline keeps `depth` device batch slots and three streams: batch k+1's
 * host->device copy and batch k-1's device->host copy overlap batch k's
 * execution.  Batches execute one after another in submission order against
 * the context's tables (the serial order of the whole stream of batches).
 * Host buffers should be pinned (ltp_host_alloc) for the copies to overlap.
 * Replaces the reference's synchronous per-epoch transfer_query_to_GPU /
 * execute_on_GPU sequence (src/scheduler.cpp:44-59).  After a batch reports
 * an error the pipeline must be drained and freed. */
typedef struct ltp_pipe ltp_pipe;
int ltp_pipe_create(ltp_ctx *ctx, uint32_t depth, uint64_t max_txns, uint64_t max_ops, ltp_pipe **out);
/* With LTP_PIPE_PERSISTENT every batch runs as one persistent-kernel launch
 * (no stage timing): fewer launches per batch, for small batches. */
#define LTP_PIPE_PERSISTENT 1u
int ltp_pipe_create2(ltp_ctx *ctx, uint32_t depth, uint64_t max_txns, uint64_t max_ops, uint32_t flags,
                     ltp_pipe **out);
int ltp_pipe_free(ltp_pipe *p);
/* Enqueues one batch (txn_first may be NULL for fixed-length transactions;
 * payload may be NULL).  commit_out / vals_out receive the results (either
 * may be NULL).  Blocks only while all slots are in flight.  *ticket numbers
 * the batch for ltp_pipe_wait. */
int ltp_pipe_submit(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                    const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                    uint8_t *commit_out, int32_t *vals_out, uint64_t *ticket);
/* The same with 32-bit keys (ltp_batch_load32). */
int ltp_pipe_submit32(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                      const uint32_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                      uint8_t *commit_out, int32_t *vals_out, uint64_t *ticket);
/* The same with the full 64-bit op values (the context must have an int64 column). */
int ltp_pipe_submit64(ltp_pipe *p, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn, uint64_t n_ops,
                      const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                      uint8_t *commit_out, int64_t *vals_out, uint64_t *ticket);
/* Waits until the ticket's results are in its host buffers; returns its status. */
int ltp_pipe_wait(ltp_pipe *p, uint64_t ticket, ltp_stats *stats);
/* LTP_OK when the ticket's results are ready, 1 while it is in flight. */
int ltp_pipe_poll(ltp_pipe *p, uint64_t ticket);

/* ---- serving loop --------------------------------------------------------- */
/* Continuous batching over a pipeline: client threads (or the built-in load
 * generator) submit transactions on numbered streams; a dispatcher thread
 * closes a batch when its oldest transaction has waited deadline_us, when
 * its read/write set reaches budget_bytes (12 bytes of key + opword per op)
 * or the slot capacity (max_txns, max_ops, 6 x max_ops payload slots), or -- work-conserving -- as soon as the device has
 * no batch queued; up to `depth` batches are in flight, so arrivals are
 * admitted while earlier batches execute.  Tables and conflict state stay
 * on the device.  Transactions aborted by the priority rule are re-queued
 * at the head of the next batch with their original arrival time (up to
 * max_attempts tries).  A stream's transactions enter batches in submission
 * order.  Latency = completion time - arrival time. */
#define LTP_SERVE_MAX_OPS 64
typedef struct {
    uint32_t deadline_us;   /* batch closes this long after its oldest arrival */
    uint32_t depth;         /* batches in flight (>= 2) */
    uint64_t budget_bytes;  /* read/write-set budget per batch */
    uint64_t max_txns;      /* slot capacity */
    uint64_t max_ops;
    uint32_t max_attempts;  /* tries before a transaction is reported aborted */
    uint32_t flags;         /* LTP_SERVE_EAGER | LTP_SERVE_KEEP_RESULTS */
} ltp_serve_config;
#define LTP_SERVE_EAGER 1u        /* close a batch as soon as the device has none queued */
#define LTP_SERVE_KEEP_RESULTS 2u /* keep per-transaction results for ltp_serve_poll */
#define LTP_SERVE_PERSISTENT 4u   /* execute each batch as one persistent-kernel launch */
#define LTP_SERVE_KEYS64 8u       /* request log: keep 64-bit keys even when every key fits 32 bits */
#define LTP_SERVE_JIT 16u         /* request log: queue the next batch only once the batch ahead is past its sort */

typedef struct {
    uint64_t tag;           /* caller's tag */
    uint64_t arrival_ns;    /* CLOCK_MONOTONIC */
    uint64_t done_ns;
    uint64_t batch_seq;     /* the batch that committed it (or last tried it) */
    uint32_t pos;           /* its position (TID) in that batch */
    uint32_t stream;
    uint32_t n_ops;
    uint32_t attempts;
    uint32_t committed;
    uint32_t pad;
    int64_t vals[LTP_SERVE_MAX_OPS]; /* op values (int32 cells sign-extended) */
} ltp_serve_result;

typedef struct {
    uint64_t submitted, completed, committed, aborted_attempts, batches;
    uint64_t closed_deadline, closed_budget, closed_idle, ops;
    double p50_us, p99_us, p999_us, mean_us, max_us;
    double elapsed_s, committed_per_s;
    /* where the host time goes: seconds the dispatcher spent forming and
     * submitting batches, seconds the completer spent on finished batches
     * (excluding its waits), and the share of load-generator submissions
     * made more than 100 us after their scheduled arrival */
    double dispatch_busy_s, complete_busy_s, loadgen_late_frac;
} ltp_serve_stats;

typedef struct ltp_server ltp_server;
int ltp_serve_open(ltp_ctx *ctx, const ltp_serve_config *cfg, ltp_server **out);
/* Thread-safe.  arrival_ns 0 = now.  Fails with LTP_E_CAPACITY when n_ops
 * exceeds LTP_SERVE_MAX_OPS or the slot capacity. */
int ltp_serve_submit(ltp_server *s, uint32_t stream, uint32_t n_ops, const uint64_t *keys, const uint32_t *opw,
                     uint64_t tag, uint64_t arrival_ns);
/* The same for a transaction with inserts: each insert op's key is an offset
 * into this transaction's own payload (n_payload int32 slots). */
int ltp_serve_submit_rows(ltp_server *s, uint32_t stream, uint32_t n_ops, const uint64_t *keys, const uint32_t *opw,
                          uint32_t n_payload, const int32_t *payload, uint64_t tag, uint64_t arrival_ns);
/* Moves up to max completed transactions into out; *n = how many. */
int ltp_serve_poll(ltp_server *s, ltp_serve_result *out, uint32_t max, uint32_t *n);
/* Open-loop Poisson load: n_streams clients at `rate` transactions/s in
 * aggregate for `seconds`, drawing transactions round-robin from the given
 * pool, on n_threads generator threads.  Returns when the offered load ends;
 * completions keep arriving until ltp_serve_close. */
int ltp_serve_loadgen(ltp_server *s, double rate, double seconds, uint32_t n_streams, uint64_t seed,
                      const uint32_t *txn_first, uint64_t n_pool, const uint64_t *keys, const uint32_t *opw,
                      uint32_t n_threads);
/* The same over a pool with inserts: transaction k's payload is
 * payload[pay_first[k] .. pay_first[k+1]) and its insert keys are offsets
 * into the whole payload array. */
int ltp_serve_loadgen_rows(ltp_server *s, double rate, double seconds, uint32_t n_streams, uint64_t seed,
                           const uint32_t *txn_first, uint64_t n_pool, const uint64_t *keys, const uint32_t *opw,
                           const uint64_t *pay_first, const int32_t *payload, uint32_t n_threads);
/* Statistics so far (latency percentiles over committed transactions). */
int ltp_serve_stats_now(ltp_server *s, ltp_serve_stats *st);
/* Drains every admitted transaction, stops the dispatcher, frees. */
int ltp_serve_close(ltp_server *s, ltp_serve_stats *st);
/* Current CLOCK_MONOTONIC time in ns (the clock arrivals are stamped with). */
uint64_t ltp_now_ns(void);
/* Arrival times (ns after the start, non-decreasing) of n requests of an
 * open-loop Poisson process at `rate` requests/s -- the merged arrivals of
 * any number of independent Poisson client streams whose rates sum to
 * `rate` -- drawn from `seed` on n_threads threads (<= 0: all hardware
 * threads); for ltp_ingest_run. */
int ltp_poisson_arrivals(uint64_t n, double rate, uint64_t seed, uint64_t *arrival_ns, int n_threads);

/* ---- serving from a device-resident request log --------------------------
 * Requests are already in HBM when they arrive -- the way a NIC writing by
 * GPUDirect RDMA places them -- and carry arrival times; the host touches no
 * request.  One host thread admits, by the clock, every request whose arrival
 * time has passed, closes batches with the rules of ltp_serve_config
 * (deadline, max_txns / max_ops / 6 x max_ops payload slots, read/write-set
 * budget, LTP_SERVE_EAGER), keeps `depth` batches in flight, and re-queues
 * transactions the priority rule aborted at the head of the next batch it
 * closes (up to max_attempts tries).  A batch of new requests only, at most
 * n_pool of them, executes in place from the log: the log's keys and
 * opwords are stored twice back to back, so a window that wraps the pool is
 * contiguous.  Other batches (re-queued transactions first, then the newly
 * arrived requests in arrival order) are gathered on the device.  Keys travel
 * as 32-bit keys when every key of the pool fits (unless LTP_SERVE_KEYS64);
 * a pool whose transactions all have the same op count runs fixed-length
 * batches.  Latency = the host time the batch was seen complete - arrival
 * time.
 *
 * The log is a pool of n_pool transactions (txn_first[n_pool + 1] op
 * offsets; optional payload as in ltp_serve_loadgen_rows); request i of a run
 * is pool transaction i mod n_pool. */
typedef struct ltp_ingest ltp_ingest;
int ltp_ingest_open(ltp_ctx *ctx, const ltp_serve_config *cfg, uint64_t n_pool, const uint32_t *txn_first,
                    const uint64_t *keys, const uint32_t *opw, const uint64_t *pay_first, const int32_t *payload,
                    ltp_ingest **out);
/* Serves n_txns requests; arrival_ns[i] = request i's arrival, in ns after
 * the run's start (non-decreasing).  Returns when every request is committed
 * or has used its tries.  Tables keep the effects; a later run continues. */
int ltp_ingest_run(ltp_ingest *g, uint64_t n_txns, const uint64_t *arrival_ns, ltp_serve_stats *st);
/* Per request of the last run (any pointer may be NULL): committed flag,
 * the batch that executed its last try and its position (TID) there, tries.
 * vals (int64, one per op of requests 0..n_txns-1 in log order) needs
 * LTP_SERVE_KEEP_RESULTS and n_txns <= n_pool. */
int ltp_ingest_results(ltp_ingest *g, uint8_t *committed, uint64_t *batch_seq, uint32_t *pos, uint32_t *attempts,
                       int64_t *vals);
int ltp_ingest_close(ltp_ingest *g);

/* ---- pinned host memory ------------------------------------------------ */
void *ltp_host_alloc(size_t bytes);
void ltp_host_free(void *p);

/* ---- seeded workload generator (host; Txn_Generator<YCSB_*> +
 *      Query::generate_txn, src/txn_generator.cpp:601-673,
 *      src/query.cpp:270-311, made seedable) ---------------------------- */
/* Returns the op count, or UINT64_MAX when cap_ops is too small or the
 * parameters are invalid.  n_threads <= 0: all hardware threads. */
uint64_t ltp_gen_ycsb(const ltp_ycsb_params *p, uint64_t batch, uint64_t n_txns, uint32_t *txn_first, uint64_t *keys,
                      uint32_t *opw, uint64_t cap_ops, int n_threads);
int32_t ltp_table_value(uint64_t seed, uint64_t row, uint32_t col, uint32_t n_cols);

/* ---- TPC-C-shaped order-entry workload (new-order / payment) ----------
 * Nine tables with the reference's TPC-C schema (data/TPCC.json) made
 * columnar: ids and counts int32, money int64 cents, tax and discount int32
 * basis points, every 24-byte text field six int32 columns.  The op shapes
 * follow the reference's TPC-C op expansion (parse<Neworder_Query>,
 * cuda/src/gpuquery.cu:2474-2606: 5 + 3 per order line; parse<Payment_Query>,
 * gpuquery.cu:2608-2734: 7), with the TPC-C input distributions (NURand
 * customers and items, 1% remote order lines, 15% remote payments, 60% of
 * payments by last name) in place of the reference's uniform draws
 * (src/txn_generator.cpp:231-381).
 *  new-order: READ W_TAX; RMW D_NEXT_O_ID += 1 (its output is the order id);
 *    READ C_DISCOUNT; INSERT new-order and order rows linked to the order
 *    id; per line: INSERT order-line (linked), RMW S_QUANTITY -= qty,
 *    RMW S_YTD += qty.
 *  payment: RMW W_YTD += amount; RMW D_YTD += amount; READ C_CREDIT;
 *    RMW C_BALANCE -= amount; RMW C_YTD_PAYMENT += amount;
 *    RMW C_PAYMENT_CNT += 1; INSERT history.
 * A payment by last name resolves the customer on the host through the
 * static last-name index (the middle customer by id among those with the
 * name), as the reference resolves it from its index (gpuquery.cu:2641-2650;
 * index built at src/database.cpp:310-393).  D_NEXT_O_ID holds the last order
 * id issued.  S_QUANTITY is decremented without TPC-C's +91 wrap. */
#define LTP_TPCC_N_TABLES 9
enum {
    LTP_TPCC_WAREHOUSE = 0, LTP_TPCC_DISTRICT, LTP_TPCC_CUSTOMER, LTP_TPCC_HISTORY, LTP_TPCC_NEW_ORDER,
    LTP_TPCC_ORDER, LTP_TPCC_ORDER_LINE, LTP_TPCC_ITEM, LTP_TPCC_STOCK
};
/* column indices (a 24-byte text field LTPC_X occupies LTPC_X .. LTPC_X+5) */
enum { LTPC_W_ID = 0, LTPC_W_TAX, LTPC_W_YTD, LTPC_W_NAME, LTPC_W_NCOLS = LTPC_W_NAME + 6 };
enum { LTPC_D_ID = 0, LTPC_D_W_ID, LTPC_D_TAX, LTPC_D_YTD, LTPC_D_NEXT_O_ID, LTPC_D_NAME, LTPC_D_NCOLS = LTPC_D_NAME + 6 };
enum {
    LTPC_C_ID = 0, LTPC_C_D_ID, LTPC_C_W_ID, LTPC_C_LAST, LTPC_C_CREDIT, LTPC_C_DISCOUNT, LTPC_C_BALANCE, LTPC_C_YTD_PAYMENT, LTPC_C_PAYMENT_CNT,
    LTPC_C_DELIVERY_CNT, LTPC_C_DATA, LTPC_C_NCOLS = LTPC_C_DATA + 6
};
enum { LTPC_H_C_ID = 0, LTPC_H_C_D_ID, LTPC_H_C_W_ID, LTPC_H_D_ID, LTPC_H_W_ID, LTPC_H_AMOUNT, LTPC_H_DATA, LTPC_H_NCOLS = LTPC_H_DATA + 6 };
enum { LTPC_NO_O_ID = 0, LTPC_NO_D_ID, LTPC_NO_W_ID, LTPC_NO_NCOLS };
enum { LTPC_O_ID = 0, LTPC_O_D_ID, LTPC_O_W_ID, LTPC_O_C_ID, LTPC_O_OL_CNT, LTPC_O_ALL_LOCAL, LTPC_O_CARRIER_ID, LTPC_O_NCOLS };
enum {
    LTPC_OL_O_ID = 0, LTPC_OL_D_ID, LTPC_OL_W_ID, LTPC_OL_NUMBER, LTPC_OL_I_ID, LTPC_OL_SUPPLY_W_ID, LTPC_OL_QUANTITY, LTPC_OL_AMOUNT, LTPC_OL_DIST_INFO,
    LTPC_OL_NCOLS = LTPC_OL_DIST_INFO + 6
};
enum { LTPC_I_ID = 0, LTPC_I_IM_ID, LTPC_I_PRICE, LTPC_I_NAME, LTPC_I_NCOLS = LTPC_I_NAME + 6 };
enum { LTPC_S_I_ID = 0, LTPC_S_W_ID, LTPC_S_QUANTITY, LTPC_S_YTD, LTPC_S_ORDER_CNT, LTPC_S_REMOTE_CNT, LTPC_S_DIST, LTPC_S_NCOLS = LTPC_S_DIST + 6 };

typedef struct {
    uint64_t seed;
    uint32_t warehouses;     /* W */
    uint32_t districts;      /* per warehouse (10) */
    uint32_t customers;      /* per district (3000) */
    uint32_t items;          /* items, and stock rows per warehouse (100000) */
    uint32_t ol_min, ol_max; /* order lines per new-order (5, 15) */
    double new_order_frac;   /* 0.5 */
    double remote_line;      /* 0.01: a line's supply warehouse is another one */
    double remote_payment;   /* 0.15: the paying customer is another warehouse's */
    double by_last_name;     /* 0.6: payment names the customer by last name */
} ltp_tpcc_params;

typedef struct ltp_tpcc ltp_tpcc;
/* Validates the parameters and builds the last-name index. */
int ltp_tpcc_create(const ltp_tpcc_params *p, ltp_tpcc **out);
void ltp_tpcc_free(ltp_tpcc *g);
/* Schema (n_cols, wide_cols) and initial row count of one table; the
 * insert-only tables (history, new-order, order, order-line) start empty. */
int ltp_tpcc_table(const ltp_tpcc *g, uint32_t table, ltp_schema *schema, uint64_t *rows);
/* Initial values of rows [row0, row0+n) of one column, at the column's width. */
int ltp_tpcc_column(const ltp_tpcc *g, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, void *dst);
/* Generates batch `batch` of n_txns transactions (TID = position).  With
 * keys == NULL only the sizes are computed.  pay_first[n_txns+1] (may be
 * NULL) receives where each transaction's payload starts; n_new_order (may
 * be NULL) the new-order count; inserts[LTP_TPCC_N_TABLES] (may be NULL) the
 * rows each table gains.  Returns LTP_OK or LTP_E_CAPACITY. */
int ltp_tpcc_gen(const ltp_tpcc *g, uint64_t batch, uint64_t n_txns, uint32_t *txn_first, uint64_t *keys,
                 uint32_t *opw, uint64_t cap_ops, int32_t *payload, uint64_t cap_payload, uint64_t *pay_first,
                 uint64_t *n_ops, uint64_t *n_payload, uint64_t *n_new_order, uint64_t *inserts, int n_threads);

/* ---- tuning --------------------------------------------------------------- */
typedef struct {
    uint32_t block;      /* threads per block of the streaming kernels: 128, 256, 512 */
    uint32_t ipt;        /* ops per thread per tile: 1, 2, 4, 8 */
    uint32_t word_bits;  /* conflict-word granularity: 32 or 64 cells per word (64 needs block x ipt <= 2048;
                          * the persistent kernel always uses 32) */
    uint32_t flags;      /* LTP_TUNE_* */
} ltp_tuning;
/* The mark kernel reads a conflict word it touched more than once in a tile
 * before its atomics and skips those whose bits are already set: a win when
 * a few words are hot in every tile (order-entry warehouse and district
 * rows), a loss when repeated words are still filling up (Zipf tails). */
#define LTP_TUNE_MARK_PRECHECK 1u
/* Tuning used for batches whose op count falls in size bucket floor(log2(ops)). */
int ltp_set_tuning(ltp_ctx *ctx, uint32_t bucket, const ltp_tuning *t);
int ltp_get_tuning(ltp_ctx *ctx, uint32_t bucket, ltp_tuning *t);

/* Turns per-kernel event timing on or off for later executions (batches
 * created while the context had LTP_FLAG_STAGE_TIMING carry the events). */
int ltp_set_stage_timing(ltp_ctx *ctx, int32_t on);

/* ---- failure injection for tests (host-side; no GPU fault) ------------- */
/* While set, the next execute's first stage polls a flag that nothing sets,
 * gives up after about `ms` milliseconds and the batch reports LTP_E_TIMEOUT;
 * the context stays usable. */
int ltp_debug_stall_next(ltp_ctx *ctx, uint32_t ms);

/* ---- execution without allocation -------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- their process hands all of it to another allocator or reserves
 * it up front, or an allocation could stall a latency-critical path -- this
 * runs one batch against ONE column-major int32 table that the caller owns
 * (table[col * rows_cap + row]), with the batch arrays, op values and
 * commit vector all in caller-provided device memory, and calls no
 * cudaMalloc, cudaFree or allocating library routine.  All scratch lives in
 * one fixed array of LTP_NOALLOC_SCRATCH_BYTES inside the library image,
 * which every GPU that loads the library holds until the process exits.
 * Limits: n_ops <= LTP_NOALLOC_MAX_OPS and n_rows * n_cols <=
 * LTP_NOALLOC_MAX_CELLS, else LTP_E_CAPACITY.  The first call on a device
 * looks the array's device address up (make that first call before any
 * stream capture).  Every call shares the array and clears what it needs at
 * its start; calls that overlap on the GPU race, so serialise them.  The
 * call waits for its stream and returns the batch's status.  Semantics and
 * outputs equal ltp_batch_execute's for the same rule and inputs (reads and
 * read-modify-writes; the call takes no insert payload).  txn_first (device
 * memory, n_txns + 1 entries, or NULL for ops_per_txn ops per transaction)
 * must start at 0, never decrease and end at n_ops: it is checked on the
 * device, and a malformed one makes the call return LTP_E_BADARG with the
 * table untouched.  rows_cap is at most 2^48.  The cached device address of
 * the array goes stale after a cudaDeviceReset of its device: do not call
 * this entry point on that device again in the same process. */
#define LTP_NOALLOC_MAX_OPS (1ull << 18)
#define LTP_NOALLOC_MAX_CELLS (1ull << 23)
#define LTP_NOALLOC_SCRATCH_BYTES 18173696ull
int ltp_execute_noalloc(int32_t device, int32_t rule, int32_t *table, uint64_t rows_cap, uint64_t n_rows,
                        uint32_t n_cols, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                        uint64_t n_ops, const uint64_t *keys, const uint32_t *opw, int32_t *out, uint8_t *commit,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif
