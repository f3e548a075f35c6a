/*
 * ltp_oracle.h -- CPU oracle for the batched transaction-processing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, and only as the checker / CPU baseline.
 *
 * Parity status: the execution rule is a restatement of the reference's
 * per-row ascending-TID order (cuda/src/gpulauncher.cu:382-418 register_cc,
 * :2439-2523 filter_commit, :2525-2671 commit).  The reference ships no golden
 * vectors or known-answer tests for this path and its operators never write
 * (gpulauncher.cu:79-103), so value-level parity of the replay is UNPINNED by
 * the reference itself.  The reference-compatible generator pieces
 * (truncated "zipf" CDF and sampler of src/random.cpp:105-161, NURand of
 * src/random.cpp:58-60, YCSB op expansion of cuda/src/gpuquery.cu:2929-3303)
 * are pinned against the reference's own host code compiled under oracle/_ref
 * (see oracle/build_ref.sh) through the fixtures in tests/golden/.
 */
#ifndef LTP_ORACLE_H
#define LTP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* opword layout (identical to the library's LTP_OPW_* macros):
 *   bits 0-1  kind   0 = read, 1 = read-modify-write add, 2 = insert
 *   bits 2-7  column
 *   bits 8-11 table
 *   bits 12-31 signed 20-bit immediate (the RMW delta) */
#define LTPO_KIND(w) ((w) & 3u)
#define LTPO_COL(w) (((w) >> 2) & 63u)
#define LTPO_TABLE(w) (((w) >> 8) & 15u)
#define LTPO_IMM(w) (((int32_t)(w)) >> 12)
#define LTPO_OPW(kind, col, table, imm) \
    ((uint32_t)(kind) | ((uint32_t)(col) << 2) | ((uint32_t)(table) << 8) | ((uint32_t)(imm) << 12))

/* ---- seeded primitives ---------------------------------------------- */
uint64_t ltpo_mix64(uint64_t x);
uint64_t ltpo_stream_seed(uint64_t seed, uint64_t batch, uint64_t txn);
uint64_t ltpo_feistel_perm(uint64_t seed, uint64_t n, uint64_t x);
double ltpo_det_log(double x);
double ltpo_det_exp(double x);
uint64_t ltpo_zipf_draw(uint64_t n, double theta, uint64_t *state);
int32_t ltpo_table_value(uint64_t seed, uint64_t row, uint32_t col, uint32_t n_cols);

/* ---- YCSB-style batch generator ------------------------------------- */
typedef struct {
    uint64_t seed;
    uint64_t n_rows;
    uint32_t n_cols;
    uint32_t ops_min;     /* ops per txn drawn uniformly in [ops_min, ops_max] */
    uint32_t ops_max;
    int32_t rmw_delta;    /* immediate of every RMW op (+1 for the YCSB shapes) */
    double read_frac;     /* probability that an op is a read */
    double theta;         /* 0 = uniform keys, else Zipf(theta) over a seeded permutation */
} ltpo_ycsb_params;

/* Writes txn_first[0..n_txns] and keys/opw for every op; returns the op count,
 * or UINT64_MAX when cap_ops is too small. */
uint64_t ltpo_gen_ycsb_batch(const ltpo_ycsb_params *p, uint64_t batch, uint64_t n_txns,
                             uint32_t *txn_first, uint64_t *keys, uint32_t *opw, uint64_t cap_ops);

/* Fills a column-major int32 table: tab[col * n_rows + row]. */
void ltpo_table_init(uint64_t seed, uint64_t n_rows, uint32_t n_cols, int32_t *tab);

/* ---- serial replay executor ----------------------------------------- */
/* rule 0 (R0): every op on a cell runs in ascending (TID, op) order; all
 *              transactions commit.  This is the reference's rule.
 * rule 1 (R1): a transaction aborts when a smaller TID has an RMW/insert on a
 *              cell it reads or writes; committed ones replay serially.
 * out[i] is the cell value right after op i (the value read, or the value
 * the RMW produced); 0 for ops of aborted transactions.
 * Returns 0, or -1 on a malformed batch (key out of range, bad column). */
int ltpo_replay(int rule, uint64_t n_rows, uint32_t n_cols, int32_t *tab, uint64_t n_txns,
                const uint32_t *txn_first, const uint64_t *keys, const uint32_t *opw,
                uint8_t *commit, int32_t *out);

/* Same rule-0 replay split over n_threads threads by cell (each thread scans
 * the batch in order and applies the ops of the cells it owns).  Used as the
 * multi-core CPU baseline; results equal ltpo_replay(0, ...). */
int ltpo_replay_r0_mt(uint64_t n_rows, uint32_t n_cols, int32_t *tab, uint64_t n_txns,
                      const uint32_t *txn_first, const uint64_t *keys, const uint32_t *opw,
                      uint8_t *commit, int32_t *out, int n_threads);

/* Multi-table replay with inserts, int32 and int64 columns.  Column c of a
 * table is the array cols[c] of rows_cap values, int64 where bit c of `wide`
 * is set, else int32; cell arithmetic wraps at the column's width.  Keys of
 * reads/RMWs must be < n_rows as of the batch start.  An insert op (kind 2)
 * appends a row to its table: slot = the table's next row (committed
 * inserts only, in (TID, op) order); its values come from payload[key ..]:
 * one int32 slot per int32 column, two (low word first) per int64 column;
 * out = slot.  A linked insert (low 10 bits of the immediate = d > 0) sets
 * column `col` of the new row to out[i - d], which must be a read or RMW of
 * the same transaction.  Each table's n_rows is advanced by its committed
 * inserts.  out holds each op's full value.
 * Returns 0, -1 on a malformed batch, -2 when an insert exceeds rows_cap. */
typedef struct {
    void **cols;
    uint64_t rows_cap;
    uint64_t n_rows;
    uint32_t n_cols;
    uint32_t pad;
    uint64_t wide;
} ltpo_table;

int ltpo_replay_tables(int rule, uint32_t n_tables, ltpo_table *tables, uint64_t n_txns, const uint32_t *txn_first,
                       const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                       uint8_t *commit, int64_t *out);

/* The ordered rule of ltpo_replay_tables on n_threads threads (reads and
 * RMWs split by cell, inserts by table); same results as rule 0 there. */
int ltpo_replay_tables_r0_mt(uint32_t n_tables, ltpo_table *tables, uint64_t n_txns, const uint32_t *txn_first,
                             const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                             uint8_t *commit, int64_t *out, int n_threads);

/* 64-bit FNV-1a over a byte range (table / result fingerprints). */
uint64_t ltpo_fnv1a(const void *data, uint64_t bytes);

/* ---- restatements of the reference's own generator pieces ------------ */
/* src/random.cpp:105-137: cumulative table of the first min(n,100) ranks of
 * a Zipf(s) law normalised over n ranks; returns the entry count. */
uint32_t ltpo_ref_zipf_table(uint64_t n, double s, double *cdf_out);
/* src/random.cpp:140-161: sample given the two rand()-style draws the
 * reference consumes (r100 = rand_test(0,99), tail = rand_test(100,b)). */
uint32_t ltpo_ref_zipf_pick(const double *cdf, uint32_t len, uint32_t r100, uint32_t tail);
/* src/random.cpp:58-60 NURand on top of two uniform draws. */
uint64_t ltpo_ref_nurand(uint64_t A, uint64_t x, uint64_t y, uint64_t r_a, uint64_t r_xy);
/* cuda/src/gpuquery.cu:2929-3303: kind of op i (0 select, 2 update, 4 scan,
 * 1 insert) in a YCSB_A..E query (variant 0..4). */
uint32_t ltpo_ref_ycsb_op_type(uint32_t variant, uint32_t i);

#ifdef __cplusplus
}
#endif
#endif
