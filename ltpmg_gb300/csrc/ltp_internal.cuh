// ltp_internal.cuh -- device-side data layout shared by the kernels and the
// C-ABI layer of the batched transaction-processing hot path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ltpmg_gb300.h"

namespace ltp {

typedef unsigned long long u64;
typedef unsigned int u32;

// opword fields (same layout as LTP_OPW in the public header)
__host__ __device__ __forceinline__ u32 opw_kind(u32 w) { return w & 3u; }
__host__ __device__ __forceinline__ u32 opw_col(u32 w) { return (w >> 2) & 63u; }
__host__ __device__ __forceinline__ u32 opw_table(u32 w) { return (w >> 8) & 15u; }
__host__ __device__ __forceinline__ int32_t opw_imm(u32 w) { return ((int32_t)w) >> 12; }

// One column-store table.  Columns are int32, or int64 where bit c of
// `wide` is set; column c starts at byte col_off(c) = rows_cap * (4c + 4 *
// (wide columns before c)) and row r of it at col_off(c) + r * width(c).
// Cells are numbered row-major within a table (cell_base + r * n_cols + c) so
// that the cells of one row share a bitmap word.
struct TableDev {
    char *data;
    u64 rows_cap;   // column stride (rows allocated, padded)
    u64 row_limit;  // rows the table may grow to (requested capacity)
    u64 n_rows;
    u64 cell_base;
    u64 wide;       // bit c: column c holds int64
    u32 n_cols;
    u32 pad;
};

__host__ __device__ __forceinline__ u64 col_off(const TableDev &t, u32 c) {
    const u64 below = c ? (t.wide & ((1ull << c) - 1ull)) : 0ull;
#ifdef __CUDA_ARCH__
    const u32 nw = __popcll(below);
#else
    const u32 nw = (u32)__builtin_popcountll(below);
#endif
    return t.rows_cap * (4ull * c + 4ull * nw);
}
__host__ __device__ __forceinline__ bool col_wide(const TableDev &t, u32 c) { return (t.wide >> c) & 1ull; }

struct TablesDev {
    TableDev t[LTP_MAX_TABLES];
    u64 *rows_now;  // [LTP_MAX_TABLES] device-resident row counts (grow with inserts)
    u32 n;
    u32 any_wide;   // some table has an int64 column
};

// Device view of one loaded batch.
struct BatchDev {
    const u64 *keys;       // [n_ops] (null when the batch carries 32-bit keys)
    const u32 *keys32;     // [n_ops] 32-bit keys (null when the batch carries 64-bit keys)
    const u32 *opw;        // [n_ops]
    const u32 *txn_first;  // [n_txns + 1]
    const u32 *op_txn;     // [n_ops] transaction of each op (variable-length batches)
    int32_t *out;          // [n_ops] value after each op (low 32 bits for int64 cells)
    long long *out64;      // [n_ops] full value, when the context has int64 columns (else null); the
                           // kernels fill it for ops on int64 cells, launch_widen_out for the rest
    uint8_t *commit;       // [n_txns]
    const int32_t *payload;  // insert row images (LTP_OP_INSERT keys index it)
    u64 payload_len;
    u64 n_ops;
    u64 n_txns;
    u32 ops_per_txn;       // > 0: fixed-length transactions (op_txn unused)
    u32 flags;             // LTP_TUNE_* flags of the batch's size bucket
};

constexpr int kMaxPasses = 4;

// Look-back status slots of the kernels that use decoupled look-back.
enum TileSlot { SLOT_CLASSIFY = 0, SLOT_SORT0 = 1, SLOT_APPLY = 5, SLOT_INSERT = 6, N_SLOTS = 7 };

// Per-batch device counters; zeroed by the host before every batch.
struct Counters {
    u64 n_tw;          // touched bitmap words
    u64 n_c;           // contended ops
    u64 bad_op;        // ~(lowest index of a malformed op); 0: none
    u64 committed;
    u32 M;             // contended cells
    int err;           // first device-side error status (LTP_E_*), 0 = none
    u32 tile_ctr[N_SLOTS];
    u32 hist[kMaxPasses][256];  // radix digit histograms of the contended list
    u32 stall;         // polled by the debug stall kernel; never set
    u32 dense;         // set by mark when it built no touched-word list: ids and finish visit every word of the range below
    u32 wlo_inv;       // ~(lowest conflict word mark touched); 0: none
    u32 whi1;          // highest conflict word mark touched + 1; 0: none
    u32 wide_ops;      // set by mark when some valid op is on an int64 cell
    u32 ins_total[LTP_MAX_TABLES];      // insert ops per table in the batch
    u32 ins_committed[LTP_MAX_TABLES];  // committed inserts per table
};

// Conflict state of 32 consecutive cells, kept together so that building,
// scanning, reading and clearing it touches one 16-byte sector per word.
struct __align__(16) WordState {
    u32 touch;   // cell touched at least once in the batch
    u32 wbits;   // cell written (RMW) at least once
    u32 multi;   // cell touched at least twice
    u32 pad;     // keeps a word to one 16-byte access (the dense ids live in Scratch::cview)
};

// Scratch owned by the context, sized by the cell space and the batch capacity.
struct Scratch {
    WordState *words; // [n_words]
    uint2 *cview;     // [n_words + 1] per 32 cells {contended mask, first dense id} (16 B per 64-cell word)
    u32 *tw_list;   // [cap_ops] touched words
    u64 *list[2];   // [cap_ops] contended-op records, ping-pong for the sort
    u64 *dcell;     // [cap_ops] cell of each contended-cell id
    long long *dbase; // [cap_ops] value of each contended cell before the batch
    u32 *dminw;     // [cap_ops] smallest writer TID of each contended cell (priority rule)
    u32 *st_sort[2];// [tiles * 256] radix look-back status
    u64 *st_cls;    // [tiles] classify look-back status (dense record offsets)
    u64 *st_apply;  // [tiles] segmented-apply look-back status
    u32 *st_ins;    // [tiles * LTP_MAX_TABLES] insert-slot look-back status
    u32 *ins_pre;   // [tiles * LTP_MAX_TABLES] per insert tile and table: insert ops (mark), then their exclusive prefix
    u64 n_words;
    u64 cap_ops;
    u64 cap_tiles;  // tiles of the smallest look-back tile size at cap_ops
    u64 cap_sort_tiles;
};

constexpr u32 kSortBlock = 256;
constexpr u32 kSortIpt = 12;
constexpr u32 kSortTile = kSortBlock * kSortIpt;
constexpr u32 kIdsBlock = 256;
constexpr u32 kIdsIpt = 8;
constexpr u32 kIdsTile = kIdsBlock * kIdsIpt;
constexpr u32 kApplyBlock = 256;
constexpr u32 kApplyIpt = 8;
constexpr u32 kApplyTile = kApplyBlock * kApplyIpt;
constexpr u32 kMinTile = 128;  // smallest classify tile (block 128 x 1 op)
constexpr u32 kInsBlock = 512;
constexpr u32 kInsIpt = 8;
constexpr u32 kInsTile = kInsBlock * kInsIpt;
constexpr u32 kInsSmem = kInsTile * (4 + 8 + 1);  // insert staging: payload offset, link value, link column

struct Tuning {
    u32 block, ipt, word_bits, flags;
};

// Host-side launch plan for one batch.
struct Launch {
    cudaStream_t stream;
    int num_sms;
    int rule;
    Tuning tune;
    bool stall;
    u32 stall_ms;
    cudaEvent_t *ev;  // LTP_N_STAGES events of the batch when timing
    bool timing;
    cudaEvent_t progress = nullptr;  // recorded after stage progress_stage (the serving loop's "nearly done")
    int progress_stage = 0;
    bool pdl = false;  // programmatic dependent launch (set by launch_execute for uncaptured streams)
};

// Kernel launch wrappers (ltp_kernels.cu).  Each returns the CUDA status of
// its launches.
cudaError_t launch_execute(const Launch &L, const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr);
// Is (threads per block, ops per thread, conflict-word bits) a built tiling?
bool tiling_supported(int block, int ipt, int word_bits);
cudaError_t launch_reset_scratch(cudaStream_t st, const Scratch &s);
cudaError_t launch_fill_seeded(cudaStream_t st, const TableDev &t, u64 seed);
cudaError_t launch_expand_op_txn(cudaStream_t st, const u32 *txn_first, u64 n_txns, u32 *op_txn);
// The same for a txn_first the host has not checked: a malformed one sets
// ctr->err = LTP_E_BADARG (the batch's kernels then do nothing) and no write
// leaves op_txn[0, n_ops).
cudaError_t launch_expand_op_txn_checked(cudaStream_t st, const u32 *txn_first, u64 n_txns, u64 n_ops, u32 *op_txn,
                                         Counters *ctr);
// Completes out64 after execution (ops on int32 cells write only out).
cudaError_t launch_widen_out(cudaStream_t st, const BatchDev &b, const TablesDev &T);
cudaError_t launch_set_u64(cudaStream_t st, u64 *dst, u64 value);
// One cooperative launch over n_batches device-resident batch descriptors.
cudaError_t launch_persistent(cudaStream_t st, int num_sms, int rule, const BatchDev *d_batches,
                              Counters *const *d_snaps, u32 n_batches, const TablesDev &T, const Scratch &s,
                              Counters *ctr, u32 *bar);
int persistent_grid(int num_sms);

}  // namespace ltp
