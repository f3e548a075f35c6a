// ltp_noalloc.cu -- batch execution that allocates no memory.
//
// Some callers cannot call cudaMalloc: code that runs while the device's
// memory is owned by another allocator (a host database's own pool, a
// framework caching allocator that must account every byte), code that runs
// where an allocation could stall or fail at an unacceptable moment (inside
// a latency-critical serving path, or after memory has been fully reserved
// up front), and plug-ins whose host process forbids allocation by contract.
// ltp_execute_noalloc serves them: the caller passes its own device buffers
// for the table, the batch and the outputs, and every byte of scratch the
// kernels need comes from one file-scope device array of fixed size that the
// library image carries (every GPU that loads the library holds it until the
// process exits).
//
// The array is shared by every call on a device and keeps the last call's
// contents, so each call first clears what must start at zero.  Calls that
// overlap on the GPU (two streams, or two host threads) race on it; callers
// must serialise them.  The array's device address is looked up once per
// device and cached: after a cudaDeviceReset of that device the cached
// address is stale, so the entry point must not be used on it again in the
// same process.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "ltp_internal.cuh"

using namespace ltp;

namespace {

constexpr u64 kNaMaxOps = LTP_NOALLOC_MAX_OPS;
constexpr u64 kNaMaxCells = LTP_NOALLOC_MAX_CELLS;
// n_words = cells / 32 + 1 at most, plus the spare entry the 64-cell layout
// and the reset use (the allocating path allocates words + 1 as well)
constexpr u64 kNaWords = kNaMaxCells / 32 + 2;
constexpr u64 kNaTiles = kNaMaxOps / kMinTile + 2;
constexpr u64 kNaMaxRowsCap = 1ull << 48;
constexpr u64 kNaSortTiles = kNaMaxOps / kSortTile + 2;

constexpr u64 align256(u64 x) { return (x + 255) & ~255ull; }

// byte offsets of the scratch regions inside the static array
constexpr u64 kOffWords = 0;
constexpr u64 kOffView = kOffWords + align256(kNaWords * sizeof(WordState));
constexpr u64 kOffTw = kOffView + align256(kNaWords * sizeof(uint2));
constexpr u64 kOffList0 = kOffTw + align256(kNaMaxOps * 4);
constexpr u64 kOffList1 = kOffList0 + align256(kNaMaxOps * 8);
constexpr u64 kOffDcell = kOffList1 + align256(kNaMaxOps * 8);
constexpr u64 kOffDbase = kOffDcell + align256(kNaMaxOps * 8);
constexpr u64 kOffDminw = kOffDbase + align256(kNaMaxOps * 8);
constexpr u64 kOffOpTxn = kOffDminw + align256(kNaMaxOps * 4);
constexpr u64 kOffSort0 = kOffOpTxn + align256(kNaMaxOps * 4);
constexpr u64 kOffSort1 = kOffSort0 + align256(kNaSortTiles * 256 * 4);
constexpr u64 kOffCls = kOffSort1 + align256(kNaSortTiles * 256 * 4);
constexpr u64 kOffApply = kOffCls + align256(kNaTiles * 8);
constexpr u64 kOffIns = kOffApply + align256(kNaTiles * 8);
constexpr u64 kOffRows = kOffIns + align256(kNaTiles * LTP_MAX_TABLES * 4);
constexpr u64 kOffCtr = kOffRows + align256(LTP_MAX_TABLES * 8);
constexpr u64 kScratchBytes = kOffCtr + align256(sizeof(Counters));

static_assert(kScratchBytes == LTP_NOALLOC_SCRATCH_BYTES, "header and layout disagree on the scratch size");

}  // namespace

// The scratch itself.  In host code this name is only a host-side stand-in
// for the symbol, never a device address: the device address is looked up
// per device with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_dev_ptr[kMaxDevices] = {};
int g_dev_sms[kMaxDevices] = {};

// Once per device, with that device current: the array's device address and
// the SM count.  No allocation happens here.
int setup_device(int device, unsigned char **ptr, int *sms) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_dev_ptr[device]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LTP_E_CUDA;
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return LTP_E_CUDA;
        g_dev_ptr[device] = (unsigned char *)p;
        g_dev_sms[device] = n;
    }
    *ptr = g_dev_ptr[device];
    *sms = g_dev_sms[device];
    return LTP_OK;
}

}  // namespace

extern "C" int ltp_execute_noalloc(int32_t device, int32_t rule, int32_t *table, uint64_t rows_cap, uint64_t n_rows,
                                   uint32_t n_cols, uint64_t n_txns, const uint32_t *txn_first, uint32_t ops_per_txn,
                                   uint64_t n_ops, const uint64_t *keys, const uint32_t *opw, int32_t *out,
                                   uint8_t *commit, void *stream) {
    if (rule != LTP_RULE_ORDERED && rule != LTP_RULE_PRIORITY) return LTP_E_BADARG;
    if (device < 0 || device >= kMaxDevices || !table || n_cols == 0 || n_cols > LTP_MAX_COLS || n_rows > rows_cap)
        return LTP_E_BADARG;
    // column offsets are rows_cap * 4 * col bytes: keep them far from wrapping
    if (rows_cap > kNaMaxRowsCap) return LTP_E_BADARG;
    // n_rows * n_cols compared without forming a product that could wrap
    if (n_ops > kNaMaxOps || n_rows > kNaMaxCells / n_cols) return LTP_E_CAPACITY;
    if (n_ops && (!keys || !opw || !out)) return LTP_E_BADARG;
    if (n_txns && !commit) return LTP_E_BADARG;
    if (!txn_first && (uint64_t)ops_per_txn * n_txns != n_ops) return LTP_E_BADARG;
    if (txn_first && n_txns == 0 && n_ops != 0) return LTP_E_BADARG;  // ops that belong to no transaction
    if (cudaSetDevice(device) != cudaSuccess) return LTP_E_CUDA;
    unsigned char *base = nullptr;
    int sms = 0;
    int rc = setup_device(device, &base, &sms);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    Scratch s;
    memset(&s, 0, sizeof(s));
    s.words = (WordState *)(base + kOffWords);
    s.cview = (uint2 *)(base + kOffView);
    s.tw_list = (u32 *)(base + kOffTw);
    s.list[0] = (u64 *)(base + kOffList0);
    s.list[1] = (u64 *)(base + kOffList1);
    s.dcell = (u64 *)(base + kOffDcell);
    s.dbase = (long long *)(base + kOffDbase);
    s.dminw = (u32 *)(base + kOffDminw);
    s.st_sort[0] = (u32 *)(base + kOffSort0);
    s.st_sort[1] = (u32 *)(base + kOffSort1);
    s.st_cls = (u64 *)(base + kOffCls);
    s.st_apply = (u64 *)(base + kOffApply);
    s.st_ins = (u32 *)(base + kOffIns);
    // these batches carry no insert payload, so mark counts no insert and
    // neither array is used: the prefix array shares the status region
    s.ins_pre = s.st_ins;
    s.n_words = (n_rows * n_cols + 31) / 32 + 1;
    s.cap_ops = kNaMaxOps;
    s.cap_tiles = kNaTiles;
    s.cap_sort_tiles = kNaSortTiles;
    Counters *ctr = (Counters *)(base + kOffCtr);
    u32 *op_txn = (u32 *)(base + kOffOpTxn);

    // what must start at zero: this table's conflict words, look-back slots, counters
    cudaError_t e = launch_reset_scratch(st, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(Counters), st);
    // the caller's table holds n_rows rows for this call (no inserts here)
    u64 *rows_now = (u64 *)(base + kOffRows);
    if (e == cudaSuccess) e = launch_set_u64(st, rows_now, n_rows);
    if (e == cudaSuccess && n_txns) e = cudaMemsetAsync(commit, 1, n_txns, st);
    // txn_first lives in device memory the host never reads: checked there
    if (e == cudaSuccess && txn_first && n_txns)
        e = launch_expand_op_txn_checked(st, txn_first, n_txns, n_ops, op_txn, ctr);
    if (e != cudaSuccess) return LTP_E_CUDA;

    TablesDev T;
    memset(&T, 0, sizeof(T));
    T.n = 1;
    T.rows_now = rows_now;
    T.t[0].data = reinterpret_cast<char *>(table);
    T.t[0].rows_cap = rows_cap;
    T.t[0].row_limit = rows_cap;
    T.t[0].n_rows = n_rows;
    T.t[0].cell_base = 0;
    T.t[0].n_cols = n_cols;
    BatchDev b;
    b.keys = (const u64 *)keys;
    b.keys32 = nullptr;
    b.opw = opw;
    b.txn_first = txn_first;
    b.op_txn = op_txn;
    b.out = out;
    b.out64 = nullptr;
    b.commit = commit;
    b.n_ops = n_ops;
    b.n_txns = n_txns;
    b.ops_per_txn = txn_first ? 0u : ops_per_txn;
    b.flags = 0;
    b.payload = nullptr;
    b.payload_len = 0;
    Launch L;
    memset(&L, 0, sizeof(L));
    L.stream = st;
    L.num_sms = sms;
    L.rule = rule;
    L.tune = Tuning{512, 4, 32, 0};
    if (n_ops && launch_execute(L, b, T, s, ctr) != cudaSuccess) return LTP_E_CUDA;

    // the device-side status of this call
    int err = 0;
    if (cudaMemcpyAsync(&err, &ctr->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return LTP_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return LTP_E_CUDA;
    return err;
}
