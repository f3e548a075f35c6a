// ltp_compat.cpp -- the reference's eight GPU entry points
// (cuda/src/gpuscheduler.cu:3-47) implemented on the C ABI.
//
// The reference keeps all GPU state in one global GPUScheduler
// (cuda/include/gpuscheduler.cuh:54); these entry points keep the same
// single-owner shape (one context, its tables and one batch) because their
// signatures carry no handle.  Query expansion follows the reference's parse
// kernels: per YCSB variant, which of the ten row slots are selects, updates,
// scans or the insert (cuda/src/gpuquery.cu:2929-3303); for TPC-C the row
// operations of new-order and payment (cuda/src/gpuquery.cu:2474-2734).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <typeinfo>

#include "../../include/ltpmg_compat.h"

namespace {

struct CompatState {
    ltp_ctx *ctx = nullptr;
    std::vector<uint32_t> table_id;  // per reference table; UINT32_MAX when it has no int column
    std::vector<uint32_t> int_cols;
    std::vector<uint64_t> rows;
    ltp_batch *batch = nullptr;
    uint64_t cap_txns = 0, cap_ops = 0;
    std::vector<uint32_t> txn_first;
    std::vector<uint64_t> keys;
    std::vector<uint32_t> opw;
    std::vector<int32_t> payload;
    std::vector<uint32_t> cust_index;  // TPC-C: the customer table's last-name index (index_for_GPU[2])
    bool tpcc = false;
    int status = 0;
    std::string error;
};

CompatState g;

// Opt-in summary for integrators: with LTPMG_COMPAT_REPORT set in the
// environment, one line on stderr at process exit -- batches executed
// through execute_on_GPU, transactions they committed, and the first failing
// status with its message (the reference's host program checks none of the
// entry points' outcomes).
struct CompatReport {
    uint64_t batches = 0, committed = 0;
    int first_status = 0;
    std::string first_error;
    ~CompatReport() {
        if (!std::getenv("LTPMG_COMPAT_REPORT")) return;
        std::fprintf(stderr, "ltp_compat: batches=%llu committed=%llu status=%d%s%s\n", (unsigned long long)batches,
                     (unsigned long long)committed, first_status, first_error.empty() ? "" : " ", first_error.c_str());
    }
};
CompatReport g_report;

void set_status(int st, const std::string &msg) {
    g.status = st;
    g.error = msg;
    if (st != 0 && g_report.first_status == 0) {
        g_report.first_status = st;
        g_report.first_error = msg;
    }
}

int check(int rc, const char *where) {
    if (rc != LTP_OK) {
        std::string m = std::string(where) + ": " + ltp_status_string(rc);
        if (g.ctx) m += std::string(" (") + ltp_last_error(g.ctx) + ")";
        set_status(rc, m);
    }
    return rc;
}

// Kind of row slot i of a YCSB query (cuda/src/gpuquery.cu:2929-3303):
// 0 select, 2 update, 4 scan of [row, row+2), 1 insert.
uint32_t ycsb_slot_kind(int variant, uint32_t i) {
    switch (variant) {
    case 0: return i < 5 ? 0u : 2u;             // YCSB_A
    case 1: case 3: return i < 9 ? 0u : 2u;     // YCSB_B, YCSB_D
    case 2: return 0u;                          // YCSB_C
    default: return i < 9 ? 4u : 1u;            // YCSB_E
    }
}

// table order of data/TPCC.json
constexpr uint32_t kTpccWarehouse = 0, kTpccDistrict = 1, kTpccCustomer = 2, kTpccNewOrder = 3, kTpccHistory = 4,
                   kTpccOrder = 5, kTpccOrderLine = 6, kTpccStock = 7;

// One reference row operation (cuda/src/gpuquery.cu:2474-2734) as cell ops:
// a select reads every int column, an update adds 1 to every int column, an
// insert appends a row whose int columns are `vals` (zero-filled).
void row_op(uint32_t kind, uint32_t table, uint64_t row, const std::vector<int32_t> &vals) {
    const uint32_t cols = g.int_cols[table];
    if (g.table_id[table] == UINT32_MAX || cols == 0) return;
    const uint32_t tb = g.table_id[table];
    if (kind == 1) {
        g.keys.push_back(g.payload.size());
        g.opw.push_back(LTP_OPW(LTP_OP_INSERT, 0, tb, 0));
        for (uint32_t c = 0; c < cols; c++) g.payload.push_back(c < vals.size() ? vals[c] : 0);
        return;
    }
    const uint64_t r = row % g.rows[table];  // as register_cc (cuda/src/gpulauncher.cu:400)
    for (uint32_t c = 0; c < cols; c++) {
        g.keys.push_back(r);
        g.opw.push_back(kind == 2 ? LTP_OPW(LTP_OP_ADD, c, tb, 1) : LTP_OPW(LTP_OP_READ, c, tb, 0));
    }
}

// parse<Neworder_Query> (cuda/src/gpuquery.cu:2474-2606): 5 + 3 per line
void expand_neworder(const Neworder_Query &q) {
    const uint64_t wd = (uint64_t)q.W_ID * 10 + q.D_ID;
    const uint32_t lines = std::min<uint32_t>(q.O_OL_CNT, 15);
    bool local = true;
    for (uint32_t i = 0; i < lines; i++) local = local && q.INFO[i].OL_SUPPLY_W_ID == q.W_ID;
    row_op(0, kTpccWarehouse, q.W_ID, {});
    row_op(0, kTpccDistrict, wd, {});
    row_op(0, kTpccCustomer, wd * 3000 + q.C_ID, {});
    row_op(1, kTpccNewOrder, 0, {(int32_t)q.N_O_ID, (int32_t)q.D_ID, (int32_t)q.W_ID});
    row_op(1, kTpccOrder, 0,
           {(int32_t)q.O_ID, (int32_t)q.D_ID, (int32_t)q.W_ID, (int32_t)q.C_ID, 0, (int32_t)lines, local ? 1 : 0});
    for (uint32_t i = 0; i < lines; i++) {
        const auto &l = q.INFO[i];
        row_op(1, kTpccOrderLine, 0,
               {(int32_t)q.O_ID, (int32_t)q.D_ID, (int32_t)q.W_ID, (int32_t)(i + 1), (int32_t)l.OL_I_ID,
                (int32_t)l.OL_SUPPLY_W_ID, 0, (int32_t)l.OL_QUANTITY});
        const uint64_t stock = (uint64_t)l.OL_SUPPLY_W_ID * 1000000ull + l.OL_I_ID;
        row_op(2, kTpccStock, stock, {});
        row_op(2, kTpccStock, stock, {});
    }
}

// parse<Payment_Query> (cuda/src/gpuquery.cu:2608-2734): 7 row operations;
// by last name, the customer is the first of the (W_ID, D_ID) district's
// 3000 whose index entry equals C_LAST (0 when none does), addressed in the
// (C_W_ID, C_D_ID) district as the reference addresses it
void expand_payment(const Payment_Query &q) {
    const uint64_t wd = (uint64_t)q.W_ID * 10 + q.D_ID;
    uint32_t c_id = q.C_ID;
    if (q.isName == 1) {
        c_id = 0;
        for (uint32_t i = 0; i < 3000; i++) {
            const uint64_t at = wd * 3000 + i;
            if (at < g.cust_index.size() && g.cust_index[at] == q.C_LAST) {
                c_id = i;
                break;
            }
        }
    }
    const uint64_t cust = ((uint64_t)q.C_W_ID * 10 + q.C_D_ID) * 3000 + c_id;
    row_op(0, kTpccWarehouse, q.W_ID, {});
    row_op(0, kTpccDistrict, wd, {});
    row_op(0, kTpccCustomer, cust, {});
    row_op(2, kTpccCustomer, cust, {});
    row_op(2, kTpccWarehouse, q.W_ID, {});
    row_op(2, kTpccDistrict, wd, {});
    row_op(1, kTpccHistory, 0,
           {(int32_t)c_id, (int32_t)q.C_D_ID, (int32_t)q.C_W_ID, (int32_t)q.D_ID, (int32_t)q.W_ID});
}

struct Linear {
    uint32_t tid;
    int variant;  // 0-4 YCSB_A..E, 5 new-order, 6 payment
    const uint32_t *rows;
    const Neworder_Query *neworder;
    const Payment_Query *payment;
};

}  // namespace

extern "C" int ltp_compat_last_status(void) { return g.status; }
extern "C" const char *ltp_compat_last_error(void) { return g.error.c_str(); }

void transfer_database_to_GPU(std::shared_ptr<Param> param, Global_Table_Info *info, Global_Table *tables,
                              Global_Table_Index *index_for_GPU) {
    set_status(0, "");
    if (!param || !info || !tables) return set_status(LTP_E_BADARG, "transfer_database_to_GPU: null argument");
    if (g.ctx) ltp_shutdown(g.ctx);
    g = CompatState();
    ltp_config cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.device = (param->device_cnt && param->device_IDs) ? (int32_t)param->device_IDs[0] : 0;
    cfg.rule = LTP_RULE_ORDERED;
    if (check(ltp_init(&cfg, &g.ctx), "ltp_init")) return;
    g.tpcc = param->benchmark == "TPCC_PART" || param->benchmark == "TPCC_ALL";
    // TPC-C payments by last name read the customer index (the reference reads
    // it on the device, cuda/src/gpuquery.cu:2641-2650); keep a host copy
    if (g.tpcc && param->table_cnt > 2 && index_for_GPU && index_for_GPU[2].index)
        g.cust_index.assign(index_for_GPU[2].index, index_for_GPU[2].index + info[2].table_size);
    for (uint32_t t = 0; t < param->table_cnt; t++) {
        const uint32_t cols = info[t].int_size;
        const uint64_t rows = info[t].table_size;
        g.int_cols.push_back(cols);
        g.rows.push_back(rows);
        if (cols == 0 || rows == 0) {
            g.table_id.push_back(UINT32_MAX);
            continue;
        }
        ltp_schema sc;
        memset(&sc, 0, sizeof(sc));
        sc.n_cols = cols;
        uint32_t id = 0;
        // YCSB_E appends one row per transaction and epoch: leave room for them
        // (the host arrays keep only the original rows)
        uint64_t cap = rows;
        const uint64_t epochs = param->epoch_tp ? param->epoch_tp : 1;
        if (param->benchmark == "YCSB_E") cap += (uint64_t)param->batch_size * epochs;
        // TPC-C inserts: new-order, history and order gain at most one row per
        // transaction, order-line at most 15
        if (g.tpcc && t >= kTpccNewOrder && t <= kTpccOrderLine)
            cap += (uint64_t)param->batch_size * epochs * (t == kTpccOrderLine ? 15 : 1);
        if (check(ltp_table_create_cap(g.ctx, &sc, rows, cap, &id), "ltp_table_create")) return;
        g.table_id.push_back(id);
        std::vector<int32_t> col(rows);
        for (uint32_t c = 0; c < cols; c++) {  // row-major host rows -> one device column
            for (uint64_t r = 0; r < rows; r++) col[r] = tables[t].int_data[r * cols + c];
            if (check(ltp_table_upload(g.ctx, id, c, 0, rows, col.data()), "ltp_table_upload")) return;
        }
    }
}

void transfer_database_to_CPU(std::shared_ptr<Param> param, Global_Table_Info *info, Global_Table *tables,
                              Global_Table_Index *index_for_GPU) {
    (void)info;
    (void)index_for_GPU;
    if (!g.ctx) return set_status(LTP_E_STATE, "transfer_database_to_CPU: no database on the GPU");
    if (param && tables) {
        for (size_t t = 0; t < g.table_id.size() && t < param->table_cnt; t++) {
            if (g.table_id[t] == UINT32_MAX) continue;
            const uint32_t cols = g.int_cols[t];
            const uint64_t rows = g.rows[t];
            std::vector<int32_t> col(rows);
            for (uint32_t c = 0; c < cols; c++) {
                if (check(ltp_table_download(g.ctx, g.table_id[t], c, 0, rows, col.data()), "ltp_table_download"))
                    return;
                for (uint64_t r = 0; r < rows; r++) tables[t].int_data[r * cols + c] = col[r];
            }
        }
    }
    if (g.batch) ltp_batch_free(g.ctx, g.batch);
    ltp_shutdown(g.ctx);
    const int st = g.status;
    const std::string err = g.error;
    g = CompatState();
    set_status(st, err);
}

void initial_query_on_GPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> batch,
                          Global_Txn_Info *global_txn_info) {
    (void)global_txn_info;
    if (!g.ctx || !param) return set_status(LTP_E_STATE, "initial_query_on_GPU: call transfer_database_to_GPU first");
    const uint64_t txns = batch ? batch->size() : param->batch_size;
    // a YCSB query expands to at most 10 rows x 2 (scans) x the int columns;
    // a TPC-C new-order to 5 + 3 x 15 rows x the widest table's int columns
    uint64_t cols = 1;
    for (size_t t = 0; t < g.int_cols.size(); t++)
        if ((t == 0 || g.tpcc) && g.int_cols[t] > cols) cols = g.int_cols[t];
    g.cap_txns = txns ? txns : 1;
    g.cap_ops = g.cap_txns * (g.tpcc ? 50 : 20) * cols;
    if (g.batch) ltp_batch_free(g.ctx, g.batch);
    g.batch = nullptr;
    check(ltp_batch_create(g.ctx, g.cap_txns, g.cap_ops, &g.batch), "ltp_batch_create");
}

void transfer_query_to_GPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> batch,
                           Global_Txn_Info *global_txn_info) {
    (void)param;
    (void)global_txn_info;
    if (!g.ctx || !g.batch || !batch) return set_status(LTP_E_STATE, "transfer_query_to_GPU: no batch allocated");
    if (g.table_id.empty() || g.table_id[0] == UINT32_MAX)
        return set_status(LTP_E_STATE, "transfer_query_to_GPU: the first table has no int column");
    std::vector<Linear> qs;
    qs.reserve(batch->size());
    for (const std::any &a : *batch) {
        const std::type_info &ty = a.type();
        const YCSB_A_Query *q = nullptr;
        int v = -1;
        // the five query structs share one layout: {TID, ROW_ID[10]}
        if (ty == typeid(YCSB_A_Query)) v = 0, q = std::any_cast<YCSB_A_Query>(&a);
        else if (ty == typeid(YCSB_B_Query)) v = 1, q = reinterpret_cast<const YCSB_A_Query *>(std::any_cast<YCSB_B_Query>(&a));
        else if (ty == typeid(YCSB_C_Query)) v = 2, q = reinterpret_cast<const YCSB_A_Query *>(std::any_cast<YCSB_C_Query>(&a));
        else if (ty == typeid(YCSB_D_Query)) v = 3, q = reinterpret_cast<const YCSB_A_Query *>(std::any_cast<YCSB_D_Query>(&a));
        else if (ty == typeid(YCSB_E_Query)) v = 4, q = reinterpret_cast<const YCSB_A_Query *>(std::any_cast<YCSB_E_Query>(&a));
        if (q) {
            qs.push_back(Linear{q->TID, v, q->ROW_ID, nullptr, nullptr});
            continue;
        }
        const Neworder_Query *no = std::any_cast<Neworder_Query>(&a);
        const Payment_Query *pm = std::any_cast<Payment_Query>(&a);
        if (g.tpcc && no) qs.push_back(Linear{no->TID, 5, nullptr, no, nullptr});
        else if (g.tpcc && pm) qs.push_back(Linear{pm->TID, 6, nullptr, nullptr, pm});
        else return set_status(LTP_E_BADARG, std::string("transfer_query_to_GPU: unsupported query type ") + ty.name());
    }
    // TID order is the serial order (the reference assigns TIDs by position)
    std::stable_sort(qs.begin(), qs.end(), [](const Linear &a, const Linear &b) { return a.tid < b.tid; });
    const uint32_t cols = g.int_cols[0];
    const uint64_t rows = g.rows[0];
    g.txn_first.assign(1, 0);
    g.keys.clear();
    g.opw.clear();
    g.payload.clear();
    for (const Linear &q : qs) {
        if (q.variant == 5) {
            expand_neworder(*q.neworder);
        } else if (q.variant == 6) {
            expand_payment(*q.payment);
        } else {
            for (uint32_t i = 0; i < 10; i++) {
                const uint32_t kind = ycsb_slot_kind(q.variant, i);
                const uint64_t r = q.rows[i];
                if (kind == 1) {  // insert: a new row whose int columns hold ROW_ID[9]
                    g.keys.push_back(g.payload.size());
                    g.opw.push_back(LTP_OPW(LTP_OP_INSERT, 0, 0, 0));
                    for (uint32_t c = 0; c < cols; c++) g.payload.push_back((int32_t)r);
                    continue;
                }
                const uint64_t span = kind == 4 ? 2 : 1;
                for (uint64_t rr = r; rr < r + span && rr < rows; rr++)
                    for (uint32_t c = 0; c < cols; c++) {
                        g.keys.push_back(rr);
                        g.opw.push_back(kind == 2 ? LTP_OPW(LTP_OP_ADD, c, 0, 1) : LTP_OPW(LTP_OP_READ, c, 0, 0));
                    }
            }
        }
        g.txn_first.push_back((uint32_t)g.keys.size());
    }
    if (g.keys.size() > g.cap_ops || qs.size() > g.cap_txns)
        return set_status(LTP_E_CAPACITY, "transfer_query_to_GPU: batch larger than initial_query_on_GPU sized");
    if (check(ltp_batch_load(g.ctx, g.batch, qs.size(), g.txn_first.data(), 0, g.keys.size(), g.keys.data(),
                             g.opw.data(), nullptr),
              "ltp_batch_load"))
        return;
    if (!g.payload.empty())
        check(ltp_batch_load_payload(g.ctx, g.batch, g.payload.data(), g.payload.size(), nullptr),
              "ltp_batch_load_payload");
}

void transfer_query_to_CPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> batch,
                           Global_Txn_Info *global_txn_info) {
    (void)param;
    (void)batch;
    (void)global_txn_info;
    if (g.ctx && g.batch) ltp_batch_free(g.ctx, g.batch);
    g.batch = nullptr;
}

void initial_launcher_on_GPU(std::shared_ptr<Param> param) { (void)param; }

void execute_on_GPU(std::shared_ptr<Param> param) {
    if (!g.ctx || !g.batch) return set_status(LTP_E_STATE, "execute_on_GPU: no batch transferred");
    const auto t0 = std::chrono::steady_clock::now();
    if (check(ltp_batch_execute(g.ctx, g.batch, nullptr), "ltp_batch_execute")) return;
    ltp_stats st;
    if (check(ltp_batch_finish(g.ctx, g.batch, &st, nullptr), "ltp_batch_finish")) return;
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    g_report.batches++;
    g_report.committed += st.committed;
    if (param) param->result.cost = s;  // as GPUlauncher sets it (cuda/src/gpulauncher.cu:1071-1077)
}

void free_launcher_on_GPU(std::shared_ptr<Param> param) { (void)param; }
