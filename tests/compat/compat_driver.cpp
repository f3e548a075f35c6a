// compat_driver.cpp -- drives libltpmg_gb300.so through the reference's eight
// entry points the way the reference's Scheduler::start does
// (src/scheduler.cpp:27-73): upload the database, allocate the query
// buffers, re-send the same batch every epoch and execute it, then take the
// tables back.  Tables and queries come from a fixed-seed generator; the
// driver writes the queries and the final int table to a binary file that
// tests/test_compat.py replays through the oracle.
//
//   compat_driver <out_path> <variant 0..4 = YCSB_A..E> <rows> <txns> <epochs> <seed>
//   compat_driver <out_path> 5 <warehouses> <txns> <epochs> <seed>     (TPCC_PART)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <memory>
#include <unordered_set>
#include <vector>

#include "ltpmg_compat.h"

// The host program defines Param's constructor (src/param.cpp); this driver
// fills the fields the GPU library reads.
Param::Param() : table_size(0), batch_size(0), epoch_tp(0), epoch_sync(0), neworder_percent(0), table_cnt(0),
                 device_cnt(0), device_IDs(nullptr), zipf_config(0.0) {
    result.cost = 0.0;
    result.epoch = 0;
    result.batch_size = 0;
}
Param::~Param() {}

static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

template <typename Q>
static void make_queries(std::vector<std::any> &out, uint32_t txns, uint32_t rows, uint64_t seed,
                         std::vector<uint32_t> &flat) {
    uint64_t s = seed;
    for (uint32_t t = 0; t < txns; t++) {
        Q q;
        q.TID = t;
        std::unordered_set<uint32_t> seen;  // distinct rows per query (src/txn_generator.cpp:627-642)
        for (int j = 0; j < 10; j++) {
            uint32_t r;
            do {
                s += 0x9E3779B97F4A7C15ULL;
                // half of the rows from a small hot set, to make conflicts
                const uint64_t x = mix(s);
                r = (x & 1) ? (uint32_t)((x >> 1) % 16) : (uint32_t)((x >> 1) % rows);
            } while (seen.count(r));
            seen.insert(r);
            q.ROW_ID[j] = r;
        }
        out.emplace_back(q);
        flat.push_back(q.TID);
        for (int j = 0; j < 10; j++) flat.push_back(q.ROW_ID[j]);
    }
}

// TPC-C through the same entry points (TPCC_PART: new-order and payment):
// the nine tables of data/TPCC.json with their int columns only, W
// warehouses at the reference's sizes (src/param.cpp: 10 districts per
// warehouse, 3000 customers, new-order, history and order rows per
// district, 45000 order-line rows per district, 100000 stock rows per
// warehouse, 100000 items), a last-name index over the customers, and a
// seeded 50/50 mix of queries.  Writes the queries, the index and the final
// int tables.
static const uint32_t kTpccIntCols[9] = {1, 3, 5, 3, 5, 7, 8, 5, 2};

static int run_tpcc(const char *out_path, uint32_t W, uint32_t txns, uint32_t epochs, uint64_t seed) {
    auto param = std::make_shared<Param>();
    param->benchmark = "TPCC_PART";
    param->table_cnt = 9;
    param->table_size = W;
    param->batch_size = txns;
    param->epoch_tp = epochs;
    param->device_cnt = 1;
    param->device_IDs = new uint32_t[1]{0};
    const uint64_t d = (uint64_t)W * 10;
    const uint64_t rows[9] = {W, d, d * 3000, d * 3000, d * 3000, d * 3000, d * 45000, (uint64_t)W * 100000, 100000};
    std::vector<Global_Table_Info> info(9);
    std::vector<std::vector<int32_t>> ints(9);
    std::vector<std::vector<double>> dbls(9);
    std::vector<std::vector<uint32_t>> strs(9);
    std::vector<Global_Table> tables(9);
    for (int t = 0; t < 9; t++) {
        info[t].int_size = kTpccIntCols[t];
        info[t].double_size = 1;
        info[t].string_size = 1;
        info[t].table_size = (uint32_t)rows[t];
        info[t].table_cnt = 9;
        ints[t].resize(rows[t] * kTpccIntCols[t]);
        for (uint64_t r = 0; r < rows[t]; r++)
            for (uint32_t c = 0; c < kTpccIntCols[t]; c++)
                ints[t][r * kTpccIntCols[t] + c] = ltp_table_value(seed + t, r, c, kTpccIntCols[t]);
        dbls[t].assign(rows[t], 0.5);
        strs[t].assign(rows[t] * 8, 0x61616161u);
        tables[t] = Global_Table{ints[t].data(), dbls[t].data(), strs[t].data()};
    }
    // customer last-name index: one name id (0..999) per customer row
    std::vector<uint32_t> cidx(rows[2]);
    uint64_t s = seed ^ 0xC0FFEEull;
    for (auto &v : cidx) v = (uint32_t)(mix(s += 0x9E3779B97F4A7C15ULL) % 1000);
    std::vector<Global_Table_Index> index(9, Global_Table_Index{nullptr});
    index[2].index = cidx.data();

    std::vector<std::any> qv;
    std::vector<uint32_t> flat;  // per query: kind (0 new-order, 1 payment) then the struct's words
    for (uint32_t t = 0; t < txns; t++) {
        auto rnd = [&](uint64_t n) { return (uint32_t)(mix(s += 0x9E3779B97F4A7C15ULL) % n); };
        if (rnd(2) == 0) {
            Neworder_Query q;
            memset(&q, 0, sizeof(q));
            q.TID = t;
            q.W_ID = rnd(W);
            q.D_ID = rnd(10);
            q.C_ID = rnd(3000);
            q.O_ID = rnd(3000);
            q.N_O_ID = rnd(3000);
            q.O_OL_CNT = 5 + rnd(11);
            q.O_OL_ID = rnd(45000);
            for (uint32_t i = 0; i < q.O_OL_CNT; i++) {
                q.INFO[i].OL_I_ID = rnd(100000);
                q.INFO[i].OL_SUPPLY_W_ID = rnd(100) == 0 ? rnd(W) : q.W_ID;
                q.INFO[i].OL_QUANTITY = 1 + rnd(10);
            }
            qv.emplace_back(q);
            flat.push_back(0);
            const uint32_t *w = reinterpret_cast<const uint32_t *>(&q);
            flat.insert(flat.end(), w, w + sizeof(q) / 4);
        } else {
            Payment_Query q;
            memset(&q, 0, sizeof(q));
            q.TID = t;
            q.W_ID = rnd(W);
            q.D_ID = rnd(10);
            q.C_ID = rnd(3000);
            q.C_LAST = rnd(1000);
            q.isName = rnd(10) < 6 ? 1 : 0;
            const bool remote = rnd(100) < 15;
            q.C_W_ID = remote ? rnd(W) : q.W_ID;
            q.C_D_ID = remote ? rnd(10) : q.D_ID;
            q.H_AMOUNT = 1 + rnd(5000);
            q.H_ID = rnd(30000);
            qv.emplace_back(q);
            flat.push_back(1);
            const uint32_t *w = reinterpret_cast<const uint32_t *>(&q);
            flat.insert(flat.end(), w, w + sizeof(q) / 4);
        }
    }
    auto batch = std::make_shared<std::vector<std::any>>(qv);
    Global_Txn_Info txn_info;
    transfer_database_to_GPU(param, info.data(), tables.data(), index.data());
    int st = ltp_compat_last_status();
    if (!st) {
        initial_query_on_GPU(param, batch, &txn_info);
        initial_launcher_on_GPU(param);
        for (uint32_t e = 0; e < epochs && !ltp_compat_last_status(); e++) {
            transfer_query_to_GPU(param, batch, &txn_info);
            if (!ltp_compat_last_status()) execute_on_GPU(param);
        }
        st = ltp_compat_last_status();
        free_launcher_on_GPU(param);
        transfer_query_to_CPU(param, batch, &txn_info);
        transfer_database_to_CPU(param, info.data(), tables.data(), index.data());
        if (!st) st = ltp_compat_last_status();
    }
    FILE *f = fopen(out_path, "wb");
    if (!f) return 3;
    const int32_t header[4] = {st, (int32_t)W, (int32_t)txns, (int32_t)epochs};
    fwrite(header, sizeof(header), 1, f);
    const uint32_t nflat = (uint32_t)flat.size();
    fwrite(&nflat, 4, 1, f);
    fwrite(flat.data(), 4, flat.size(), f);
    fwrite(cidx.data(), 4, cidx.size(), f);
    for (int t = 0; t < 9; t++) fwrite(ints[t].data(), 4, ints[t].size(), f);
    fclose(f);
    if (st) fprintf(stderr, "compat status %d: %s\n", st, ltp_compat_last_error());
    printf("status %d cost %.6f s\n", st, param->result.cost);
    delete[] param->device_IDs;
    return st ? 1 : 0;
}

int main(int argc, char **argv) {
    if (argc < 7) {
        fprintf(stderr, "usage: %s out variant rows txns epochs seed\n", argv[0]);
        return 2;
    }
    const char *out_path = argv[1];
    const int variant = atoi(argv[2]);
    const uint32_t rows = (uint32_t)atoi(argv[3]);
    const uint32_t txns = (uint32_t)atoi(argv[4]);
    const uint32_t epochs = (uint32_t)atoi(argv[5]);
    const uint64_t seed = strtoull(argv[6], nullptr, 10);
    static const char *names[5] = {"YCSB_A", "YCSB_B", "YCSB_C", "YCSB_D", "YCSB_E"};
    if (variant == 5) return run_tpcc(out_path, rows, txns, epochs, seed);  // rows = warehouses

    auto param = std::make_shared<Param>();
    param->benchmark = names[variant];
    param->table_cnt = 1;
    param->batch_size = txns;
    param->epoch_tp = epochs;
    param->device_cnt = 1;
    param->device_IDs = new uint32_t[1]{0};

    // the YCSB schema (data/YCSB.json): 3 int, 3 double, 4 string columns
    Global_Table_Info info;
    info.int_size = 3;
    info.double_size = 3;
    info.string_size = 4;
    info.table_size = rows;
    info.table_cnt = 1;
    std::vector<int32_t> ints((size_t)rows * 3);
    std::vector<double> dbls((size_t)rows * 3, 0.5);
    std::vector<uint32_t> strs((size_t)rows * 4 * 8, 0x61616161u);
    for (uint32_t r = 0; r < rows; r++)
        for (uint32_t c = 0; c < 3; c++) ints[(size_t)r * 3 + c] = ltp_table_value(seed, r, c, 3);
    Global_Table table{ints.data(), dbls.data(), strs.data()};
    Global_Table_Index index{nullptr};

    std::vector<std::any> qv;
    std::vector<uint32_t> flat;
    switch (variant) {
    case 0: make_queries<YCSB_A_Query>(qv, txns, rows, seed, flat); break;
    case 1: make_queries<YCSB_B_Query>(qv, txns, rows, seed, flat); break;
    case 2: make_queries<YCSB_C_Query>(qv, txns, rows, seed, flat); break;
    case 3: make_queries<YCSB_D_Query>(qv, txns, rows, seed, flat); break;
    default: make_queries<YCSB_E_Query>(qv, txns, rows, seed, flat); break;
    }
    auto batch = std::make_shared<std::vector<std::any>>(qv);
    Global_Txn_Info txn_info;

    // Scheduler::start order (src/scheduler.cpp:33-71)
    transfer_database_to_GPU(param, &info, &table, &index);
    int st = ltp_compat_last_status();
    if (!st) {
        initial_query_on_GPU(param, batch, &txn_info);
        initial_launcher_on_GPU(param);
        for (uint32_t e = 0; e < epochs && !ltp_compat_last_status(); e++) {
            transfer_query_to_GPU(param, batch, &txn_info);
            if (!ltp_compat_last_status()) execute_on_GPU(param);
        }
        st = ltp_compat_last_status();
        free_launcher_on_GPU(param);
        transfer_query_to_CPU(param, batch, &txn_info);
        transfer_database_to_CPU(param, &info, &table, &index);
        if (!st) st = ltp_compat_last_status();
    }
    FILE *f = fopen(out_path, "wb");
    if (!f) return 3;
    const int32_t header[4] = {st, (int32_t)rows, (int32_t)txns, (int32_t)epochs};
    fwrite(header, sizeof(header), 1, f);
    fwrite(flat.data(), 4, flat.size(), f);
    fwrite(ints.data(), 4, ints.size(), f);
    fclose(f);
    if (st) fprintf(stderr, "compat status %d: %s\n", st, ltp_compat_last_error());
    printf("status %d cost %.6f s\n", st, param->result.cost);
    delete[] param->device_IDs;
    return st ? 1 : 0;
}
