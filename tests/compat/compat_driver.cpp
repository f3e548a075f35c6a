// compat_driver.cpp -- drives libltpmg_gb300.so through the reference's eight
// entry points the way the reference's Scheduler::start does
// (src/scheduler.cpp:27-73): upload the database, allocate the query
// buffers, re-send the same batch every epoch and execute it, then take the
// tables back.  Tables and queries come from a fixed-seed generator; the
// driver writes the queries and the final int table to a binary file that
// tests/test_compat.py replays through the oracle.
//
//   compat_driver <out_path> <variant 0..4 = YCSB_A..E> <rows> <txns> <epochs> <seed>
#include <cstdio>
#include <cstdlib>
#include <cstring>
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
