// ref_gen_harness.cpp -- times the reference's own host workload generator:
// Query::generate_txn (src/query.cpp:270-311 for YCSB_A: Txn_Generator's
// generate_txn on std::thread::hardware_concurrency() threads,
// src/txn_generator.cpp:601-673, then the shuffle and TID assignment),
// compiled unchanged from the reference's src/*.cpp by oracle/build_ref.sh
// with the gflags/glog stand-ins under oracle/ref_shim.
//
// TEST AND BENCHMARK INFRASTRUCTURE ONLY: the product never links or runs it.
// It is the CPU baseline's generator/scheduler part; the execution part is
// the oracle's serial replay.
//
//   ltpmg_ref_gen <benchmark YCSB_A|YCSB_B> <table_size (x 10^6 rows)> <batch_size>
//                 <unif|zipf> <zipf_config> <reps>
// prints one JSON line: seconds per generate_txn call, threads, transactions.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "query.h"

DECLARE_string(benchmark);
DECLARE_uint32(table_size);
DECLARE_uint32(batch_size);
DECLARE_string(data_distribution);
DECLARE_double(zipf_config);

// query.cpp names the GPU library's entry points; the generator never calls
// them, so they have no body here
void initial_query_on_GPU(std::shared_ptr<Param>, std::shared_ptr<std::vector<std::any>>, Global_Txn_Info *) {}
void transfer_query_to_GPU(std::shared_ptr<Param>, std::shared_ptr<std::vector<std::any>>, Global_Txn_Info *) {}
void transfer_query_to_CPU(std::shared_ptr<Param>, std::shared_ptr<std::vector<std::any>>, Global_Txn_Info *) {}

int main(int argc, char **argv) {
    if (argc < 7) {
        fprintf(stderr, "usage: %s benchmark table_size batch_size unif|zipf zipf_config reps\n", argv[0]);
        return 2;
    }
    FLAGS_benchmark = argv[1];
    FLAGS_table_size = (uint32_t)atoi(argv[2]);
    FLAGS_batch_size = (uint32_t)atoi(argv[3]);
    FLAGS_data_distribution = argv[4];
    FLAGS_zipf_config = atof(argv[5]);
    const int reps = atoi(argv[6]) > 0 ? atoi(argv[6]) : 1;
    auto param = std::make_shared<Param>();
    std::vector<double> secs;
    for (int r = 0; r < reps; r++) {
        Query q;  // a fresh query set per call: generate_txn appends to it
        const auto t0 = std::chrono::steady_clock::now();
        q.generate_txn(param);
        const auto t1 = std::chrono::steady_clock::now();
        secs.push_back(std::chrono::duration<double>(t1 - t0).count());
    }
    printf("{\"benchmark\": \"%s\", \"rows\": %llu, \"txns\": %u, \"distribution\": \"%s\", \"zipf_config\": %g, "
           "\"threads\": %u, \"seconds\": [",
           FLAGS_benchmark.c_str(), (unsigned long long)FLAGS_table_size * 1000000ull, FLAGS_batch_size,
           FLAGS_data_distribution.c_str(), FLAGS_zipf_config, std::thread::hardware_concurrency());
    for (size_t i = 0; i < secs.size(); i++) printf("%s%.6f", i ? ", " : "", secs[i]);
    printf("]}\n");
    return 0;
}
