// ref_cuda_harness.cu -- runs the reference's own CUDA path (cuda/src/*.cu,
// compiled unchanged next to this file by oracle/build_ref.sh) on one GPU
// with a batch chosen by the caller, and writes out what that path computes.
//
// TEST INFRASTRUCTURE ONLY: the product never links or runs it.  It plays the
// reference host program's part (Scheduler::start, src/scheduler.cpp:27-73:
// transfer_database_to_GPU, initial_query_on_GPU, initial_launcher_on_GPU,
// then per epoch transfer_query_to_GPU + execute_on_GPU, all declared at
// cuda/include/gpuscheduler.cuh:57-77) with two differences: the YCSB_A
// queries and the table come from a file (the reference's generator is not
// seedable: src/random.cpp:6, src/query.cpp:282), and after the last epoch
// it copies back what the GPU built:
//   - the op records the parse kernel wrote (the host copy made at
//     cuda/src/gpuquery.cu:2132): TID, type, table, row per record;
//   - per row: ops registered by txn_executor (cnt_TID, register_cc at
//     cuda/src/gpulauncher.cu:413-417) and ops scattered into the row's bucket
//     by txn_analyze_regular (tmp_TID, :2375-2437);
//   - the rows with ops (used_rows_cnt, txn_prefix_offset :1558-1589) and the
//     type-list lengths (select_cur / update_cur, register_txn_exec :360-381);
//   - the int columns of the table after the batch (the reference has no
//     copy-back of its own: transfer_database_to_CPU only frees);
//   - the launcher's own timer (param->result.cost = cost_gpu, :1070-1099).
// The free entry points are not called: the process ends after the copy-back.
//
//   ltpmg_ref_cuda <in> <out>
//   in : u32 {rows, n_txns, epochs, 0}, u32 row_ids[n_txns][10], i32 ints[rows][3]
//   out: u32 {status, n_ops, rows, used_rows_cnt, select_cur, update_cur},
//        f32 cost_gpu of each epoch [epochs],
//        u32 rec[n_ops][4] = {TID, type, table_ID, dest_Row_1} in record order,
//        u32 cnt_TID[rows], u32 tmp_TID[rows], i32 ints_after[rows][3]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "define.cuh"
// read the private members of the reference's classes (layout unchanged)
#define private public
#include "gpudatabase.cuh"
#include "gpuquery.cuh"
#include "gpulauncher.cuh"
// the scheduler header also defines the library's global instance; this file
// must only name it, so the header's definition lands on an unused name
#define gpuscheduler ltpmg_harness_unused_scheduler
#include "gpuscheduler.cuh"
#undef gpuscheduler
#undef private

extern GPUScheduler gpuscheduler;

static bool ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fprintf(stderr, "ref harness: %s: %s\n", what, cudaGetErrorString(e));
    return e == cudaSuccess;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s in out\n", argv[0]);
        return 2;
    }
    FILE *fi = fopen(argv[1], "rb");
    if (!fi) return 3;
    uint32_t hdr[4];
    if (fread(hdr, sizeof(hdr), 1, fi) != 1) return 3;
    const uint32_t rows = hdr[0], n = hdr[1], epochs = hdr[2] ? hdr[2] : 1;
    std::vector<uint32_t> row_ids((size_t)n * 10);
    std::vector<int32_t> ints((size_t)rows * 3);
    if (fread(row_ids.data(), 4, row_ids.size(), fi) != row_ids.size()) return 3;
    if (fread(ints.data(), 4, ints.size(), fi) != ints.size()) return 3;
    fclose(fi);
    for (uint32_t v : row_ids)
        if (v >= rows) return 4;  // the reference indexes rows unchecked

    // Param as src/param.cpp:101-111 sets it for YCSB_A on one device
    auto param = std::make_shared<Param>();
    param->benchmark = "YCSB_A";
    param->table_size = 1;
    param->batch_size = n;
    param->epoch_tp = epochs;
    param->epoch_sync = 1;
    param->deviceIDs = "0";
    param->neworder_percent = 100;
    param->table_cnt = 1;
    param->device_cnt = 1;
    param->device_IDs = new uint32_t[1]{0};
    param->data_distribution = "unif";
    param->zipf_config = 0.0;
    param->ycsb_size = rows;
    param->bitmap_row_cnt = 100;
    param->bitmap_table_cnt = 1;
    param->ycsb_a_query_batch_size = n;
    param->ycsb_a_query_subtxn_cnt = 10;
    param->ycsb_a_sub_txn_size = 10 * n;
    param->ycsb_a_query_subtxn_kinds = 10;
    param->result.cost = 0.0;
    param->result.epoch = epochs;
    param->result.batch_size = n;

    // the YCSB table of data/YCSB.json: 3 int, 3 double, 4 string attributes
    Global_Table_Info info;
    info.int_size = 3;
    info.double_size = 3;
    info.string_size = 4;
    info.string_length = 8;
    info.table_size = rows;
    info.table_cnt = 1;
    std::vector<double> dbls((size_t)rows * 3, 0.25);
    std::vector<uint32_t> strs((size_t)rows * 4 * 8, 0x72616e64u);
    Global_Table table;
    table.int_data = ints.data();
    table.double_data = dbls.data();
    table.string_data = strs.data();
    Global_Table_Index index;
    index.index = nullptr;

    auto batch = std::make_shared<std::vector<std::any>>();
    batch->reserve(n);
    for (uint32_t t = 0; t < n; t++) {
        YCSB_A_Query q;
        q.TID = t;
        for (int j = 0; j < 10; j++) q.ROW_ID[j] = row_ids[(size_t)t * 10 + j];
        batch->emplace_back(q);
    }
    Global_Txn_Info txn_info;

    transfer_database_to_GPU(param, &info, &table, &index);
    initial_query_on_GPU(param, batch, &txn_info);
    initial_launcher_on_GPU(param);
    std::vector<float> costs;
    for (uint32_t e = 0; e < epochs; e++) {
        transfer_query_to_GPU(param, batch, &txn_info);
        execute_on_GPU(param);
        costs.push_back((float)param->result.cost);
    }

    // copy back what the last epoch built
    GPUquery *q = gpuscheduler.gpuquery;
    GPUdatabase *d = gpuscheduler.gpudatabase;
    const uint32_t n_ops = 10 * n;
    bool ok = ck(cudaSetDevice(0), "set device") && ck(cudaDeviceSynchronize(), "sync");
    std::vector<uint32_t> rec((size_t)n_ops * 4);
    for (uint32_t k = 0; k < n_ops; k++) {
        const Global_Txn &g = q->global_txn[k];
        rec[(size_t)k * 4 + 0] = g.subtxn.TID;
        rec[(size_t)k * 4 + 1] = g.subtxn.type;
        rec[(size_t)k * 4 + 2] = g.subtxn.table_ID;
        rec[(size_t)k * 4 + 3] = g.subtxn.dest_Row_1;
    }
    std::vector<uint32_t> cnt(rows), tmp(rows);
    std::vector<int32_t> after((size_t)rows * 3);
    Global_Txn_Aux_Struct aux;
    Global_Txn_Exec ex;
    ok = ok && ck(cudaMemcpy(&aux, &q->aux_struct_d[0][0], sizeof(aux), cudaMemcpyDeviceToHost), "aux");
    ok = ok && ck(cudaMemcpy(&ex, q->global_txn_exec_d[0], sizeof(ex), cudaMemcpyDeviceToHost), "exec");
    ok = ok && ck(cudaMemcpy(cnt.data(), q->aux_struct_d_h[0][0].cnt_TID, 4ull * rows, cudaMemcpyDeviceToHost), "cnt");
    ok = ok && ck(cudaMemcpy(tmp.data(), q->aux_struct_d_h[0][0].tmp_TID, 4ull * rows, cudaMemcpyDeviceToHost), "tmp");
    ok = ok && ck(cudaMemcpy(after.data(), d->tables_d_h[0][0].int_data, 4ull * rows * 3, cudaMemcpyDeviceToHost),
                  "table");

    FILE *fo = fopen(argv[2], "wb");
    if (!fo) return 5;
    const uint32_t oh[6] = {ok ? 0u : 1u, n_ops, rows, aux.used_rows_cnt, ex.select_cur, ex.update_cur};
    fwrite(oh, sizeof(oh), 1, fo);
    fwrite(costs.data(), 4, costs.size(), fo);
    fwrite(rec.data(), 4, rec.size(), fo);
    fwrite(cnt.data(), 4, cnt.size(), fo);
    fwrite(tmp.data(), 4, tmp.size(), fo);
    fwrite(after.data(), 4, after.size(), fo);
    fclose(fo);
    printf("ref harness: %u txns x %u epochs, cost_gpu of the last epoch %.6f s\n", n, epochs,
           costs.empty() ? 0.0 : costs.back());
    return ok ? 0 : 1;
}
