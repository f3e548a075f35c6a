/*
 * ltpmg_compat.h -- the reference host program's view of its GPU library,
 * served by libltpmg_gb300.so.
 *
 * The reference's host code (src/) talks to its CUDA library through eight
 * C++ functions (defined at cuda/src/gpuscheduler.cu:3-47, declared in
 * include/database.h:66-70, include/query.h:63-70, include/scheduler.h:33-37)
 * that take a std::shared_ptr<Param> and the host table / query structures.
 * This header declares those functions and the structures they receive with
 * the same names, members and member order, so that the reference's host
 * objects can be handed to this library unchanged (the layouts must agree
 * byte for byte; that is why the member lists below mirror include/param.h,
 * include/db_structure.h and include/txn_structure.h).  The definitions live
 * in ltpmg_gb300/csrc/ltp_compat.cpp and forward to the C ABI of
 * ltpmg_gb300.h.  Param's member functions are the host program's own
 * (src/param.cpp); this library only reads Param's data members.
 *
 * Mapping of the reference's operations (cuda/src/gpuquery.cu:2929-3303):
 *  - a YCSB "select" of a row reads every int column of the row; an "update"
 *    adds 1 to every int column of the row (the reference's operators leave
 *    the row unchanged, cuda/src/gpulauncher.cu:79-103; the YCSB workloads here add +1);
 *  - YCSB_E's 9 scans of rows [r, r+2) read those rows; its insert appends a
 *    row whose int columns are the query's ROW_ID[9] (the reference's insert
 *    operator is also an identity on an existing row);
 *  - TPC-C (TPCC_PART / TPCC_ALL; Neworder_Query and Payment_Query): the
 *    row operations of parse<Neworder_Query> / parse<Payment_Query>
 *    (cuda/src/gpuquery.cu:2474-2734), on the tables in data/TPCC.json order
 *    (0 warehouse, 1 district, 2 customer, 3 new-order, 4 history, 5 order,
 *    6 order-line, 7 stock, 8 item), each row taken modulo its table's rows
 *    as the reference's register_cc does (cuda/src/gpulauncher.cu:400):
 *    new-order reads warehouse W_ID, district W_ID*10+D_ID, customer
 *    (W_ID*10+D_ID)*3000+C_ID, inserts a new-order and an order row, and per
 *    line inserts an order-line row and updates stock
 *    OL_SUPPLY_W_ID*1000000+OL_I_ID twice; payment reads warehouse,
 *    district and the customer (by last name: the first of the district's
 *    3000 customers whose index entry equals C_LAST, :2641-2650), updates the
 *    customer, the warehouse and the district and inserts a history row.
 *    Selects and updates act on every int column as for YCSB.  An insert
 *    appends a row (the reference writes a preallocated row that its insert
 *    operator leaves unchanged) whose int columns hold the ids the query
 *    names, in the schema's int-column order: new-order (N_O_ID, D_ID, W_ID);
 *    order (O_ID, D_ID, W_ID, C_ID, 0, O_OL_CNT, all lines local);
 *    order-line (O_ID, D_ID, W_ID, line number, OL_I_ID, OL_SUPPLY_W_ID, 0,
 *    OL_QUANTITY); history (C_ID, C_D_ID, C_W_ID, D_ID, W_ID);
 *  - double and string columns stay on the host: this library stores int32
 *    columns only, and no reference operation changes the others.
 */
#ifndef LTPMG_COMPAT_H
#define LTPMG_COMPAT_H

#include <any>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "ltpmg_gb300.h"

/* include/db_structure.h */
struct Global_Table_Info {
    uint32_t int_size = 0;
    uint32_t double_size = 0;
    uint32_t string_size = 0;
    uint32_t string_length = 8;
    uint32_t table_size = 0;
    uint32_t table_cnt = 0;
};

struct Global_Table {
    int32_t *int_data;     /* row-major: int_data[row * int_size + col] */
    double *double_data;
    uint32_t *string_data;
};

struct Global_Table_Index {
    uint32_t *index;
};

/* include/txn_structure.h */
struct Global_Txn_Info {
    uint32_t cur_subtxn_cnt = 0;
    uint32_t select_cnt = 0;
    uint32_t insert_cnt = 0;
    uint32_t update_cnt = 0;
    uint32_t scan_cnt = 0;
    uint32_t delete_cnt = 0;
};

struct YCSB_A_Query { uint32_t TID; uint32_t ROW_ID[10]; };
struct YCSB_B_Query { uint32_t TID; uint32_t ROW_ID[10]; };
struct YCSB_C_Query { uint32_t TID; uint32_t ROW_ID[10]; };
struct YCSB_D_Query { uint32_t TID; uint32_t ROW_ID[10]; };
struct YCSB_E_Query { uint32_t TID; uint32_t ROW_ID[10]; };

struct Neworder_Query {
    uint32_t TID;
    uint32_t W_ID;
    uint32_t D_ID;
    uint32_t C_ID;
    uint32_t O_ID;
    uint32_t N_O_ID;
    uint32_t O_OL_CNT;
    uint32_t O_OL_ID;
    struct Info {
        uint32_t OL_I_ID;
        uint32_t OL_SUPPLY_W_ID;
        uint32_t OL_QUANTITY;
    };
    Info INFO[15];
};

struct Payment_Query {
    uint32_t TID;
    uint32_t W_ID;
    uint32_t D_ID;
    uint32_t C_ID;
    uint32_t C_LAST;
    uint32_t isName; /* 0: by C_ID, 1: by C_LAST through the customer index */
    uint32_t C_D_ID;
    uint32_t C_W_ID;
    uint32_t H_AMOUNT;
    uint32_t H_ID;
};

/* include/param.h: data members in the reference's order */
struct Result {
    double cost;
    uint32_t epoch;
    uint32_t batch_size;
};

class Param {
public:
    std::string benchmark;
    uint32_t table_size;
    uint32_t batch_size;
    uint32_t epoch_tp;
    uint32_t epoch_sync;
    std::string deviceIDs;
    uint32_t neworder_percent;
    std::string filepath;
    uint32_t table_cnt;
    uint32_t device_cnt;
    uint32_t *device_IDs;
    std::string data_distribution;
    double zipf_config;

    uint32_t test_1_size = 0;
    uint32_t test_2_size = 0;

    uint32_t warehouse_size = 0;
    uint32_t district_size = 0;
    uint32_t customer_size = 0;
    uint32_t neworder_size = 0;
    uint32_t history_size = 0;
    uint32_t order_size = 0;
    uint32_t orderline_size = 0;
    uint32_t stock_size = 0;
    uint32_t item_size = 100000;

    uint32_t ycsb_size = 0;
    uint32_t bitmap_row_cnt = 0;
    uint32_t bitmap_table_cnt = 0;

    uint32_t test_query_batch_size = 0;
    uint32_t test_query_2_batch_size = 0;
    uint32_t neworder_query_batch_size = 0;
    uint32_t payment_query_batch_size = 0;
    uint32_t orderstatus_query_batch_size = 0;
    uint32_t delivery_query_batch_size = 0;
    uint32_t stocklevel_query_batch_size = 0;
    uint32_t ycsb_a_query_batch_size = 0;
    uint32_t ycsb_b_query_batch_size = 0;
    uint32_t ycsb_c_query_batch_size = 0;
    uint32_t ycsb_d_query_batch_size = 0;
    uint32_t ycsb_e_query_batch_size = 0;

    uint32_t test_query_subtxn_cnt = 0;
    uint32_t test_query_2_subtxn_cnt = 0;
    uint32_t neworder_query_subtxn_cnt = 0;
    uint32_t payment_query_subtxn_cnt = 0;
    uint32_t orderstatus_query_subtxn_cnt = 0;
    uint32_t delivery_query_subtxn_cnt = 0;
    uint32_t stocklevel_query_subtxn_cnt = 0;
    uint32_t ycsb_a_query_subtxn_cnt = 0;
    uint32_t ycsb_b_query_subtxn_cnt = 0;
    uint32_t ycsb_c_query_subtxn_cnt = 0;
    uint32_t ycsb_d_query_subtxn_cnt = 0;
    uint32_t ycsb_e_query_subtxn_cnt = 0;

    uint32_t test_sub_txn_size = 0;
    uint32_t tpcc_all_sub_txn_size = 0;
    uint32_t tpcc_part_sub_txn_size = 0;
    uint32_t ycsb_a_sub_txn_size = 0;
    uint32_t ycsb_b_sub_txn_size = 0;
    uint32_t ycsb_c_sub_txn_size = 0;
    uint32_t ycsb_d_sub_txn_size = 0;
    uint32_t ycsb_e_sub_txn_size = 0;

    uint32_t test_query_subtxn_kinds = 0;
    uint32_t tpcc_all_query_subtxn_kinds = 0;
    uint32_t tpcc_part_query_subtxn_kinds = 0;
    uint32_t ycsb_a_query_subtxn_kinds = 0;
    uint32_t ycsb_b_query_subtxn_kinds = 0;
    uint32_t ycsb_c_query_subtxn_kinds = 0;
    uint32_t ycsb_d_query_subtxn_kinds = 0;
    uint32_t ycsb_e_query_subtxn_kinds = 0;

    uint32_t select_batch_size = 0;
    uint32_t insert_batch_size = 0;
    uint32_t update_batch_size = 0;
    uint32_t scan_batch_size = 0;
    uint32_t delete_batch_size = 0;

    Result result;

    Param();
    ~Param();
};

/* The reference's eight entry points (cuda/src/gpuscheduler.cu:3-47). */
void transfer_database_to_GPU(std::shared_ptr<Param> param, Global_Table_Info *table_for_gpu_info,
                              Global_Table *table_for_gpu, Global_Table_Index *index_for_GPU);
/* Also copies the int columns back into table_for_gpu (the reference only
 * freed its device copies, cuda/src/gpudatabase.cu:240-339). */
void transfer_database_to_CPU(std::shared_ptr<Param> param, Global_Table_Info *table_for_gpu_info,
                              Global_Table *table_for_gpu, Global_Table_Index *index_for_GPU);
void initial_query_on_GPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> transactions_batch_ptr,
                          Global_Txn_Info *global_txn_info);
void transfer_query_to_GPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> transactions_batch_ptr,
                           Global_Txn_Info *global_txn_info);
void transfer_query_to_CPU(std::shared_ptr<Param> param, std::shared_ptr<std::vector<std::any>> transactions_batch_ptr,
                           Global_Txn_Info *global_txn_info);
void initial_launcher_on_GPU(std::shared_ptr<Param> param);
void execute_on_GPU(std::shared_ptr<Param> param);
void free_launcher_on_GPU(std::shared_ptr<Param> param);

/* Status of the last compat call (0 = ok) and its message: the reference's
 * entry points return void, so failures are reported here instead of the
 * reference's print-and-exit. */
extern "C" int ltp_compat_last_status(void);
extern "C" const char *ltp_compat_last_error(void);

#endif
