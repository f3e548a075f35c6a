// ltp_tpcc.cpp -- seeded TPC-C-shaped order-entry workload: the nine-table
// schema, its initial contents and batches of new-order / payment
// transactions expanded into ops.
//
// Replaces the reference's TPC-C pieces on the hot path: the schema of
// data/TPCC.json parsed by Row_Parser (src/row_parser.cpp:3-28), the table
// fill of src/database.cpp:78-395 (with the customer last-name index,
// database.cpp:310-393), the Neworder / Payment generators
// (src/txn_generator.cpp:231-381) and their op expansion on the GPU
// (parse<Neworder_Query> cuda/src/gpuquery.cu:2474-2606, parse<Payment_Query>
// gpuquery.cu:2608-2734).  Every value is a pure function of the seed, so a
// batch and a table are the same for any thread count and on any machine.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <thread>
#include <vector>

#include "../../include/ltpmg_gb300.h"
#include "ltp_rng.h"

using ltp_rng::mix;
using ltp_rng::Stream;

namespace {

constexpr uint32_t kMaxLines = 15;
constexpr uint32_t kNames = 1000;  // distinct customer last names

struct TableShape {
    uint32_t n_cols;
    uint64_t wide;
};

const TableShape kShape[LTP_TPCC_N_TABLES] = {
    {LTPC_W_NCOLS, 1ull << LTPC_W_YTD},
    {LTPC_D_NCOLS, 1ull << LTPC_D_YTD},
    {LTPC_C_NCOLS, (1ull << LTPC_C_BALANCE) | (1ull << LTPC_C_YTD_PAYMENT)},
    {LTPC_H_NCOLS, 1ull << LTPC_H_AMOUNT},
    {LTPC_NO_NCOLS, 0},
    {LTPC_O_NCOLS, 0},
    {LTPC_OL_NCOLS, 1ull << LTPC_OL_AMOUNT},
    {LTPC_I_NCOLS, 0},
    {LTPC_S_NCOLS, 1ull << LTPC_S_YTD},
};

// NURand(A, x, y) as the reference draws it (Random::non_uniform_distribution,
// src/random.cpp:58-60; no run-time constant C):
// ((U[0, A] | U[x, y]) mod (y - x + 1)) + x.
uint64_t nurand(Stream &st, uint64_t A, uint64_t x, uint64_t y) {
    const uint64_t a = st.range(0, A), b = st.range(x, y);
    return (a | b) % (y - x + 1) + x;
}

}  // namespace

struct ltp_tpcc {
    ltp_tpcc_params p;
    uint64_t thr_no, thr_rl, thr_rp, thr_bn;
    std::vector<int32_t> by_name;  // [W * D * kNames] customer index per (district, last name), -1: none

    uint64_t districts() const { return (uint64_t)p.warehouses * p.districts; }
    uint64_t rows(uint32_t t) const {
        switch (t) {
        case LTP_TPCC_WAREHOUSE: return p.warehouses;
        case LTP_TPCC_DISTRICT: return districts();
        case LTP_TPCC_CUSTOMER: return districts() * p.customers;
        case LTP_TPCC_ITEM: return p.items;
        case LTP_TPCC_STOCK: return (uint64_t)p.warehouses * p.items;
        default: return 0;  // insert-only tables start empty
        }
    }
    // raw 64-bit draw of one initial cell
    uint64_t h(uint32_t t, uint64_t row, uint32_t col) const {
        return mix(mix(p.seed ^ (0x5450434300000000ull + t)) + row * 64 + col);
    }
    int32_t text(uint32_t t, uint64_t row, uint32_t col) const { return (int32_t)(uint32_t)h(t, row, col); }
    int32_t c_last(uint64_t row) const {
        const uint64_t c = row % p.customers;
        if (c < kNames) return (int32_t)c;
        Stream st{mix(p.seed ^ 0x434C415354ull ^ mix(row))};
        return (int32_t)nurand(st, 255, 0, kNames - 1);
    }
    int32_t price(uint64_t item) const { return (int32_t)(100 + h(LTP_TPCC_ITEM, item, LTPC_I_PRICE) % 9901); }

    int64_t value(uint32_t t, uint32_t col, uint64_t r) const {
        const uint64_t x = h(t, r, col);
        switch (t) {
        case LTP_TPCC_WAREHOUSE:
            if (col == LTPC_W_ID) return (int64_t)r + 1;
            if (col == LTPC_W_TAX) return (int64_t)(x % 2001);  // basis points, 0 .. 20%
            if (col == LTPC_W_YTD) return 30000000;             // 300,000.00
            return text(t, r, col);
        case LTP_TPCC_DISTRICT:
            if (col == LTPC_D_ID) return (int64_t)(r % p.districts) + 1;
            if (col == LTPC_D_W_ID) return (int64_t)(r / p.districts) + 1;
            if (col == LTPC_D_TAX) return (int64_t)(x % 2001);
            if (col == LTPC_D_YTD) return 3000000;
            if (col == LTPC_D_NEXT_O_ID) return 3000;  // the populated orders 1..3000
            return text(t, r, col);
        case LTP_TPCC_CUSTOMER: {
            const uint64_t dist = r / p.customers;
            switch (col) {
            case LTPC_C_ID: return (int64_t)(r % p.customers) + 1;
            case LTPC_C_D_ID: return (int64_t)(dist % p.districts) + 1;
            case LTPC_C_W_ID: return (int64_t)(dist / p.districts) + 1;
            case LTPC_C_LAST: return c_last(r);
            case LTPC_C_CREDIT: return x % 10 == 0 ? 1 : 0;  // 1: bad credit (10%)
            case LTPC_C_DISCOUNT: return (int64_t)(x % 5001);
            case LTPC_C_BALANCE: return -1000;
            case LTPC_C_YTD_PAYMENT: return 1000;
            case LTPC_C_PAYMENT_CNT: return 1;
            case LTPC_C_DELIVERY_CNT: return 0;
            default: return text(t, r, col);
            }
        }
        case LTP_TPCC_ITEM:
            if (col == LTPC_I_ID) return (int64_t)r + 1;
            if (col == LTPC_I_IM_ID) return (int64_t)(1 + x % 10000);
            if (col == LTPC_I_PRICE) return price(r);
            return text(t, r, col);
        case LTP_TPCC_STOCK:
            switch (col) {
            case LTPC_S_I_ID: return (int64_t)(r % p.items) + 1;
            case LTPC_S_W_ID: return (int64_t)(r / p.items) + 1;
            case LTPC_S_QUANTITY: return (int64_t)(10 + x % 91);
            case LTPC_S_YTD:
            case LTPC_S_ORDER_CNT:
            case LTPC_S_REMOTE_CNT: return 0;
            default: return text(t, r, col);
            }
        default: return 0;
        }
    }

    // The draws of one transaction; pass 1 stops after the sizes.
    struct Txn {
        bool new_order;
        uint32_t w, d, c, ol;
        uint32_t item[kMaxLines], supply[kMaxLines], qty[kMaxLines];
        uint32_t cw, cd, amount;
    };
    uint32_t other_wh(Stream &st, uint32_t w) const {
        const uint32_t x = (uint32_t)st.below(p.warehouses - 1);
        return x >= w ? x + 1 : x;
    }
    void draw(Stream &st, Txn &x, bool sizes_only) const {
        x.new_order = st.chance(thr_no);
        x.w = (uint32_t)st.below(p.warehouses);
        x.d = (uint32_t)st.below(p.districts);
        if (x.new_order) {
            x.c = (uint32_t)nurand(st, 1023, 1, p.customers) - 1;
            x.ol = (uint32_t)st.range(p.ol_min, p.ol_max);
            if (sizes_only) return;
            for (uint32_t l = 0; l < x.ol; l++) {
                x.item[l] = (uint32_t)nurand(st, 8191, 1, p.items) - 1;
                x.supply[l] = (p.warehouses > 1 && st.chance(thr_rl)) ? other_wh(st, x.w) : x.w;
                x.qty[l] = (uint32_t)st.range(1, 10);
            }
        } else {
            x.ol = 0;
            if (sizes_only) return;
            x.amount = (uint32_t)st.range(100, 500000);  // cents
            if (p.warehouses > 1 && st.chance(thr_rp)) {
                x.cw = other_wh(st, x.w);
                x.cd = (uint32_t)st.below(p.districts);
            } else {
                x.cw = x.w;
                x.cd = x.d;
            }
            if (st.chance(thr_bn)) {
                const uint32_t name = (uint32_t)nurand(st, 255, 0, kNames - 1);
                const int32_t c = by_name[((uint64_t)x.cw * p.districts + x.cd) * kNames + name];
                x.c = c >= 0 ? (uint32_t)c : name % p.customers;
            } else {
                x.c = (uint32_t)nurand(st, 1023, 1, p.customers) - 1;
            }
        }
    }
    static uint32_t n_ops(const Txn &x) { return x.new_order ? 5 + 3 * x.ol : 7; }
    static uint32_t n_payload(const Txn &x) {
        return x.new_order ? LTPC_NO_NCOLS + LTPC_O_NCOLS + (LTPC_OL_NCOLS + 1) * x.ol : LTPC_H_NCOLS + 1;
    }
};

namespace {

uint32_t opw(uint32_t kind, uint32_t col, uint32_t table, int32_t imm) { return LTP_OPW(kind, col, table, imm); }

void put64(int32_t *p, int64_t v) {
    p[0] = (int32_t)(uint32_t)(uint64_t)v;
    p[1] = (int32_t)(uint32_t)((uint64_t)v >> 32);
}

}  // namespace

extern "C" {

int ltp_tpcc_create(const ltp_tpcc_params *p, ltp_tpcc **out) {
    if (!p || !out) return LTP_E_BADARG;
    *out = nullptr;
    if (p->warehouses == 0 || p->districts == 0 || p->customers == 0 || p->items == 0 || p->ol_min == 0 ||
        p->ol_min > p->ol_max || p->ol_max > kMaxLines)
        return LTP_E_BADARG;
    if ((uint64_t)p->warehouses * p->items > (1ull << 31) ||
        (uint64_t)p->warehouses * p->districts * p->customers > (1ull << 31))
        return LTP_E_CAPACITY;
    ltp_tpcc *g = new (std::nothrow) ltp_tpcc();
    if (!g) return LTP_E_NOMEM;
    g->p = *p;
    g->thr_no = ltp_rng::prob_threshold(p->new_order_frac);
    g->thr_rl = ltp_rng::prob_threshold(p->remote_line);
    g->thr_rp = ltp_rng::prob_threshold(p->remote_payment);
    g->thr_bn = ltp_rng::prob_threshold(p->by_last_name);
    // last-name index: per district and name, the middle customer (by id)
    // among those with that name -- position ceil(n/2) in 1-based terms
    const uint64_t nd = g->districts();
    g->by_name.assign(nd * kNames, -1);
    std::vector<uint32_t> cnt(kNames), seen(kNames);
    std::vector<int32_t> last(p->customers);
    for (uint64_t dist = 0; dist < nd; dist++) {
        std::fill(cnt.begin(), cnt.end(), 0u);
        std::fill(seen.begin(), seen.end(), 0u);
        for (uint32_t c = 0; c < p->customers; c++) {
            last[c] = g->c_last(dist * p->customers + c);
            cnt[last[c]]++;
        }
        int32_t *idx = &g->by_name[dist * kNames];
        for (uint32_t c = 0; c < p->customers; c++) {
            const int32_t L = last[c];
            if (seen[L]++ == (cnt[L] - 1) / 2) idx[L] = (int32_t)c;
        }
    }
    *out = g;
    return LTP_OK;
}

void ltp_tpcc_free(ltp_tpcc *g) { delete g; }

int ltp_tpcc_table(const ltp_tpcc *g, uint32_t table, ltp_schema *schema, uint64_t *rows) {
    if (!g || table >= LTP_TPCC_N_TABLES) return LTP_E_BADARG;
    if (schema) {
        memset(schema, 0, sizeof(*schema));
        schema->n_cols = kShape[table].n_cols;
        schema->wide_cols = kShape[table].wide;
    }
    if (rows) *rows = g->rows(table);
    return LTP_OK;
}

int ltp_tpcc_column(const ltp_tpcc *g, uint32_t table, uint32_t col, uint64_t row0, uint64_t n, void *dst) {
    if (!g || table >= LTP_TPCC_N_TABLES || col >= kShape[table].n_cols) return LTP_E_BADARG;
    const uint64_t rows = g->rows(table);
    if (row0 > rows || n > rows - row0 || (n && !dst)) return LTP_E_BADARG;
    const bool wide = (kShape[table].wide >> col) & 1ull;
    auto work = [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; i++) {
            const int64_t v = g->value(table, col, row0 + i);
            if (wide) ((int64_t *)dst)[i] = v;
            else ((int32_t *)dst)[i] = (int32_t)v;
        }
    };
    const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < (1u << 16) || nt == 1) {
        work(0, n);
    } else {
        std::vector<std::thread> th;
        const uint64_t chunk = (n + nt - 1) / nt;
        for (unsigned k = 0; k < nt; k++) {
            const uint64_t a = k * chunk, b = std::min<uint64_t>(n, a + chunk);
            if (a < b) th.emplace_back(work, a, b);
        }
        for (auto &x : th) x.join();
    }
    return LTP_OK;
}

int ltp_tpcc_gen(const ltp_tpcc *g, uint64_t batch, uint64_t n_txns, uint32_t *txn_first, uint64_t *keys,
                 uint32_t *opw_out, uint64_t cap_ops, int32_t *payload, uint64_t cap_payload, uint64_t *pay_first_out,
                 uint64_t *n_ops_out, uint64_t *n_payload_out, uint64_t *n_new_order, uint64_t *inserts,
                 int n_threads) {
    if (!g) return LTP_E_BADARG;
    const ltp_tpcc_params &p = g->p;
    const uint64_t tseed = p.seed ^ 0x54504343ull;
    // pass 1: sizes, from the first draws of every transaction's stream
    std::vector<uint64_t> pay_first(n_txns + 1);
    uint64_t ops = 0, pay = 0, no = 0, lines = 0;
    for (uint64_t t = 0; t < n_txns; t++) {
        Stream st{ltp_rng::txn_stream(tseed, batch, t)};
        ltp_tpcc::Txn x;
        g->draw(st, x, true);
        if (txn_first) txn_first[t] = (uint32_t)ops;
        pay_first[t] = pay;
        ops += ltp_tpcc::n_ops(x);
        pay += ltp_tpcc::n_payload(x);
        no += x.new_order ? 1 : 0;
        lines += x.ol;
        if (ops >= (1ull << 32)) return LTP_E_CAPACITY;
    }
    pay_first[n_txns] = pay;
    if (txn_first) txn_first[n_txns] = (uint32_t)ops;
    if (pay_first_out) memcpy(pay_first_out, pay_first.data(), (n_txns + 1) * sizeof(uint64_t));
    if (n_ops_out) *n_ops_out = ops;
    if (n_payload_out) *n_payload_out = pay;
    if (n_new_order) *n_new_order = no;
    if (inserts) {
        for (int k = 0; k < LTP_TPCC_N_TABLES; k++) inserts[k] = 0;
        inserts[LTP_TPCC_HISTORY] = n_txns - no;
        inserts[LTP_TPCC_NEW_ORDER] = no;
        inserts[LTP_TPCC_ORDER] = no;
        inserts[LTP_TPCC_ORDER_LINE] = lines;
    }
    if (!keys) return LTP_OK;
    if (!txn_first || !opw_out || !payload || ops > cap_ops || pay > cap_payload) return LTP_E_CAPACITY;
    const uint64_t D = p.districts, C = p.customers, I = p.items;
    auto work = [&](uint64_t t0, uint64_t t1) {
        for (uint64_t t = t0; t < t1; t++) {
            Stream st{ltp_rng::txn_stream(tseed, batch, t)};
            ltp_tpcc::Txn x;
            g->draw(st, x, false);
            uint64_t *k = keys + txn_first[t];
            uint32_t *w = opw_out + txn_first[t];
            int32_t *pl = payload + pay_first[t];
            uint64_t po = pay_first[t];
            const uint64_t dist = (uint64_t)x.w * D + x.d;
            if (x.new_order) {
                const uint64_t cust = dist * C + x.c;
                uint32_t all_local = 1;
                for (uint32_t l = 0; l < x.ol; l++) all_local &= x.supply[l] == x.w ? 1u : 0u;
                k[0] = x.w;
                w[0] = opw(LTP_OP_READ, LTPC_W_TAX, LTP_TPCC_WAREHOUSE, 0);
                k[1] = dist;
                w[1] = opw(LTP_OP_ADD, LTPC_D_NEXT_O_ID, LTP_TPCC_DISTRICT, 1);
                k[2] = cust;
                w[2] = opw(LTP_OP_READ, LTPC_C_DISCOUNT, LTP_TPCC_CUSTOMER, 0);
                // new-order row (its order id comes from op 1)
                k[3] = po;
                w[3] = LTP_INSERT_LINK(LTPC_NO_O_ID, LTP_TPCC_NEW_ORDER, 2);
                pl[LTPC_NO_O_ID] = 0;
                pl[LTPC_NO_D_ID] = (int32_t)x.d + 1;
                pl[LTPC_NO_W_ID] = (int32_t)x.w + 1;
                pl += LTPC_NO_NCOLS;
                po += LTPC_NO_NCOLS;
                // order row
                k[4] = po;
                w[4] = LTP_INSERT_LINK(LTPC_O_ID, LTP_TPCC_ORDER, 3);
                pl[LTPC_O_ID] = 0;
                pl[LTPC_O_D_ID] = (int32_t)x.d + 1;
                pl[LTPC_O_W_ID] = (int32_t)x.w + 1;
                pl[LTPC_O_C_ID] = (int32_t)x.c + 1;
                pl[LTPC_O_OL_CNT] = (int32_t)x.ol;
                pl[LTPC_O_ALL_LOCAL] = (int32_t)all_local;
                pl[LTPC_O_CARRIER_ID] = 0;
                pl += LTPC_O_NCOLS;
                po += LTPC_O_NCOLS;
                for (uint32_t l = 0; l < x.ol; l++) {
                    const uint32_t j = 5 + 3 * l;
                    const uint64_t srow = (uint64_t)x.supply[l] * I + x.item[l];
                    k[j] = po;
                    w[j] = LTP_INSERT_LINK(LTPC_OL_O_ID, LTP_TPCC_ORDER_LINE, j - 1);
                    // payload slots: one per int32 column, two for OL_AMOUNT
                    pl[0] = 0;
                    pl[1] = (int32_t)x.d + 1;
                    pl[2] = (int32_t)x.w + 1;
                    pl[3] = (int32_t)l + 1;
                    pl[4] = (int32_t)x.item[l] + 1;
                    pl[5] = (int32_t)x.supply[l] + 1;
                    pl[6] = (int32_t)x.qty[l];
                    put64(pl + 7, (int64_t)x.qty[l] * g->price(x.item[l]));
                    for (int q = 0; q < 6; q++) pl[9 + q] = g->text(LTP_TPCC_STOCK, srow, LTPC_S_DIST + q);
                    pl += LTPC_OL_NCOLS + 1;
                    po += LTPC_OL_NCOLS + 1;
                    k[j + 1] = srow;
                    w[j + 1] = opw(LTP_OP_ADD, LTPC_S_QUANTITY, LTP_TPCC_STOCK, -(int32_t)x.qty[l]);
                    k[j + 2] = srow;
                    w[j + 2] = opw(LTP_OP_ADD, LTPC_S_YTD, LTP_TPCC_STOCK, (int32_t)x.qty[l]);
                }
            } else {
                const uint64_t cust = ((uint64_t)x.cw * D + x.cd) * C + x.c;
                const int32_t h = (int32_t)x.amount;
                k[0] = x.w;
                w[0] = opw(LTP_OP_ADD, LTPC_W_YTD, LTP_TPCC_WAREHOUSE, h);
                k[1] = dist;
                w[1] = opw(LTP_OP_ADD, LTPC_D_YTD, LTP_TPCC_DISTRICT, h);
                k[2] = cust;
                w[2] = opw(LTP_OP_READ, LTPC_C_CREDIT, LTP_TPCC_CUSTOMER, 0);
                k[3] = cust;
                w[3] = opw(LTP_OP_ADD, LTPC_C_BALANCE, LTP_TPCC_CUSTOMER, -h);
                k[4] = cust;
                w[4] = opw(LTP_OP_ADD, LTPC_C_YTD_PAYMENT, LTP_TPCC_CUSTOMER, h);
                k[5] = cust;
                w[5] = opw(LTP_OP_ADD, LTPC_C_PAYMENT_CNT, LTP_TPCC_CUSTOMER, 1);
                k[6] = po;
                w[6] = opw(LTP_OP_INSERT, 0, LTP_TPCC_HISTORY, 0);
                pl[0] = (int32_t)x.c + 1;
                pl[1] = (int32_t)x.cd + 1;
                pl[2] = (int32_t)x.cw + 1;
                pl[3] = (int32_t)x.d + 1;
                pl[4] = (int32_t)x.w + 1;
                put64(pl + 5, h);
                // H_DATA: the first 12 bytes of W_NAME and of D_NAME
                for (int q = 0; q < 3; q++) {
                    pl[7 + q] = g->text(LTP_TPCC_WAREHOUSE, x.w, LTPC_W_NAME + q);
                    pl[10 + q] = g->text(LTP_TPCC_DISTRICT, dist, LTPC_D_NAME + q);
                }
            }
        }
    };
    unsigned nt = n_threads > 0 ? (unsigned)n_threads : std::max(1u, std::thread::hardware_concurrency());
    if (nt > 256) nt = 256;
    if (n_txns < 4096 || nt == 1) {
        work(0, n_txns);
    } else {
        std::vector<std::thread> th;
        const uint64_t chunk = (n_txns + nt - 1) / nt;
        for (unsigned k = 0; k < nt; k++) {
            const uint64_t a = k * chunk, b = std::min<uint64_t>(n_txns, a + chunk);
            if (a < b) th.emplace_back(work, a, b);
        }
        for (auto &x : th) x.join();
    }
    return LTP_OK;
}

}  // extern "C"
