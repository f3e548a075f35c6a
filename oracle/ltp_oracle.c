/*
 * ltp_oracle.c -- CPU oracle for the batched transaction-processing hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see ltp_oracle.h): the checker for the CUDA path
 * and the CPU baseline.  The shipped library never links or calls it.
 *
 * Parity unpinned for the replay values: the reference has no known-answer
 * tests for execution and its update operators are identity
 * (cuda/src/gpulauncher.cu:79-103).  The replay restates the reference's
 * ordering rule -- all operations on a row execute in ascending TID order,
 * nothing aborts (register_cc gpulauncher.cu:382-418, filter_commit
 * :2439-2523 which sorts each row's bucket by TID, commit :2525-2671 which
 * applies them in that order) -- with the read-modify-write semantics made
 * real (+imm, two's-complement wrap).
 *
 * Must be compiled with -ffp-contract=off so that the double arithmetic of
 * the Zipf sampler gives the same bits on x86-64 and aarch64.
 */
#include "ltp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------- */
/* SplitMix64 (Steele, Lea & Flood 2014): finaliser and sequence.          */
uint64_t ltpo_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static inline uint64_t next_u64(uint64_t *s) {
    *s += 0x9E3779B97F4A7C15ULL;
    return ltpo_mix64(*s);
}

static inline uint64_t below(uint64_t x, uint64_t n) { /* multiply-shift range map */
    return (uint64_t)(((unsigned __int128)x * n) >> 64);
}

static inline double unit_double(uint64_t x) { return (double)(x >> 11) * 0x1.0p-53; }

/* Independent stream per (batch, transaction): generation can run in any
 * order or in parallel and still give identical batches. */
uint64_t ltpo_stream_seed(uint64_t seed, uint64_t batch, uint64_t txn) {
    uint64_t s = ltpo_mix64(seed ^ ltpo_mix64(batch + 0x4241544348ULL));
    return ltpo_mix64(s + (txn + 1) * 0x9E3779B97F4A7C15ULL);
}

/* Seeded bijection of [0, n): 4-round balanced Feistel network on the
 * smallest even bit width covering n, cycle-walking back into range. */
uint64_t ltpo_feistel_perm(uint64_t seed, uint64_t n, uint64_t x) {
    if (n <= 1) return 0;
    unsigned bits = 2;
    while (bits < 64 && (1ULL << bits) < n) bits++;
    if (bits & 1) bits++;
    unsigned half = bits / 2;
    uint64_t mask = (1ULL << half) - 1;
    uint64_t k[4];
    for (int r = 0; r < 4; r++) k[r] = ltpo_mix64(seed ^ (0x5045524D00000000ULL + (uint64_t)r));
    do {
        uint64_t L = x >> half, R = x & mask;
        for (int r = 0; r < 4; r++) {
            uint64_t F = ltpo_mix64(R ^ k[r]) & mask;
            uint64_t nl = R;
            R = L ^ F;
            L = nl;
        }
        x = (L << half) | R;
    } while (x >= n);
    return x;
}

/* ---------------------------------------------------------------------- */
/* Deterministic elementary functions in plain IEEE double arithmetic, so the
 * generator is bit-identical across machines and C libraries.
 * exp: Cody-Waite reduction by ln2 (split in a 32-bit-exact high part and a
 * low part) and a degree-15 Taylor polynomial; log: reduction of the mantissa
 * to [sqrt(1/2), sqrt(2)) and the series 2*atanh(s).  Both are accurate to a
 * few ulp, which is all the sampler needs; what matters is that every
 * machine computes the same bits. */
static const double LN2_HI = 6.93147180369123816490e-01;
static const double LN2_LO = 1.90821492927058770002e-10;
static const double INV_LN2 = 1.44269504088896338700e+00;

double ltpo_det_exp(double x) {
    if (x != x) return x;
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    double kd = floor(x * INV_LN2 + 0.5);
    int k = (int)kd;
    double r = (x - kd * LN2_HI) - kd * LN2_LO;
    double p = 1.0 / 1307674368000.0; /* 1/15! */
    static const double inv_fact[15] = {
        1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040, 1.0 / 40320,
        1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800, 1.0 / 479001600, 1.0 / 6227020800.0,
        1.0 / 87178291200.0};
    for (int i = 14; i >= 0; i--) p = p * r + inv_fact[i];
    return ldexp(p, k);
}

double ltpo_det_log(double x) {
    if (x != x || x < 0) return NAN;
    if (x == 0) return -HUGE_VAL;
    if (isinf(x)) return x;
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double z = s * s;
    double poly = 1.0 / 25.0;
    for (int k = 11; k >= 0; k--) poly = poly * z + 1.0 / (double)(2 * k + 1);
    double lm = 2.0 * s * poly;
    return (double)e * LN2_HI + ((double)e * LN2_LO + lm);
}

static double det_log1p(double x) {
    if (fabs(x) < 1e-5) return x * (1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x)));
    double u = 1.0 + x;
    if (u == 1.0) return x;
    return ltpo_det_log(u) * (x / (u - 1.0));
}

static double det_expm1(double x) {
    if (fabs(x) < 1e-5) return x * (1.0 + x * (0.5 + x * (1.0 / 6.0 + x / 24.0)));
    double u = ltpo_det_exp(x);
    if (u == 1.0) return x;
    double um1 = u - 1.0;
    if (um1 == -1.0) return -1.0;
    return um1 * x / ltpo_det_log(u);
}

/* ---------------------------------------------------------------------- */
/* Zipf(theta) on {1..n} by rejection-inversion (W. Hoermann, G. Derflinger,
 * "Rejection-inversion to generate variates from monotone discrete
 * distributions", ACM TOMACS 6(3), 1996).  H is the integral of x^-theta,
 * h the density; samples are exact draws from P(k) ~ k^-theta. */
typedef struct {
    double theta, hx1, hn, sdiv;
    uint64_t n;
} zipf_t;

static double zh_helper1(double x) { return fabs(x) > 1e-8 ? det_log1p(x) / x : 1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x)); }
static double zh_helper2(double x) {
    return fabs(x) > 1e-8 ? det_expm1(x) / x : 1.0 + x * 0.5 * (1.0 + x * (1.0 / 3.0) * (1.0 + 0.25 * x));
}
static double zH(const zipf_t *z, double x) {
    double lx = ltpo_det_log(x);
    return zh_helper2((1.0 - z->theta) * lx) * lx;
}
static double zh(const zipf_t *z, double x) { return ltpo_det_exp(-z->theta * ltpo_det_log(x)); }
static double zHinv(const zipf_t *z, double x) {
    double t = x * (1.0 - z->theta);
    if (t < -1.0) t = -1.0;
    return ltpo_det_exp(zh_helper1(t) * x);
}
static void zipf_setup(zipf_t *z, uint64_t n, double theta) {
    z->theta = theta;
    z->n = n;
    z->hx1 = zH(z, 1.5) - 1.0;
    z->hn = zH(z, (double)n + 0.5);
    z->sdiv = 2.0 - zHinv(z, zH(z, 2.5) - zh(z, 2.0));
}
static uint64_t zipf_sample(const zipf_t *z, uint64_t *st) {
    for (;;) {
        double u = z->hn + unit_double(next_u64(st)) * (z->hx1 - z->hn);
        double x = zHinv(z, u);
        double kd = floor(x + 0.5);
        uint64_t k;
        if (kd < 1.0) k = 1;
        else if (kd > (double)z->n) k = z->n;
        else k = (uint64_t)kd;
        if ((double)k - x <= z->sdiv || u >= zH(z, (double)k + 0.5) - zh(z, (double)k)) return k;
    }
}

uint64_t ltpo_zipf_draw(uint64_t n, double theta, uint64_t *state) {
    zipf_t z;
    zipf_setup(&z, n, theta);
    return zipf_sample(&z, state);
}

/* ---------------------------------------------------------------------- */
int32_t ltpo_table_value(uint64_t seed, uint64_t row, uint32_t col, uint32_t n_cols) {
    uint64_t base = ltpo_mix64(seed ^ 0x5441424C45ULL);
    return (int32_t)(uint32_t)ltpo_mix64(base + row * (uint64_t)n_cols + col);
}

void ltpo_table_init(uint64_t seed, uint64_t n_rows, uint32_t n_cols, int32_t *tab) {
    for (uint32_t c = 0; c < n_cols; c++)
        for (uint64_t r = 0; r < n_rows; r++) tab[(uint64_t)c * n_rows + r] = ltpo_table_value(seed, r, c, n_cols);
}

/* Transaction t of batch b: op count, then per op a key (redrawn until it
 * differs from the transaction's earlier keys, as the reference generator
 * does at src/txn_generator.cpp:627-642), a read/RMW coin and a column. */
uint64_t ltpo_gen_ycsb_batch(const ltpo_ycsb_params *p, uint64_t batch, uint64_t n_txns, uint32_t *txn_first,
                             uint64_t *keys, uint32_t *opw, uint64_t cap_ops) {
    if (p->n_rows < p->ops_max || p->ops_min > p->ops_max || p->n_cols == 0 || p->n_cols > 64) return UINT64_MAX;
    zipf_t z;
    int use_zipf = p->theta > 0.0;
    if (use_zipf) zipf_setup(&z, p->n_rows, p->theta);
    uint64_t perm_seed = ltpo_mix64(p->seed ^ 0x5045524DULL);
    uint64_t thr = (uint64_t)(p->read_frac * 9007199254740992.0);
    uint64_t span = (uint64_t)(p->ops_max - p->ops_min) + 1;
    uint64_t at = 0;
    for (uint64_t t = 0; t < n_txns; t++) {
        uint64_t st = ltpo_stream_seed(p->seed, batch, t);
        uint32_t nops = p->ops_min + (uint32_t)below(next_u64(&st), span);
        if (at + nops > cap_ops) return UINT64_MAX;
        txn_first[t] = (uint32_t)at;
        for (uint32_t j = 0; j < nops; j++) {
            uint64_t key;
            int dup;
            do {
                if (use_zipf) key = ltpo_feistel_perm(perm_seed, p->n_rows, zipf_sample(&z, &st) - 1);
                else key = below(next_u64(&st), p->n_rows);
                dup = 0;
                for (uint32_t q = 0; q < j; q++)
                    if (keys[at + q] == key) { dup = 1; break; }
            } while (dup);
            int is_read = (next_u64(&st) >> 11) < thr;
            uint32_t col = (uint32_t)below(next_u64(&st), p->n_cols);
            keys[at + j] = key;
            opw[at + j] = is_read ? LTPO_OPW(0, col, 0, 0) : LTPO_OPW(1, col, 0, (uint32_t)p->rmw_delta & 0xFFFFFu);
        }
        at += nops;
    }
    txn_first[n_txns] = (uint32_t)at;
    return at;
}

/* ---------------------------------------------------------------------- */
/* Serial replay.                                                          */
static int check_op(uint64_t n_rows, uint32_t n_cols, uint64_t key, uint32_t w) {
    if (key >= n_rows) return -1;
    if (LTPO_COL(w) >= n_cols) return -1;
    if (LTPO_KIND(w) > 1) return -1;
    if (LTPO_TABLE(w) != 0) return -1;
    return 0;
}

static inline void apply(int32_t *tab, uint64_t n_rows, uint64_t key, uint32_t w, int32_t *out) {
    int32_t *cell = &tab[(uint64_t)LTPO_COL(w) * n_rows + key];
    int32_t v = *cell;
    if (LTPO_KIND(w) == 1) {
        v = (int32_t)((uint32_t)v + (uint32_t)LTPO_IMM(w));
        *cell = v;
    }
    *out = v;
}

/* Minimal open-addressing map cell -> minimum writer TID (rule 1). */
typedef struct {
    uint64_t *key;
    uint32_t *val;
    uint64_t mask;
} minmap_t;

static int minmap_init(minmap_t *m, uint64_t n) {
    uint64_t cap = 16;
    while (cap < 2 * n + 16) cap <<= 1;
    m->key = (uint64_t *)malloc(cap * sizeof(uint64_t));
    m->val = (uint32_t *)malloc(cap * sizeof(uint32_t));
    if (!m->key || !m->val) return -1;
    memset(m->key, 0xFF, cap * sizeof(uint64_t));
    m->mask = cap - 1;
    return 0;
}
static uint32_t *minmap_slot(minmap_t *m, uint64_t k, int create) {
    uint64_t h = ltpo_mix64(k) & m->mask;
    for (;;) {
        if (m->key[h] == k) return &m->val[h];
        if (m->key[h] == UINT64_MAX) {
            if (!create) return NULL;
            m->key[h] = k;
            m->val[h] = UINT32_MAX;
            return &m->val[h];
        }
        h = (h + 1) & m->mask;
    }
}

int ltpo_replay(int rule, uint64_t n_rows, uint32_t n_cols, int32_t *tab, uint64_t n_txns, const uint32_t *txn_first,
                const uint64_t *keys, const uint32_t *opw, uint8_t *commit, int32_t *out) {
    uint64_t n_ops = txn_first[n_txns];
    for (uint64_t i = 0; i < n_ops; i++)
        if (check_op(n_rows, n_cols, keys[i], opw[i])) return -1;
    if (rule == 0) {
        for (uint64_t t = 0; t < n_txns; t++) {
            commit[t] = 1;
            for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) apply(tab, n_rows, keys[i], opw[i], &out[i]);
        }
        return 0;
    }
    if (rule != 1) return -1;
    minmap_t m;
    if (minmap_init(&m, n_ops)) return -1;
    for (uint64_t t = 0; t < n_txns; t++)
        for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++)
            if (LTPO_KIND(opw[i]) != 0) {
                uint32_t *v = minmap_slot(&m, keys[i] * n_cols + LTPO_COL(opw[i]), 1);
                if ((uint32_t)t < *v) *v = (uint32_t)t;
            }
    for (uint64_t t = 0; t < n_txns; t++) {
        uint8_t ok = 1;
        for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) {
            uint32_t *v = minmap_slot(&m, keys[i] * n_cols + LTPO_COL(opw[i]), 0);
            if (v && *v < (uint32_t)t) ok = 0;
        }
        commit[t] = ok;
    }
    free(m.key);
    free(m.val);
    for (uint64_t t = 0; t < n_txns; t++)
        for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) {
            if (commit[t]) apply(tab, n_rows, keys[i], opw[i], &out[i]);
            else out[i] = 0;
        }
    return 0;
}

typedef struct {
    uint64_t n_rows, n_txns;
    uint32_t n_cols;
    int32_t *tab;
    const uint32_t *txn_first;
    const uint64_t *keys;
    const uint32_t *opw;
    int32_t *out;
    int tid, nth;
} mt_arg_t;

static void *mt_worker(void *vp) {
    mt_arg_t *a = (mt_arg_t *)vp;
    uint64_t n_ops = a->txn_first[a->n_txns];
    for (uint64_t i = 0; i < n_ops; i++) {
        uint64_t cell = a->keys[i] * a->n_cols + LTPO_COL(a->opw[i]);
        if ((int)(ltpo_mix64(cell) % (uint64_t)a->nth) != a->tid) continue;
        apply(a->tab, a->n_rows, a->keys[i], a->opw[i], &a->out[i]);
    }
    return NULL;
}

int ltpo_replay_r0_mt(uint64_t n_rows, uint32_t n_cols, int32_t *tab, uint64_t n_txns, const uint32_t *txn_first,
                      const uint64_t *keys, const uint32_t *opw, uint8_t *commit, int32_t *out, int n_threads) {
    uint64_t n_ops = txn_first[n_txns];
    for (uint64_t i = 0; i < n_ops; i++)
        if (check_op(n_rows, n_cols, keys[i], opw[i])) return -1;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    pthread_t th[256];
    mt_arg_t args[256];
    for (int k = 0; k < n_threads; k++) {
        mt_arg_t a = {n_rows, n_txns, n_cols, tab, txn_first, keys, opw, out, k, n_threads};
        args[k] = a;
        if (pthread_create(&th[k], NULL, mt_worker, &args[k])) return -1;
    }
    for (int k = 0; k < n_threads; k++) pthread_join(th[k], NULL);
    memset(commit, 1, n_txns);
    return 0;
}

/* General replay: several tables, inserts.  The same serial rule as
 * ltpo_replay; inserts never conflict (a new row cannot be named by another
 * op of the same batch) and take the next slot of their table in serial
 * order, which is "table count + rank among earlier committed inserts". */
static uint32_t popc64(uint64_t x) {
    uint32_t n = 0;
    while (x) {
        x &= x - 1;
        n++;
    }
    return n;
}

static int col_is_wide(const ltpo_table *t, uint32_t c) { return (int)((t->wide >> c) & 1u); }

static int64_t cell_get(const ltpo_table *t, uint32_t c, uint64_t row) {
    return col_is_wide(t, c) ? ((int64_t *)t->cols[c])[row] : (int64_t)((int32_t *)t->cols[c])[row];
}

static void cell_set(ltpo_table *t, uint32_t c, uint64_t row, int64_t v) {
    if (col_is_wide(t, c)) ((int64_t *)t->cols[c])[row] = v;
    else ((int32_t *)t->cols[c])[row] = (int32_t)(uint32_t)(uint64_t)v;
}

/* Checks op i of transaction t (ops [first, end)). */
static int check_op_t(uint32_t n_tables, const ltpo_table *T, uint64_t i, uint64_t first, const uint64_t *keys,
                      const uint32_t *opw, uint64_t payload_len) {
    const uint32_t w = opw[i], tb = LTPO_TABLE(w), kind = LTPO_KIND(w);
    if (tb >= n_tables) return -1;
    if (kind == 2) {
        const uint64_t slots = T[tb].n_cols + popc64(T[tb].wide);
        const uint32_t d = (uint32_t)LTPO_IMM(w) & 0x3FFu;
        if (keys[i] + slots > payload_len) return -1;
        if (d && (LTPO_COL(w) >= T[tb].n_cols || d > i - first || LTPO_KIND(opw[i - d]) > 1)) return -1;
        return 0;
    }
    if (kind > 2) return -1;
    if (keys[i] >= T[tb].n_rows || LTPO_COL(w) >= T[tb].n_cols) return -1;
    return 0;
}

int ltpo_replay_tables(int rule, uint32_t n_tables, ltpo_table *T, uint64_t n_txns, const uint32_t *txn_first,
                       const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                       uint8_t *commit, int64_t *out) {
    const uint64_t n_ops = txn_first[n_txns];
    uint64_t ins[16] = {0};
    for (uint64_t t = 0; t < n_txns; t++)
        for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) {
            if (check_op_t(n_tables, T, i, txn_first[t], keys, opw, payload_len)) return -1;
            if (LTPO_KIND(opw[i]) == 2) ins[LTPO_TABLE(opw[i])]++;
        }
    for (uint32_t k = 0; k < n_tables && k < 16; k++)
        if (T[k].n_rows + ins[k] > T[k].rows_cap) return -2;
    if (rule != 0 && rule != 1) return -1;
    for (uint64_t t = 0; t < n_txns; t++) commit[t] = 1;
    if (rule == 1) {
        /* cells are (table, row, col); key them as one 64-bit id per table */
        minmap_t m;
        if (minmap_init(&m, n_ops)) return -1;
        for (uint64_t t = 0; t < n_txns; t++)
            for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++)
                if (LTPO_KIND(opw[i]) == 1) {
                    const uint32_t tb = LTPO_TABLE(opw[i]);
                    uint64_t cid = ((uint64_t)tb << 58) | (keys[i] * T[tb].n_cols + LTPO_COL(opw[i]));
                    uint32_t *v = minmap_slot(&m, cid, 1);
                    if ((uint32_t)t < *v) *v = (uint32_t)t;
                }
        for (uint64_t t = 0; t < n_txns; t++)
            for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) {
                if (LTPO_KIND(opw[i]) == 2) continue;
                const uint32_t tb = LTPO_TABLE(opw[i]);
                uint64_t cid = ((uint64_t)tb << 58) | (keys[i] * T[tb].n_cols + LTPO_COL(opw[i]));
                uint32_t *v = minmap_slot(&m, cid, 0);
                if (v && *v < (uint32_t)t) commit[t] = 0;
            }
        free(m.key);
        free(m.val);
    }
    for (uint64_t t = 0; t < n_txns; t++)
        for (uint64_t i = txn_first[t]; i < txn_first[t + 1]; i++) {
            const uint32_t w = opw[i], tb = LTPO_TABLE(w);
            ltpo_table *tab = &T[tb];
            if (!commit[t]) {
                out[i] = 0;
                continue;
            }
            if (LTPO_KIND(w) == 2) {
                const uint64_t slot = tab->n_rows++;
                const uint32_t d = (uint32_t)LTPO_IMM(w) & 0x3FFu;
                uint64_t p = keys[i];
                for (uint32_t c = 0; c < tab->n_cols; c++) {
                    int64_t v;
                    if (col_is_wide(tab, c)) {
                        v = (int64_t)(((uint64_t)(uint32_t)payload[p + 1] << 32) | (uint64_t)(uint32_t)payload[p]);
                        p += 2;
                    } else {
                        v = payload[p];
                        p += 1;
                    }
                    if (d && c == LTPO_COL(w)) v = out[i - d];
                    cell_set(tab, c, slot, v);
                }
                out[i] = (int64_t)slot;
                continue;
            }
            const uint32_t c = LTPO_COL(w);
            int64_t v = cell_get(tab, c, keys[i]);
            if (LTPO_KIND(w) == 1) {
                v = (int64_t)((uint64_t)v + (uint64_t)(int64_t)LTPO_IMM(w));
                cell_set(tab, c, keys[i], v);
                v = cell_get(tab, c, keys[i]); /* wrapped at the column's width */
            }
            out[i] = v;
        }
    return 0;
}

/* Ordered-rule (R0) replay of ltpo_replay_tables on n_threads threads:
 * phase 1 splits reads and RMWs by cell (each thread walks the whole batch
 * in order and executes the ops of the cells it owns), phase 2 splits
 * inserts by table (they only need phase 1's outputs for their links).
 * Results equal ltpo_replay_tables(0, ...); the multi-core CPU baseline. */
typedef struct {
    uint32_t n_tables;
    ltpo_table *T;
    uint64_t n_txns;
    const uint32_t *txn_first;
    const uint64_t *keys;
    const uint32_t *opw;
    const int32_t *payload;
    uint64_t payload_len;
    int64_t *out;
    int k, n;
    int err;
} mtt_arg_t;

static uint32_t owner_of(uint32_t tb, uint64_t cell, int n) {
    return (uint32_t)((((cell + 1) * 0x9E3779B97F4A7C15ULL) ^ ((uint64_t)tb << 59)) >> 40) % (uint32_t)n;
}

static void *mtt_cells(void *p) {
    mtt_arg_t *a = (mtt_arg_t *)p;
    const uint64_t n_ops = a->txn_first[a->n_txns];
    for (uint64_t i = 0; i < n_ops; i++) {
        const uint32_t w = a->opw[i], tb = LTPO_TABLE(w);
        if (LTPO_KIND(w) == 2) continue;
        if (tb >= a->n_tables || LTPO_KIND(w) > 2) {
            a->err = 1;
            continue;
        }
        ltpo_table *tab = &a->T[tb];
        const uint32_t c = LTPO_COL(w);
        const uint64_t r = a->keys[i];
        if (owner_of(tb, r * tab->n_cols + c, a->n) != (uint32_t)a->k) continue;
        if (r >= tab->n_rows || c >= tab->n_cols) {
            a->err = 1;
            continue;
        }
        int64_t v = cell_get(tab, c, r);
        if (LTPO_KIND(w) == 1) {
            v = (int64_t)((uint64_t)v + (uint64_t)(int64_t)LTPO_IMM(w));
            cell_set(tab, c, r, v);
            v = cell_get(tab, c, r);
        }
        a->out[i] = v;
    }
    return NULL;
}

static void *mtt_inserts(void *p) {
    mtt_arg_t *a = (mtt_arg_t *)p;
    for (uint64_t t = 0; t < a->n_txns; t++)
        for (uint64_t i = a->txn_first[t]; i < a->txn_first[t + 1]; i++) {
            const uint32_t w = a->opw[i], tb = LTPO_TABLE(w);
            if (LTPO_KIND(w) != 2 || tb % (uint32_t)a->n != (uint32_t)a->k) continue;
            if (check_op_t(a->n_tables, a->T, i, a->txn_first[t], a->keys, a->opw, a->payload_len)) {
                a->err = 1;
                continue;
            }
            ltpo_table *tab = &a->T[tb];
            if (tab->n_rows >= tab->rows_cap) {
                a->err = 2;
                continue;
            }
            const uint64_t slot = tab->n_rows++;
            const uint32_t d = (uint32_t)LTPO_IMM(w) & 0x3FFu;
            uint64_t q = a->keys[i];
            for (uint32_t c = 0; c < tab->n_cols; c++) {
                int64_t v;
                if (col_is_wide(tab, c)) {
                    v = (int64_t)(((uint64_t)(uint32_t)a->payload[q + 1] << 32) | (uint64_t)(uint32_t)a->payload[q]);
                    q += 2;
                } else {
                    v = a->payload[q];
                    q += 1;
                }
                if (d && c == LTPO_COL(w)) v = a->out[i - d];
                cell_set(tab, c, slot, v);
            }
            a->out[i] = (int64_t)slot;
        }
    return NULL;
}

int ltpo_replay_tables_r0_mt(uint32_t n_tables, ltpo_table *T, uint64_t n_txns, const uint32_t *txn_first,
                             const uint64_t *keys, const uint32_t *opw, const int32_t *payload, uint64_t payload_len,
                             uint8_t *commit, int64_t *out, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    pthread_t th[256];
    mtt_arg_t args[256];
    int err = 0;
    for (int phase = 0; phase < 2; phase++) {
        const int nt = phase == 0 ? n_threads : (n_threads < (int)n_tables ? n_threads : (int)(n_tables ? n_tables : 1));
        for (int k = 0; k < nt; k++) {
            mtt_arg_t a = {n_tables, T, n_txns, txn_first, keys, opw, payload, payload_len, out, k, nt, 0};
            args[k] = a;
            if (pthread_create(&th[k], NULL, phase == 0 ? mtt_cells : mtt_inserts, &args[k])) return -1;
        }
        for (int k = 0; k < nt; k++) {
            pthread_join(th[k], NULL);
            if (args[k].err) err = args[k].err;
        }
        if (err) return err == 2 ? -2 : -1;
    }
    memset(commit, 1, n_txns);
    return 0;
}

uint64_t ltpo_fnv1a(const void *data, uint64_t bytes) {
    const uint8_t *p = (const uint8_t *)data;
    uint64_t h = 0xCBF29CE484222325ULL;
    for (uint64_t i = 0; i < bytes; i++) {
        h ^= p[i];
        h *= 0x100000001B3ULL;
    }
    return h;
}

/* ---------------------------------------------------------------------- */
/* Restatements of the reference generator pieces (pinned by tests/golden). */
uint32_t ltpo_ref_zipf_table(uint64_t n, double s, double *cdf_out) {
    /* src/random.cpp:105-137: normaliser over all n ranks, cumulative sum of
     * the first min(n,100) terms, stopping once it reaches 1. */
    double zipf = 0.0;
    for (uint64_t i = 1; i <= n; ++i) zipf += 1 / pow((double)(uint32_t)i, s);
    double tmp = 0.0;
    uint32_t size = n < 100 ? (uint32_t)n : 100, len = 0;
    for (uint32_t i = 1; i <= size; ++i) {
        tmp += 1 / pow(i, s) / zipf;
        cdf_out[len++] = tmp;
        if (tmp >= 1.0) break;
    }
    return len;
}

uint32_t ltpo_ref_zipf_pick(const double *cdf, uint32_t len, uint32_t r100, uint32_t tail) {
    /* src/random.cpp:140-161: a 1/100-resolution uniform draw looked up in the
     * table; past the table the rank comes from the uniform tail draw. */
    double u = r100 / 100.0;
    for (uint32_t i = 0; i < len; ++i)
        if (u < cdf[i]) return i;
    return tail;
}

uint64_t ltpo_ref_nurand(uint64_t A, uint64_t x, uint64_t y, uint64_t r_a, uint64_t r_xy) {
    (void)A;
    return (r_a | r_xy) % (y - x + 1) + x;
}

uint32_t ltpo_ref_ycsb_op_type(uint32_t variant, uint32_t i) {
    switch (variant) {
    case 0: return i < 5 ? 0u : 2u;            /* YCSB_A: 5 selects, 5 updates */
    case 1: case 3: return i < 9 ? 0u : 2u;    /* YCSB_B, YCSB_D: 9 selects, 1 update */
    case 2: return 0u;                          /* YCSB_C: read only */
    case 4: return i < 9 ? 4u : 1u;            /* YCSB_E: 9 scans, 1 insert */
    default: return 0xFFFFFFFFu;
    }
}
