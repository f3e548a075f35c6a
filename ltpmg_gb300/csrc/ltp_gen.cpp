// ltp_gen.cpp -- seeded, multi-threaded YCSB-style workload generator.
//
// Replaces the reference's host generator (Txn_Generator<YCSB_*>::
// generate_txn, src/txn_generator.cpp:601-673, and Query::generate_txn,
// src/query.cpp:270-311), which seeds rand() from the clock, shares it
// between threads and shuffles with a time-seeded engine, so no batch can be
// reproduced.  Here every transaction draws from its own SplitMix64 stream
// keyed by (seed, batch, transaction index), so any thread count yields the
// same batch, and the TID is the transaction's position in the batch (as the
// reference assigns TIDs after its shuffle).  Keys are distinct within a
// transaction (src/txn_generator.cpp:627-642).  Zipf keys are rank draws by
// rejection-inversion mapped through a seeded Feistel permutation of the row
// ids.
//
// Must be compiled with -ffp-contract=off: the sampler's double arithmetic
// has to give the same bits on every machine.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/ltpmg_gb300.h"
#include "ltp_rng.h"

namespace {

using ltp_rng::mix;
using ltp_rng::Stream;
using ltp_rng::txn_stream;

// Seeded permutation of [0, n): balanced 4-round Feistel network on the
// smallest even bit width >= log2(n), cycle-walking back into range.
struct Permutation {
    uint64_t n, mask;
    unsigned half;
    uint64_t k[4];
    Permutation(uint64_t seed, uint64_t n_) : n(n_) {
        unsigned bits = 2;
        while (bits < 64 && (1ULL << bits) < n) bits++;
        if (bits & 1) bits++;
        half = bits / 2;
        mask = (1ULL << half) - 1;
        for (int r = 0; r < 4; r++) k[r] = mix(seed ^ (0x5045524D00000000ULL + (uint64_t)r));
    }
    uint64_t operator()(uint64_t x) const {
        if (n <= 1) return 0;
        do {
            uint64_t L = x >> half, R = x & mask;
            for (int r = 0; r < 4; r++) {
                const uint64_t F = mix(R ^ k[r]) & mask;
                const uint64_t nl = R;
                R = L ^ F;
                L = nl;
            }
            x = (L << half) | R;
        } while (x >= n);
        return x;
    }
};

// Elementary functions in plain double arithmetic (identical bits on every
// machine): exp by Cody-Waite reduction with ln2 split into a high part
// exact in 32 bits and a low part, then a degree-15 Taylor polynomial; log
// by reducing the mantissa into [sqrt(1/2), sqrt(2)) and summing
// 2*atanh(s) = 2*(s + s^3/3 + s^5/5 + ...).
const double kLn2Hi = 6.93147180369123816490e-01;
const double kLn2Lo = 1.90821492927058770002e-10;

double dexp(double x) {
    if (x != x) return x;
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    const double kd = floor(x * 1.44269504088896338700e+00 + 0.5);
    const double r = (x - kd * kLn2Hi) - kd * kLn2Lo;
    static const double inv_fact[16] = {1.0,
                                        1.0,
                                        1.0 / 2,
                                        1.0 / 6,
                                        1.0 / 24,
                                        1.0 / 120,
                                        1.0 / 720,
                                        1.0 / 5040,
                                        1.0 / 40320,
                                        1.0 / 362880,
                                        1.0 / 3628800,
                                        1.0 / 39916800,
                                        1.0 / 479001600,
                                        1.0 / 6227020800.0,
                                        1.0 / 87178291200.0,
                                        1.0 / 1307674368000.0};
    double p = inv_fact[15];
    for (int i = 14; i >= 0; i--) p = p * r + inv_fact[i];
    return ldexp(p, (int)kd);
}

double dlog(double x) {
    if (x != x || x < 0) return NAN;
    if (x == 0) return -HUGE_VAL;
    if (isinf(x)) return x;
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0), z = s * s;
    double poly = 1.0 / 25.0;
    for (int k = 11; k >= 0; k--) poly = poly * z + 1.0 / (double)(2 * k + 1);
    return (double)e * kLn2Hi + ((double)e * kLn2Lo + 2.0 * s * poly);
}

double dlog1p(double x) {
    if (fabs(x) < 1e-5) return x * (1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x)));
    const double u = 1.0 + x;
    if (u == 1.0) return x;
    return dlog(u) * (x / (u - 1.0));
}

double dexpm1(double x) {
    if (fabs(x) < 1e-5) return x * (1.0 + x * (0.5 + x * (1.0 / 6.0 + x / 24.0)));
    const double u = dexp(x);
    if (u == 1.0) return x;
    const double um1 = u - 1.0;
    if (um1 == -1.0) return -1.0;
    return um1 * x / dlog(u);
}

// Zipf(theta) on {1..n}: rejection-inversion of Hoermann & Derflinger
// (ACM TOMACS 6(3), 1996) with H(x) = integral of x^-theta.
struct Zipf {
    double theta, hx1, hn, sdiv;
    uint64_t n;
    static double q1(double x) { return fabs(x) > 1e-8 ? dlog1p(x) / x : 1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x)); }
    static double q2(double x) {
        return fabs(x) > 1e-8 ? dexpm1(x) / x : 1.0 + x * 0.5 * (1.0 + x * (1.0 / 3.0) * (1.0 + 0.25 * x));
    }
    double H(double x) const {
        const double lx = dlog(x);
        return q2((1.0 - theta) * lx) * lx;
    }
    double h(double x) const { return dexp(-theta * dlog(x)); }
    double Hinv(double x) const {
        double t = x * (1.0 - theta);
        if (t < -1.0) t = -1.0;
        return dexp(q1(t) * x);
    }
    Zipf(uint64_t n_, double th) : theta(th), n(n_) {
        hx1 = H(1.5) - 1.0;
        hn = H((double)n + 0.5);
        sdiv = 2.0 - Hinv(H(2.5) - h(2.0));
    }
    uint64_t sample(Stream &st) const {
        for (;;) {
            const double u = hn + st.unit() * (hx1 - hn);
            const double x = Hinv(u);
            const double kd = floor(x + 0.5);
            uint64_t k = kd < 1.0 ? 1 : (kd > (double)n ? n : (uint64_t)kd);
            if ((double)k - x <= sdiv || u >= H((double)k + 0.5) - h((double)k)) return k;
        }
    }
};

}  // namespace

extern "C" {

int32_t ltp_table_value(uint64_t seed, uint64_t row, uint32_t col, uint32_t n_cols) {
    const uint64_t base = mix(seed ^ 0x5441424C45ULL);
    return (int32_t)(uint32_t)mix(base + row * (uint64_t)n_cols + col);
}

uint64_t ltp_gen_ycsb(const ltp_ycsb_params *p, uint64_t batch, uint64_t n_txns, uint32_t *txn_first, uint64_t *keys,
                      uint32_t *opw, uint64_t cap_ops, int n_threads) {
    if (!p || !txn_first || p->n_cols == 0 || p->n_cols > LTP_MAX_COLS || p->ops_min > p->ops_max ||
        p->n_rows < p->ops_max || p->n_rows == 0 || p->ops_max > 4096 || p->theta < 0)
        return UINT64_MAX;
    const uint64_t span = (uint64_t)(p->ops_max - p->ops_min) + 1;
    // pass 1: op counts (first draw of every transaction stream)
    uint64_t total = 0;
    for (uint64_t t = 0; t < n_txns; t++) {
        Stream st{txn_stream(p->seed, batch, t)};
        txn_first[t] = (uint32_t)total;
        total += p->ops_min + st.below(span);
        if (total > cap_ops || total >= (1ull << 32)) return UINT64_MAX;
    }
    txn_first[n_txns] = (uint32_t)total;
    if (total && (!keys || !opw)) return UINT64_MAX;
    const bool zipf = p->theta > 0.0;
    const Zipf Z(zipf ? p->n_rows : 2, zipf ? p->theta : 0.5);
    const Permutation perm(mix(p->seed ^ 0x5045524DULL), p->n_rows);
    const uint64_t thr = (uint64_t)(p->read_frac * 9007199254740992.0);
    const uint32_t imm = ((uint32_t)p->rmw_delta & 0xFFFFFu) << 12;
    auto work = [&](uint64_t t0, uint64_t t1) {
        for (uint64_t t = t0; t < t1; t++) {
            Stream st{txn_stream(p->seed, batch, t)};
            st.next();  // op count, consumed in pass 1
            const uint64_t at = txn_first[t];
            const uint32_t nops = txn_first[t + 1] - txn_first[t];
            for (uint32_t j = 0; j < nops; j++) {
                uint64_t key;
                bool dup;
                do {
                    key = zipf ? perm(Z.sample(st) - 1) : st.below(p->n_rows);
                    dup = false;
                    for (uint32_t q = 0; q < j; q++)
                        if (keys[at + q] == key) {
                            dup = true;
                            break;
                        }
                } while (dup);
                const bool is_read = (st.next() >> 11) < thr;
                const uint32_t col = (uint32_t)st.below(p->n_cols);
                keys[at + j] = key;
                opw[at + j] = is_read ? (LTP_OP_READ | (col << 2)) : (LTP_OP_ADD | (col << 2) | imm);
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
    return total;
}

}  // extern "C"
