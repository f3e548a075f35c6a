// Checks the serving loops' latency histogram: adding a sorted run of
// arrivals with one binary search per bucket (Histo::add_sorted) must give
// the same buckets, count and maximum as adding every latency one by one,
// and its mean within 0.5%.  Prints "ok" or the first difference.
#include <stdio.h>

#include <random>
#include <vector>

#include "../../ltpmg_gb300/csrc/ltp_histo.h"

int main() {
    std::mt19937_64 rng(7);
    for (int trial = 0; trial < 200; trial++) {
        const uint64_t n = 1 + rng() % 20000;
        std::vector<uint64_t> arr(n);
        uint64_t t = rng() % 1000;
        const double rate = 1e-3 * (1 + rng() % 5000);  // arrivals per ns
        std::exponential_distribution<double> gap(rate);
        for (auto &a : arr) {
            t += (uint64_t)gap(rng);
            a = t;
        }
        const uint64_t done = t + rng() % 3000000;
        ltp::Histo bulk, each;
        const uint64_t a = rng() % n, b = a + rng() % (n - a + 1);
        bulk.add_sorted(done, arr.data(), a, b);
        for (uint64_t i = a; i < b; i++) each.add(done - arr[i]);
        // taking one latency out again (an aborted request)
        if (b > a) {
            const uint64_t k = a + rng() % (b - a);
            bulk.remove(done - arr[k]);
            each.remove(done - arr[k]);
        }
        if (bulk.h != each.h || bulk.n != each.n || (b > a && bulk.mx != each.mx)) {
            printf("trial %d: buckets, count or max differ (n %llu)\n", trial, (unsigned long long)n);
            return 1;
        }
        const double m1 = bulk.n ? bulk.sum / bulk.n : 0, m2 = each.n ? each.sum / each.n : 0;
        if (m2 > 0 && (m1 - m2 > 0.005 * m2 || m2 - m1 > 0.005 * m2)) {
            printf("trial %d: mean %.1f vs %.1f\n", trial, m1, m2);
            return 1;
        }
        for (double p : {0.5, 0.99, 0.999})
            if (bulk.pct(p) != each.pct(p)) {
                printf("trial %d: percentile %.3f differs\n", trial, p);
                return 1;
            }
    }
    printf("ok\n");
    return 0;
}
