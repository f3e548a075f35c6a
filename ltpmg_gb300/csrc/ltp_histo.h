// ltp_histo.h -- latency histogram of the serving loops.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace ltp {

// Latency histogram without floating point: 64 linear sub-buckets per
// power of two of nanoseconds (~1.6% wide).
struct Histo {
    static constexpr int kSub = 64;
    std::vector<uint64_t> h = std::vector<uint64_t>(64 * kSub, 0);
    uint64_t n = 0, mx = 0;
    double sum = 0;
    static int bucket(uint64_t ns) {
        if (ns < kSub) return (int)ns;
        const int e = 63 - __builtin_clzll(ns);  // >= 6
        return e * kSub + (int)((ns >> (e - 6)) & (kSub - 1));
    }
    static double lower(int b) {
        const int e = b / kSub, m = b % kSub;
        if (e < 6) return (double)b;
        return std::ldexp(1.0 + m / (double)kSub, e);
    }
    void add(uint64_t ns) {
        h[bucket(ns)]++;
        n++;
        sum += (double)ns;
        mx = std::max(mx, ns);
    }
    static uint64_t lower_ns(int b) {  // smallest latency in bucket b
        const int e = b / kSub, m = b % kSub;
        return e < 6 ? (uint64_t)b : (uint64_t)(kSub + m) << (e - 6);
    }
    // Adds done - arr[i] for i in [a, b) with arr non-decreasing and at most
    // done (so the latencies fall along the range): one binary search per
    // bucket the range spans instead of one step per request.  The sum takes
    // each bucket's middle request as the bucket's mean.
    void add_sorted(uint64_t done, const uint64_t *arr, uint64_t a, uint64_t b) {
        if (a >= b) return;
        mx = std::max(mx, done - arr[a]);
        n += b - a;
        for (uint64_t i = a; i < b;) {
            const int bk = bucket(done - arr[i]);
            const uint64_t j = (uint64_t)(std::upper_bound(arr + i, arr + b, done - lower_ns(bk)) - arr);
            h[bk] += j - i;
            sum += (double)(j - i) * (double)(done - arr[i + (j - i) / 2]);
            i = j;
        }
    }
    void remove(uint64_t ns) {
        h[bucket(ns)]--;
        n--;
        sum -= (double)ns;
    }
    double pct(double p) const {
        if (!n) return 0;
        const uint64_t want = (uint64_t)std::ceil(p * (double)n);
        uint64_t acc = 0;
        for (size_t b = 0; b < h.size(); b++) {
            acc += h[b];
            if (acc >= want) return std::min(lower((int)b + 1), (double)mx);
        }
        return (double)mx;
    }
};

}  // namespace ltp
