// ltp_rng.h -- the generators' shared random streams: SplitMix64 finaliser
// and per-(seed, batch, transaction) streams, so that a batch is the same
// for any thread count and on any machine.
#pragma once
#include <stdint.h>

namespace ltp_rng {

inline uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Stream {
    uint64_t s;
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ULL;
        return mix(s);
    }
    // uniform on [0, n) by a 64x64 -> 128-bit multiply
    uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
    // uniform on [lo, hi]
    uint64_t range(uint64_t lo, uint64_t hi) { return lo + below(hi - lo + 1); }
    double unit() { return (double)(next() >> 11) * 0x1.0p-53; }
    // true with probability thr / 2^53 (thr from prob_threshold)
    bool chance(uint64_t thr) { return (next() >> 11) < thr; }
};

inline uint64_t prob_threshold(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return 1ULL << 53;
    return (uint64_t)(p * 9007199254740992.0);
}

inline uint64_t txn_stream(uint64_t seed, uint64_t batch, uint64_t txn) {
    const uint64_t s = mix(seed ^ mix(batch + 0x4241544348ULL));
    return mix(s + (txn + 1) * 0x9E3779B97F4A7C15ULL);
}

}  // namespace ltp_rng
