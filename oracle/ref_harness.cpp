// ref_harness.cpp -- extern "C" probes into the reference's own host
// generator code (src/random.cpp), compiled together with it by
// oracle/build_ref.sh into oracle/_ref/.  TEST INFRASTRUCTURE ONLY: it exists
// to produce the golden vectors under tests/golden/ that pin the oracle's
// restatements of the reference generator.
#include <cstdint>
#include <cstdlib>
#include <iostream>

#include "common.h"  // pulls in every standard header first
#define private public  // read Random::zipfian_distribution (src/random.cpp:105-137)
#include "random.h"
#undef private

extern "C" {

// Cumulative table built by Random::init_rand_zipf(n, s).
uint32_t ref_zipf_table(uint64_t n, double s, double *out, uint32_t cap) {
    Random rnd;
    std::cout.setstate(std::ios::failbit);  // init_rand_zipf prints the table
    rnd.init_rand_zipf(n, s);
    std::cout.clear();
    uint32_t len = 0;
    for (double v : rnd.zipfian_distribution) {
        if (len < cap) out[len] = v;
        len++;
    }
    return len;
}

// K draws of Random::rand_zipf(0, n-1) after srand(seed), plus the raw libc
// rand() stream re-read from the same seed so that the draws each sample
// consumed can be matched up by the test.
void ref_zipf_trace(uint32_t seed, uint64_t n, double s, uint32_t K, uint32_t *result, uint32_t *raw, uint32_t raw_cap) {
    Random rnd;
    std::cout.setstate(std::ios::failbit);
    rnd.init_rand_zipf(n, s);
    std::cout.clear();
    srand(seed);
    for (uint32_t k = 0; k < K; k++) result[k] = rnd.rand_zipf(0, n - 1);
    srand(seed);
    for (uint32_t k = 0; k < raw_cap; k++) raw[k] = (uint32_t)rand();
}

// K draws of Random::non_uniform_distribution(A, x, y) (NURand) after
// srand(seed), plus the raw rand() stream from the same seed.
void ref_nurand_trace(uint32_t seed, uint64_t A, uint64_t x, uint64_t y, uint32_t K, uint64_t *result, uint32_t *raw,
                      uint32_t raw_cap) {
    Random rnd;
    srand(seed);
    for (uint32_t k = 0; k < K; k++) result[k] = rnd.non_uniform_distribution(A, x, y);
    srand(seed);
    for (uint32_t k = 0; k < raw_cap; k++) raw[k] = (uint32_t)rand();
}
}
