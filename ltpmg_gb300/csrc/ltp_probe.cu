// ltp_probe.cu -- random-access ceilings of the GPU, for the roofline of the
// batch kernels.  Their ops touch random cells and random conflict words, so
// what bounds them is the rate of random 4-byte loads and atomics, not the
// copy bandwidth: each random 4-byte access moves a whole 32-byte sector.
// The probe runs one kernel of independent random accesses over an array of
// the given size (a table-sized array lives in HBM, a conflict-word-sized
// one in L2) and reports accesses per second.
//
// A measurement tool for the benchmark, not part of the product: it builds
// into its own library (libltpmg_probe.so), outside libltpmg_gb300.so and
// its C ABI.
//
//   int ltp_probe_random_access(int32_t device, uint64_t bytes, int32_t mode,
//                               double *accesses_per_s);
//
// bytes: 4 KB .. 16 GB; mode 0 loads, 1 atomicOr with its result used,
// 2 atomicOr as a reduction.  Returns 0, or a negative status as the
// product's (-4 bad argument, -6 no memory, -1 CUDA error).
#include <cuda_runtime.h>
#include <stdint.h>

#define LTP_PROBE_LOAD 0
#define LTP_PROBE_ATOMIC 1
#define LTP_PROBE_REDUCE 2
#define LTP_OK 0
#define LTP_E_CUDA (-1)
#define LTP_E_BADARG (-4)
#define LTP_E_NOMEM (-6)

namespace {

__device__ __forceinline__ uint32_t probe_hash(uint64_t x) {  // splitmix64 finaliser
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (uint32_t)x;
}

// Each thread issues `per_thread` accesses in groups of 8 independent ones.
template <int MODE>
__global__ void k_probe(uint32_t *a, uint32_t n, uint32_t per_thread, uint64_t seed, uint32_t *sink) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t acc = 0;
    for (uint32_t it = 0; it < per_thread; it += 8) {
        uint32_t v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint32_t idx = probe_hash(seed ^ (t * 0x9E3779B97F4A7C15ull + it + j)) % n;
            if (MODE == LTP_PROBE_LOAD) v[j] = __ldcg(&a[idx]);
            else if (MODE == LTP_PROBE_ATOMIC) v[j] = atomicOr(&a[idx], 1u << j);
            else {
                atomicOr(&a[idx], 1u << j);  // result unused: a reduction
                v[j] = 0;
            }
        }
#pragma unroll
        for (int j = 0; j < 8; j++) acc += v[j];
    }
    if (acc == 0x9E3779B9u) sink[0] = acc;  // keeps the loads live
}

}  // namespace

extern "C" int ltp_probe_random_access(int32_t device, uint64_t bytes, int32_t mode, double *accesses_per_s) {
    if (!accesses_per_s || bytes < 4096 || bytes >= (16ull << 30) || mode < 0 || mode > 2) return LTP_E_BADARG;
    if (cudaSetDevice(device) != cudaSuccess) return LTP_E_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return LTP_E_CUDA;
    const uint32_t n = (uint32_t)(bytes / 4), threads = 256, blocks = (uint32_t)sms * 8, per_thread = 256;
    uint32_t *a = nullptr, *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = LTP_OK;
    float best = 1e30f;
    if (cudaMalloc((void **)&a, (size_t)n * 4) != cudaSuccess || cudaMalloc((void **)&sink, 4) != cudaSuccess ||
        cudaMemset(a, 0, (size_t)n * 4) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rc = LTP_E_CUDA;
    } else {
        for (int rep = 0; rep < 4 && rc == LTP_OK; rep++) {  // the first run warms up; the best of the rest counts
            cudaEventRecord(e0);
            if (mode == LTP_PROBE_LOAD) k_probe<LTP_PROBE_LOAD><<<blocks, threads>>>(a, n, per_thread, rep, sink);
            else if (mode == LTP_PROBE_ATOMIC) k_probe<LTP_PROBE_ATOMIC><<<blocks, threads>>>(a, n, per_thread, rep, sink);
            else k_probe<LTP_PROBE_REDUCE><<<blocks, threads>>>(a, n, per_thread, rep, sink);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                rc = LTP_E_CUDA;
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep && ms < best) best = ms;
        }
    }
    if (rc == LTP_OK) *accesses_per_s = (double)blocks * threads * per_thread / (best * 1e-3);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(sink);
    return rc;
}
