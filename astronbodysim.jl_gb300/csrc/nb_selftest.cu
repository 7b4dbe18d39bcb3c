// nb_selftest.cu -- exercises the bounded-wait path that every mbarrier wait
// of the force kernels takes, without any fault: one warp waits on an
// mbarrier that nothing arrives on, gives up after the limit, records
// DEVERR_TIMEOUT in a device error word and returns.  The host reads the word;
// the context stays usable.
#include <cstdio>

#include "nb_internal.cuh"

namespace {

__global__ void k_wait_nothing(uint64_t timeout_ns, uint32_t* err, unsigned long long* waited_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        nb::mbar_init(&bar, 1);  // expects one arrival that never comes
        nb::fence_mbar_init();
    }
    __syncthreads();
    const uint64_t t0 = nb::globaltimer_ns();
    const bool ok = __all_sync(0xffffffffu, nb::mbar_wait_bounded(&bar, 0u, timeout_ns));
    if (threadIdx.x == 0) {
        *waited_ns = (unsigned long long)(nb::globaltimer_ns() - t0);
        if (!ok) atomicOr(err, nb::DEVERR_TIMEOUT);
    }
}

}  // namespace

extern "C" int nb_selftest_wait_timeout(int device, int64_t timeout_ns, double* waited_ms) {
    if (timeout_ns <= 0 || timeout_ns > 2000000000LL) return NB_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return NB_ERR_CUDA;
    void* mem = nullptr;
    if (cudaMalloc(&mem, 64) != cudaSuccess) return NB_ERR_OOM;
    uint32_t* err = static_cast<uint32_t*>(mem);
    unsigned long long* waited = reinterpret_cast<unsigned long long*>(static_cast<char*>(mem) + 8);
    cudaMemset(mem, 0, 64);
    k_wait_nothing<<<1, 32>>>((uint64_t)timeout_ns, err, waited);
    cudaError_t e = cudaDeviceSynchronize();
    uint32_t bits = 0;
    unsigned long long ns = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&bits, err, sizeof bits, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&ns, waited, sizeof ns, cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return NB_ERR_CUDA;
    if (waited_ms) *waited_ms = (double)ns * 1e-6;
    return (bits & nb::DEVERR_TIMEOUT) ? NB_ERR_TIMEOUT : NB_OK;
}

// ---------------------------------------------------------------------------
// FP32 throughput probe: the denominator of the force kernel's roofline,
// measured instead of assumed.  Every thread runs 8 independent dependency
// chains a = a * b + c (scalar fma.rn.f32, or packed fma.rn.f32x2 on float2),
// so the FMA pipe, not latency, bounds the rate.  Grid: 4 CTAs of 256 threads
// per SM.  The chains stay finite (|b| < 1); one thread stores a value that
// depends on every chain so nothing is dead code.
// ---------------------------------------------------------------------------
namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakChains = 8;

__global__ void __launch_bounds__(kPeakThreads) k_fma_scalar(int iters, float b, float c,
                                                              float* sink) {
    float a[kPeakChains];
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int k = 0; k < kPeakChains; ++k) a[k] = __fmaf_rn(a[k], b, c);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) s += a[k];
    if (s == 12345.0f) *sink = s;  // never true for these inputs; keeps the chains live
}

__global__ void __launch_bounds__(kPeakThreads) k_fma_packed(int iters, float b, float c,
                                                              float* sink) {
    float2 a[kPeakChains];
    const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k)
        a[k] = make_float2((float)(threadIdx.x + k) * 1e-3f, (float)(threadIdx.x - k) * 1e-3f);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int k = 0; k < kPeakChains; ++k) a[k] = __ffma2_rn(a[k], b2, c2);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) s += a[k].x + a[k].y;
    if (s == 12345.0f) *sink = s;
}

}  // namespace

extern "C" int nb_selftest_fp32_peak(int device, int packed, double* tflops, double* ms) {
    if (cudaSetDevice(device) != cudaSuccess) return NB_ERR_CUDA;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return NB_ERR_CUDA;
    float* sink = nullptr;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) return NB_ERR_OOM;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int grid = 4 * nsm;
    const int iters = 4096;  // x 16 x 8 chains per thread
    const double lanes_per_op = packed ? 2.0 : 1.0;
    const double flop = 2.0 * lanes_per_op * (double)grid * kPeakThreads * iters * 16.0 * kPeakChains;
    float best = 1e30f;
    cudaError_t e = cudaSuccess;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0);
        if (packed)
            k_fma_packed<<<grid, kPeakThreads>>>(iters, 0.9999f, 1e-4f, sink);
        else
            k_fma_scalar<<<grid, kPeakThreads>>>(iters, 0.9999f, 1e-4f, sink);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && t < best) best = t;  // first launch is the warm-up
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return NB_ERR_CUDA;
    if (ms) *ms = best;
    if (tflops) *tflops = flop / (best * 1e-3) / 1e12;
    return NB_OK;
}
