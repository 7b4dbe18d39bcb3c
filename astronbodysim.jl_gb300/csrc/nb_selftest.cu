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
