// nb_noalloc.cu -- force evaluation that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: a Julia host whose device
// arrays all come from CUDA.jl's pooled allocator (memory taken behind the
// pool's back is invisible to it and can exhaust the device), or a serving
// process that reserves its whole HBM budget at start-up and must not see a
// later allocation fail or stall.  nb_force_noalloc serves them: the caller
// passes device arrays for the particles and for the results, and every
// intermediate buffer (Morton keys and permutation, radix-sort counts, packed
// FP32 tiles, tile origins, the device error word) lives in one file-scope
// __device__ array of fixed size, sized for systems of at most
// kNoAllocMaxParticles particles.
//
// Properties of that shared array:
//   * every GPU that loads this library holds it (about 2.7 MB) until exit;
//   * all calls share it and it keeps the last call's contents; each call
//     writes every byte it later reads, and clears the error word itself;
//   * calls whose work overlaps on the GPU (other streams, other host threads)
//     race on it and corrupt each other's results -- serialise them.
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current and caches it.  Every
// call reads the error word back and synchronises its stream, so no call can
// run inside a stream capture.  Later calls check the cached
// address with cudaPointerGetAttributes (no allocation) and repeat the set-up
// when it no longer names device memory of the current device -- after a
// cudaDeviceReset, which ends the context the address belonged to.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "nb_internal.cuh"

namespace {

constexpr int64_t kNoAllocMaxParticles = 65536;
constexpr int kTile = 256;
constexpr int kMaxDevices = 64;

constexpr size_t al256(size_t v) { return (v + 255) / 256 * 256; }

// Layout of the shared scratch for kNoAllocMaxParticles particles.
constexpr size_t kOffPerm = 0;
constexpr size_t kOffPack = kOffPerm + al256(sizeof(int32_t) * kNoAllocMaxParticles);
constexpr size_t kOffOrigin = kOffPack + al256(sizeof(float4) * kNoAllocMaxParticles);
constexpr size_t kOffExt = kOffOrigin + al256(sizeof(nb::TileOrigin) * (kNoAllocMaxParticles / kTile));
constexpr size_t kOffErr = kOffExt + al256(sizeof(float4) * (kNoAllocMaxParticles / kTile));
constexpr size_t kOffSort = kOffErr + 256;
// Upper bound of the radix-sort scratch for kNoAllocMaxParticles (two key
// buffers, one value buffer, 256 digit counts per 2048-particle block, bounding
// box partials); checked against nb::sort_scratch_bytes at set-up.
constexpr size_t kSortBytes = 2 * al256(8 * kNoAllocMaxParticles) +
                              al256(4 * kNoAllocMaxParticles) +
                              al256(4 * 256 * ((kNoAllocMaxParticles + 2047) / 2048)) +
                              al256(8 * 6 * 256) + al256(8 * 8) +
                              al256(4 * ((256 * ((kNoAllocMaxParticles + 2047) / 2048) + 4095) / 4096 + 1));
constexpr size_t kScratchBytes = kOffSort + kSortBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

void set_msg(char* buf, int64_t len, const char* msg) {
    if (!buf || len <= 0) return;
    std::snprintf(buf, (size_t)len, "nb_force_noalloc: %s", msg);
}

// True when p still names device memory of device dev (the cached scratch
// address of a context that has not been reset).
bool still_valid(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();  // clear the error the failed query recorded
        return false;
    }
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Device address of the shared scratch on the current device (set-up on first use).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_scratch_addr[dev] && !still_valid(g_scratch_addr[dev], dev)) g_scratch_addr[dev] = nullptr;
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int nb_force_noalloc(int64_t n, const double* x, const double* y, const double* z,
                                const double* m, int32_t law, double G, double softening,
                                double* ax, double* ay, double* az, double* pot, void* stream,
                                char* errbuf, int64_t errbuf_len) {
    if (errbuf && errbuf_len > 0) errbuf[0] = '\0';
    if (n < 1 || n > kNoAllocMaxParticles) {
        if (errbuf && errbuf_len > 0)
            std::snprintf(errbuf, (size_t)errbuf_len,
                          "nb_force_noalloc: %lld particles requested; this entry point handles "
                          "1..%lld (its scratch is a fixed %.1f MB device array); use a handle "
                          "(nb_create) for larger systems",
                          (long long)n, (long long)kNoAllocMaxParticles, kScratchBytes / 1.0e6);
        return NB_ERR_INVALID_ARG;
    }
    if (!x || !y || !z || !m || !ax || !ay || !az) {
        set_msg(errbuf, errbuf_len, "null particle or result array");
        return NB_ERR_INVALID_ARG;
    }
    if (law != NB_LAW_SPLINE_G2 && law != NB_LAW_PLUMMER) {
        set_msg(errbuf, errbuf_len, "unknown law");
        return NB_ERR_INVALID_ARG;
    }
    if (!(softening > 0.0) || softening != softening || softening > 1e300) {
        set_msg(errbuf, errbuf_len, "softening must be finite and > 0");
        return NB_ERR_INVALID_ARG;
    }
    if (nb::sort_scratch_bytes(kNoAllocMaxParticles) > kSortBytes) {
        set_msg(errbuf, errbuf_len, "internal scratch layout mismatch");
        return NB_ERR_STATE;
    }
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) {
        set_msg(errbuf, errbuf_len, cudaGetErrorString(e));
        return NB_ERR_CUDA;
    }
    char* b = static_cast<char*>(base);
    int32_t* perm = reinterpret_cast<int32_t*>(b + kOffPerm);
    float4* pack = reinterpret_cast<float4*>(b + kOffPack);
    nb::TileOrigin* origin = reinterpret_cast<nb::TileOrigin*>(b + kOffOrigin);
    float4* ext = reinterpret_cast<float4*>(b + kOffExt);
    uint32_t* err = reinterpret_cast<uint32_t*>(b + kOffErr);
    void* sort_scratch = b + kOffSort;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // The error word is the only state that must start at zero.
    e = cudaMemsetAsync(err, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess) e = nb::launch_morton_sort(x, y, z, n, sort_scratch, perm, s);
    if (e == cudaSuccess) e = nb::launch_pack(x, y, z, m, n, perm, kTile, pack, origin, ext, s);
    if (e == cudaSuccess) {
        nb::Sources32 src{pack, origin, ext, (int32_t)((n + kTile - 1) / kTile), kTile};
        nb::Targets tg{};
        tg.x = x;
        tg.y = y;
        tg.z = z;
        tg.type = nullptr;
        tg.idx = perm;
        tg.d_count = nullptr;
        tg.n = n;
        for (int k = 0; k < 6; ++k) tg.soft[k] = softening;
        tg.h_const = softening;
        tg.ax = ax;
        tg.ay = ay;
        tg.az = az;
        tg.pot = pot;
        tg.self_mass = m;
        e = nb::launch_force_mixed(law, pot != nullptr, src, tg, G, err, 128, 2, s);
    }
    uint32_t bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, err, sizeof bits, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_msg(errbuf, errbuf_len, cudaGetErrorString(e));
        return NB_ERR_CUDA;
    }
    if (bits & nb::DEVERR_TIMEOUT) {
        set_msg(errbuf, errbuf_len, "device wait timed out");
        return NB_ERR_TIMEOUT;
    }
    return NB_OK;
}
