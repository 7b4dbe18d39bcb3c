// nb_sort.cu -- spatial ordering of the sources for the mixed-precision force.
//
// The FP32 pair arithmetic works on coordinates relative to an FP64 origin per
// j-tile; its rounding error scales with the size of the tile.  Sorting the
// particles along a Morton (Z-order) curve makes every tile spatially compact,
// so close pairs are evaluated on small relative coordinates.
//
//   1. FP64 bounding box of all particles (two-stage min/max, deterministic);
//   2. 63-bit Morton key per particle (21 bits per axis over the box);
//   3. stable LSD radix sort of (key, index), 8-bit digits, 8 passes:
//      per-block digit histograms -> one exclusive scan -> stable scatter that
//      ranks equal digits by (round, warp, lane) order.
// The result is a deterministic permutation for given positions.
#include "nb_internal.cuh"

namespace nb {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;  // per thread
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kWarps = kSortThreads / 32;
constexpr int kBboxBlocks = 256;

int64_t sort_blocks(int64_t n) { return (n + kSortTile - 1) / kSortTile; }
int64_t scan_tmp_words(int64_t len);
cudaError_t launch_exclusive_scan2(uint32_t* counts, int64_t len, uint32_t* tmp, cudaStream_t s);

// Scratch layout (bytes) for n particles.
size_t sort_scratch_bytes(int64_t n) {
    const int64_t nb = sort_blocks(n);
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    return al(sizeof(uint64_t) * n) * 2 + al(sizeof(int32_t) * n) +
           al(sizeof(uint32_t) * (size_t)kRadix * nb) + al(sizeof(double) * 6 * kBboxBlocks) +
           al(sizeof(double) * 8) + al(sizeof(uint32_t) * (size_t)scan_tmp_words(kRadix * nb));
}

struct SortScratch {
    uint64_t* keys_a;
    uint64_t* keys_b;
    int32_t* vals_b;
    uint32_t* counts;
    double* bbox_part;
    double* bbox;
    uint32_t* scan_tmp;
};

static SortScratch carve(void* base, int64_t n) {
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    char* p = static_cast<char*>(base);
    SortScratch s;
    s.keys_a = (uint64_t*)p;
    p += al(sizeof(uint64_t) * n);
    s.keys_b = (uint64_t*)p;
    p += al(sizeof(uint64_t) * n);
    s.vals_b = (int32_t*)p;
    p += al(sizeof(int32_t) * n);
    s.counts = (uint32_t*)p;
    p += al(sizeof(uint32_t) * (size_t)kRadix * sort_blocks(n));
    s.bbox_part = (double*)p;
    p += al(sizeof(double) * 6 * kBboxBlocks);
    s.bbox = (double*)p;
    p += al(sizeof(double) * 8);
    s.scan_tmp = (uint32_t*)p;
    return s;
}

__global__ void __launch_bounds__(kSortThreads)
    k_bbox_partial(const double* __restrict__ x, const double* __restrict__ y,
                   const double* __restrict__ z, int64_t n, double* __restrict__ part) {
    __shared__ double red[6][kWarps];
    double v[6] = {1e300, 1e300, 1e300, 1e300, 1e300, 1e300};  // min x,y,z and min -x,-y,-z
    for (int64_t i = (int64_t)blockIdx.x * kSortThreads + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kSortThreads) {
        const double a = x[i], b = y[i], c = z[i];
        v[0] = fmin(v[0], a);
        v[1] = fmin(v[1], b);
        v[2] = fmin(v[2], c);
        v[3] = fmin(v[3], -a);
        v[4] = fmin(v[4], -b);
        v[5] = fmin(v[5], -c);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = fmin(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) red[k][threadIdx.x >> 5] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        double r = red[threadIdx.x][0];
        for (int w = 1; w < kWarps; ++w) r = fmin(r, red[threadIdx.x][w]);
        part[blockIdx.x * 6 + threadIdx.x] = r;
    }
}

__global__ void k_bbox_final(const double* __restrict__ part, int nblocks, double* __restrict__ bbox) {
    if (threadIdx.x < 6) {
        double r = part[threadIdx.x];
        for (int b = 1; b < nblocks; ++b) r = fmin(r, part[b * 6 + threadIdx.x]);
        bbox[threadIdx.x] = r;  // lo[0..2] = r[0..2], hi[k] = -r[3+k]
    }
}

__device__ __forceinline__ uint64_t spread3_21(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void k_morton(const double* __restrict__ x, const double* __restrict__ y,
                         const double* __restrict__ z, int64_t n, const double* __restrict__ bbox,
                         uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * kSortThreads + threadIdx.x;
    if (i >= n) return;
    const double lo[3] = {bbox[0], bbox[1], bbox[2]};
    const double hi[3] = {-bbox[3], -bbox[4], -bbox[5]};
    const double p[3] = {x[i], y[i], z[i]};
    uint64_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double ext = hi[k] - lo[k];
        double f = ext > 0.0 ? (p[k] - lo[k]) / ext : 0.0;
        f = fmin(fmax(f, 0.0), 1.0);
        q[k] = (uint64_t)(f * 2097151.0);
    }
    keys[i] = spread3_21(q[0]) | (spread3_21(q[1]) << 1) | (spread3_21(q[2]) << 2);
    vals[i] = (int32_t)i;
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int shift, int nblocks,
                 uint32_t* __restrict__ counts) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of len counts with one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ c, int64_t len) {
    __shared__ uint32_t part[1024];
    const int64_t per = (len + 1023) / 1024;
    const int64_t b = threadIdx.x * per;
    const int64_t e = min(len, b + per);
    uint32_t s = 0;
    for (int64_t i = b; i < e; ++i) s += c[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;  // exclusive
    for (int64_t i = b; i < e; ++i) {
        const uint32_t v = c[i];
        c[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_scatter(const uint64_t* __restrict__ kin, const int32_t* __restrict__ vin,
                    uint64_t* __restrict__ kout, int32_t* __restrict__ vout, int64_t n, int shift,
                    int nblocks, const uint32_t* __restrict__ offs) {
    __shared__ uint32_t wcnt[kWarps][kRadix + 1];
    __shared__ uint32_t wbase[kWarps][kRadix + 1];
    __shared__ uint32_t run[kRadix];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    run[tid] = offs[(int64_t)tid * nblocks + blockIdx.x];
    for (int w = 0; w < kWarps; ++w) wcnt[w][tid] = 0;
    if (tid < kWarps) wcnt[tid][kRadix] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    const uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = base + r * kSortThreads + tid;
        const bool valid = i < n;
        uint64_t key = 0;
        int32_t val = 0;
        uint32_t d = kRadix;  // sentinel bin for lanes past the end
        if (valid) {
            key = kin[i];
            val = vin ? vin[i] : (int32_t)i;
            d = (uint32_t)((key >> shift) & (kRadix - 1));
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt);
        if (lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = run[tid];
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = wcnt[w][tid];
                wbase[w][tid] = acc;
                acc += c;
                wcnt[w][tid] = 0;
            }
            run[tid] = acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wbase[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        if (tid < kWarps) wcnt[tid][kRadix] = 0;
        __syncthreads();
    }
}

// Multi-CTA exclusive scan for long arrays: each CTA sums a chunk of
// kScanChunk counts, one CTA scans the chunk sums, each CTA rescans its chunk
// from its offset.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanChunk = kScanThreads * kScanPer;
constexpr int64_t kScanMaxChunks = 1024;  // chunk sums scanned by one k_scan CTA

__global__ void __launch_bounds__(kScanThreads)
    k_scan_chunk_sums(const uint32_t* __restrict__ c, int64_t len, uint32_t* __restrict__ sums) {
    const int64_t b = (int64_t)blockIdx.x * kScanChunk;
    uint32_t s = 0;
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        const int64_t j = b + i;
        if (j < len) s += c[j];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ uint32_t w[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int k = 0; k < kScanThreads / 32; ++k) t += w[k];
        sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kScanThreads)
    k_scan_chunk_apply(uint32_t* __restrict__ c, int64_t len, const uint32_t* __restrict__ offs) {
    __shared__ uint32_t part[kScanThreads];
    const int64_t b = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        const int64_t j = b + k;
        v[k] = j < len ? c[j] : 0u;
        s += v[k];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {
        const uint32_t t = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = offs[blockIdx.x] + part[threadIdx.x] - s;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        const int64_t j = b + k;
        if (j < len) c[j] = run;
        run += v[k];
    }
}

// Exclusive prefix sum of len 32-bit counts in place.  `tmp` (may be null for
// len <= kScanChunk * 4) holds scan_tmp_words(len) words.
int64_t scan_tmp_words(int64_t len) { return (len + kScanChunk - 1) / kScanChunk + 1; }

cudaError_t launch_exclusive_scan2(uint32_t* counts, int64_t len, uint32_t* tmp, cudaStream_t s) {
    if (len <= 0) return cudaSuccess;
    const int64_t nchunks = (len + kScanChunk - 1) / kScanChunk;
    if (!tmp || nchunks <= 4 || nchunks > kScanMaxChunks * kScanChunk) {
        k_scan<<<1, 1024, 0, s>>>(counts, len);
        return cudaGetLastError();
    }
    k_scan_chunk_sums<<<(unsigned)nchunks, kScanThreads, 0, s>>>(counts, len, tmp);
    k_scan<<<1, 1024, 0, s>>>(tmp, nchunks);
    k_scan_chunk_apply<<<(unsigned)nchunks, kScanThreads, 0, s>>>(counts, len, tmp);
    return cudaGetLastError();
}

// Exclusive prefix sum of len 32-bit counts in place (one CTA of 1024 threads).
cudaError_t launch_exclusive_scan(uint32_t* counts, int64_t len, cudaStream_t s) {
    if (len <= 0) return cudaSuccess;
    k_scan<<<1, 1024, 0, s>>>(counts, len);
    return cudaGetLastError();
}

// Key buffer inside a sort scratch of sort_scratch_bytes(n) bytes.
uint64_t* sort_keys_buffer(void* scratch, int64_t n) { return carve(scratch, n).keys_a; }

// Stable LSD radix sort of (keys, vals): keys in sort_keys_buffer(scratch, n),
// vals (n int32) in place; `passes` 8-bit digits from the bottom (even).
cudaError_t launch_sort_keys(void* scratch, int64_t n, int32_t* vals, int passes, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    SortScratch sc = carve(scratch, n);
    const int nblocks = (int)sort_blocks(n);
    cudaError_t e = cudaSuccess;
    uint64_t* kin = sc.keys_a;
    uint64_t* kout = sc.keys_b;
    int32_t* vin = vals;
    int32_t* vout = sc.vals_b;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * kRadixBits;
        k_radix_hist<<<nblocks, kSortThreads, 0, s>>>(kin, n, shift, nblocks, sc.counts);
        e = launch_exclusive_scan2(sc.counts, (int64_t)kRadix * nblocks, sc.scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_radix_scatter<<<nblocks, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, nblocks,
                                                         sc.counts);
        uint64_t* tk = kin;
        kin = kout;
        kout = tk;
        int32_t* tv = vin;
        vin = vout;
        vout = tv;
    }
    // After an even number of passes the sorted values are back in vals.
    return cudaGetLastError();
}

// Computes perm[0..n) = particle indices in Morton order of (x, y, z).
cudaError_t launch_morton_sort(const double* x, const double* y, const double* z, int64_t n,
                               void* scratch, int32_t* perm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    SortScratch sc = carve(scratch, n);
    int64_t gb = (n + kSortThreads - 1) / kSortThreads;
    const int bb = (int)(gb < kBboxBlocks ? gb : kBboxBlocks);
    k_bbox_partial<<<bb, kSortThreads, 0, s>>>(x, y, z, n, sc.bbox_part);
    k_bbox_final<<<1, 32, 0, s>>>(sc.bbox_part, bb, sc.bbox);
    k_morton<<<(unsigned)gb, kSortThreads, 0, s>>>(x, y, z, n, sc.bbox, sc.keys_a, perm);
    return launch_sort_keys(scratch, n, perm, 8, s);
}

}  // namespace nb
