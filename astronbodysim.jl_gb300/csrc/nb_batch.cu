// nb_batch.cu -- kernels of the many-system engine (nb_engine.cu).
//
// Many independent systems live in one particle arena; system slot s owns a
// contiguous range of arena particles, and every particle carries its slot
// (sysid, -1 for free space).  The running systems are ranked 0..R-1; a step
// of the engine is
//   drift -> Morton order per system (small systems in shared memory at
//   admission and every 64 of their own steps; large ones by a radix sort of
//   their own particles every step) -> per-system packed FP32 tiles -> force
//   over whole i-blocks with the kick in its epilogue -> step counter.
// The force kernel never splits an i-block and a system's order depends only
// on its own particles, so a system's trajectory is bit-identical whether it
// runs alone or among others.
#include <algorithm>

#include "nb_pairs.cuh"

namespace nb {

constexpr int kBThreads = 256;

// gridDim.y limit: launches over the large systems go in slabs of this many.
constexpr int32_t kMaxGridY = 65535;

// BatchSys (per rank, device memory): aoff = first arena particle, soff =
// first slot of the large systems' sort (compact over the large systems),
// n = particles, slot = system slot.

// Order-preserving unsigned image of a double (for atomicMin over boxes).
__device__ __forceinline__ unsigned long long ord_key(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_value(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// Box of each large system: blockIdx.y = large index (box_key[6 * it ..]),
// blockIdx.x = chunk of kBThreads * 4 particles; minima of (x, y, z, -x, -y,
// -z) by atomicMin, so the box does not depend on the order of the CTAs.
__global__ void __launch_bounds__(kBThreads)
    k_batch_large_box(const BatchSys* __restrict__ bs, const int32_t* __restrict__ ranks, int32_t y0,
                      const double* __restrict__ x, const double* __restrict__ y,
                      const double* __restrict__ z, unsigned long long* __restrict__ box_key) {
    __shared__ double red[6][kBThreads / 32];
    const int32_t lr = y0 + (int32_t)blockIdx.y;
    const int32_t r = ranks[lr];
    const BatchSys d = bs[r];
    const int64_t i0 = (int64_t)blockIdx.x * kBThreads * 4;
    if (i0 >= d.n) return;  // CTA-uniform
    double v[6] = {1e300, 1e300, 1e300, 1e300, 1e300, 1e300};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t i = i0 + u * kBThreads + threadIdx.x;
        if (i < d.n) {
            const int64_t p = d.aoff + i;
            const double a = x[p], b = y[p], c = z[p];
            v[0] = fmin(v[0], a);
            v[1] = fmin(v[1], b);
            v[2] = fmin(v[2], c);
            v[3] = fmin(v[3], -a);
            v[4] = fmin(v[4], -b);
            v[5] = fmin(v[5], -c);
        }
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
        double m = red[threadIdx.x][0];
        for (int w = 1; w < kBThreads / 32; ++w) m = fmin(m, red[threadIdx.x][w]);
        atomicMin(&box_key[(int64_t)lr * 6 + threadIdx.x], ord_key(m));
    }
}

// Spreads the low 14 bits of v to every third bit (bits 0, 3, ..., 39).
__device__ __forceinline__ uint64_t spread3_14(uint64_t v) {
    v &= 0x3fffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// key = large index << 42 | Morton code (14 bits per axis over the system's
// box), at the system's compact offset; vals = arena index.  Within a system
// the input is in arena order, so the stable sort breaks ties by it.
__global__ void __launch_bounds__(kBThreads)
    k_batch_large_keys(const BatchSys* __restrict__ bs, const int32_t* __restrict__ ranks, int32_t y0,
                       const unsigned long long* __restrict__ box_key, const double* __restrict__ x,
                       const double* __restrict__ y, const double* __restrict__ z,
                       uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    const int32_t lr = y0 + (int32_t)blockIdx.y;
    const int32_t r = ranks[lr];
    const BatchSys d = bs[r];
    const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
    if (i >= d.n) return;
    const int64_t p = d.aoff + i;
    const double pp[3] = {x[p], y[p], z[p]};
    uint64_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double lo = ord_value(box_key[(int64_t)lr * 6 + k]),
                     hi = -ord_value(box_key[(int64_t)lr * 6 + 3 + k]);
        const double ext = hi - lo;
        double f = ext > 0.0 ? (pp[k] - lo) / ext : 0.0;
        f = fmin(fmax(f, 0.0), 1.0);
        q[k] = (uint64_t)(f * 16383.0);
    }
    keys[d.soff + i] = ((uint64_t)lr << 42) | spread3_14(q[0]) | (spread3_14(q[1]) << 1) |
                       (spread3_14(q[2]) << 2);
    vals[d.soff + i] = (int32_t)p;
}

// Systems of at most kSmallSort particles are ordered by one CTA each, in
// shared memory: FP64 bounding box, 14-bit-per-axis Morton code, bitonic sort
// of (code << 14 | local index), written to lperm[aoff .. aoff + n) as local
// indices.  Keys are unique, so the order depends only on the system's own
// positions.
constexpr int kSmallSort = 16384;
constexpr int kSortCta = 1024;

__global__ void __launch_bounds__(kSortCta)
    k_batch_sort_small(const BatchSys* __restrict__ bs, const int64_t* __restrict__ steps_slot,
                       const int64_t* __restrict__ nsteps_slot, int32_t every, int32_t force_all,
                       const double* __restrict__ x,
                       const double* __restrict__ y, const double* __restrict__ z,
                       double* __restrict__ bbox, int32_t* __restrict__ lperm) {
    extern __shared__ uint64_t sk[];
    __shared__ double red[6][kSortCta / 32];
    const BatchSys d = bs[blockIdx.x];
    if (d.n > kSmallSort) return;  // ordered by the global radix sort
    // Re-ordered at admission and every `every` of the system's own steps, so
    // the schedule does not depend on the other systems.
    if (!force_all && steps_slot[d.slot] % every != 0) return;
    // a system that has made all its steps keeps its order (and positions)
    if (!force_all && nsteps_slot && steps_slot[d.slot] >= nsteps_slot[d.slot]) return;
    const int tid = threadIdx.x;
    double v[6] = {1e300, 1e300, 1e300, 1e300, 1e300, 1e300};
    for (int i = tid; i < d.n; i += kSortCta) {
        const int64_t p = d.aoff + i;
        const double a = x[p], b = y[p], c = z[p];
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
    if ((tid & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) red[k][tid >> 5] = v[k];
    __syncthreads();
    double lo[3], inv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double a = red[k][0], b = red[k + 3][0];
        for (int w = 1; w < kSortCta / 32; ++w) {
            a = fmin(a, red[k][w]);
            b = fmin(b, red[k + 3][w]);
        }
        lo[k] = a;
        const double ext = -b - a;
        inv[k] = ext > 0.0 ? 16383.0 / ext : 0.0;
    }
    (void)bbox;
    int np2 = 1;
    while (np2 < d.n) np2 <<= 1;
    for (int i = tid; i < np2; i += kSortCta) {
        uint64_t key = ~0ull;
        if (i < d.n) {
            const int64_t p = d.aoff + i;
            const double q[3] = {x[p], y[p], z[p]};
            uint64_t c[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double f = (q[k] - lo[k]) * inv[k];
                f = fmin(fmax(f, 0.0), 16383.0);
                c[k] = (uint64_t)f;
            }
            key = ((spread3_14(c[0]) | (spread3_14(c[1]) << 1) | (spread3_14(c[2]) << 2)) << 14) |
                  (uint64_t)i;
        }
        sk[i] = key;
    }
    __syncthreads();
    for (int k = 2; k <= np2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < np2; i += kSortCta) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = sk[i], b = sk[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        sk[i] = b;
                        sk[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < d.n; i += kSortCta) lperm[d.aoff + i] = (int32_t)(sk[i] & 0x3fffull);
}

// Radix-sort result of the large systems as arena-relative local order:
// lperm[aoff + k] = perm[soff + k] - aoff (grid: chunks x large index).
__global__ void __launch_bounds__(kBThreads)
    k_batch_perm_to_local(const BatchSys* __restrict__ bs, const int32_t* __restrict__ ranks, int32_t y0,
                          const int32_t* __restrict__ perm, int32_t* __restrict__ lperm) {
    const BatchSys d = bs[ranks[y0 + (int32_t)blockIdx.y]];
    const int64_t k = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
    if (k < d.n) lperm[d.aoff + k] = (int32_t)(perm[d.soff + k] - d.aoff);
}

// A system whose count has reached its target (nsteps_slot) stops counting.
__global__ void k_batch_tick(const BatchSys* __restrict__ bs, int32_t nrank,
                             int64_t* __restrict__ steps_slot,
                             const int64_t* __restrict__ nsteps_slot) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrank) return;
    const int32_t s = bs[r].slot;
    if (!nsteps_slot || steps_slot[s] < nsteps_slot[s]) steps_slot[s] += 1;
}

int batch_small_sort_limit() { return kSmallSort; }

cudaError_t prepare_batch_sort_small() {
    return cudaFuncSetAttribute(k_batch_sort_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(uint64_t) * kSmallSort));
}

cudaError_t launch_batch_sort_small(const BatchSys* bs, int32_t nrank, int32_t max_small_n,
                                    const int64_t* steps_slot, const int64_t* nsteps_slot,
                                    int32_t every, int32_t force_all, const double* x,
                                    const double* y, const double* z, double* bbox, int32_t* lperm,
                                    cudaStream_t s) {
    if (nrank <= 0 || max_small_n <= 0) return cudaSuccess;
    int np2 = 1;
    while (np2 < max_small_n) np2 <<= 1;
    k_batch_sort_small<<<nrank, kSortCta, sizeof(uint64_t) * np2, s>>>(bs, steps_slot, nsteps_slot, every,
                                                                        force_all, x, y, z, bbox, lperm);
    return cudaGetLastError();
}

cudaError_t launch_batch_perm_to_local(const BatchSys* bs, const int32_t* ranks, int32_t nlarge,
                                       int32_t max_n, const int32_t* perm, int32_t* lperm,
                                       cudaStream_t s) {
    if (nlarge <= 0 || max_n <= 0) return cudaSuccess;
    for (int32_t y0 = 0; y0 < nlarge; y0 += kMaxGridY) {
        const dim3 grid((unsigned)((max_n + kBThreads - 1) / kBThreads),
                        (unsigned)std::min<int32_t>(kMaxGridY, nlarge - y0));
        k_batch_perm_to_local<<<grid, kBThreads, 0, s>>>(bs, ranks, y0, perm, lperm);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_tick(const BatchSys* bs, int32_t nrank, int64_t* steps_slot,
                              const int64_t* nsteps_slot, cudaStream_t s) {
    if (nrank <= 0) return cudaSuccess;
    k_batch_tick<<<(nrank + 255) / 256, 256, 0, s>>>(bs, nrank, steps_slot, nsteps_slot);
    return cudaGetLastError();
}

// One CTA per packed tile: tile g belongs to rank tile_rank[g]; same per-tile
// origin, radius and paired layout as the single-system pack.
__global__ void __launch_bounds__(kTileJ)
    k_batch_pack(const int32_t* __restrict__ tile_rank, const SysDesc* __restrict__ sys,
                 const double* __restrict__ bbox, const int32_t* __restrict__ perm,
                 const double* __restrict__ x, const double* __restrict__ y,
                 const double* __restrict__ z, const double* __restrict__ m,
                 float4* __restrict__ pack, TileOrigin* __restrict__ origin,
                 float4* __restrict__ ext, const int32_t* __restrict__ sysid,
                 const int64_t* __restrict__ steps_slot, const int64_t* __restrict__ nsteps_slot) {
    // Each particle is split once into a double-float pair (the FP64 work of
    // this kernel, slow on this GPU: 12 FP64-pipe operations per particle).
    // The tile's bounding box is reduced in FP32 from the pairs relative to
    // the tile's first particle c; thread 0 alone forms the tile origin c +
    // float offset in FP64 and shares it.  Sources are re-expressed relative
    // to it from their pairs by the steps the force kernel applies to targets.
    // The common-mass test compares bit patterns.  Everything depends on this
    // tile's particles only.
    __shared__ float red[6][kTileJ / 32];
    __shared__ double cref[4];
    __shared__ float2 csplit[3];
    __shared__ TileOrigin tile_o;
    const int32_t g = blockIdx.x;
    const int32_t r = tile_rank[g];
    const SysDesc& d = sys[r];
    (void)bbox;
    if (nsteps_slot) {
        // a system that has made all its steps is skipped by the force too
        const int32_t s = sysid[d.off];
        if (steps_slot[s] >= nsteps_slot[s]) return;  // CTA-uniform
    }
    const int32_t t = g - d.tile_off;
    const int32_t slot = t * kTileJ + threadIdx.x;
    const bool valid = slot < d.n;
    double px = 0.0, py = 0.0, pz = 0.0, pm = 0.0;
    if (valid) {
        const int64_t p = d.off + perm[d.off + slot];  // perm: arena-relative local order
        px = x[p];
        py = y[p];
        pz = z[p];
        pm = m[p];
    }
    const float2 sx = split_df(px), sy = split_df(py), sz = split_df(pz);
    if (threadIdx.x == 0) {
        cref[0] = px;
        cref[1] = py;
        cref[2] = pz;
        cref[3] = pm;
        csplit[0] = sx;
        csplit[1] = sy;
        csplit[2] = sz;
    }
    __syncthreads();
    const double m0 = cref[3];
    // offsets from c for the box (within a few FP32 ulp of the FP64 offsets;
    // the box is enlarged below to cover that)
    const float fx = rel_df(sx, csplit[0].x, csplit[0].y);
    const float fy = rel_df(sy, csplit[1].x, csplit[1].y);
    const float fz = rel_df(sz, csplit[2].x, csplit[2].y);
    const bool same_mass = !valid || __double_as_longlong(pm) == __double_as_longlong(m0);
    float v[6];
    v[0] = valid ? fx : 3e38f;
    v[1] = valid ? fy : 3e38f;
    v[2] = valid ? fz : 3e38f;
    v[3] = valid ? -fx : 3e38f;
    v[4] = valid ? -fy : 3e38f;
    v[5] = valid ? -fz : 3e38f;
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k) red[k][warp] = v[k];
    }
    const bool uniform = __syncthreads_and(same_mass) && m0 > 0.0;
    float lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float a = red[k][0], b = red[k + 3][0];
#pragma unroll
        for (int w = 1; w < kTileJ / 32; ++w) {
            a = fminf(a, red[k][w]);
            b = fminf(b, red[k + 3][w]);
        }
        lo[k] = a;
        hi[k] = -b;
    }
    if (threadIdx.x == 0) {
        const float oxf = 0.5f * (lo[0] + hi[0]), oyf = 0.5f * (lo[1] + hi[1]),
                    ozf = 0.5f * (lo[2] + hi[2]);
        tile_o = make_tile_origin(cref[0] + (double)oxf, cref[1] + (double)oyf, cref[2] + (double)ozf, 0.0);
    }
    __syncthreads();
    TileOrigin to = tile_o;
    // Sources relative to the origin by the same FP32 steps the force kernel
    // applies to targets (rel_df): a particle's own entry and its target
    // coordinates are bit-identical, so the self pair has r = 0.
    float qx = 1e18f, qy = 1e18f, qz = 1e18f, qm = 0.0f;
    if (valid) {
        qx = rel_df(sx, to.hi.x, to.lo.x);
        qy = rel_df(sy, to.hi.y, to.lo.y);
        qz = rel_df(sz, to.hi.z, to.lo.z);
        qm = (float)pm;
    }
    // A full tile of one common mass keeps that mass in ext.w only; its mass
    // slots hold |q|^2 for the expanded far loop (pair_loop_expand).
    if (uniform && (t + 1) * kTileJ <= d.n) qm = fmaf(qx, qx, fmaf(qy, qy, qz * qz));
    float* base = reinterpret_cast<float*>(pack + (int64_t)g * kTileJ);
    const int pr = threadIdx.x >> 1, half = threadIdx.x & 1;
    base[8 * pr + half] = qx;
    base[8 * pr + 2 + half] = qy;
    base[8 * pr + 4 + half] = qz;
    base[8 * pr + 6 + half] = qm;
    if (threadIdx.x == 0) {
        // Half diagonal from the FP32 box, enlarged to cover the rounding of the
        // relative coordinates (the near test must never under-estimate it).
        const float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
        const float rr = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez);
        const float amax = fmaxf(fmaxf(fabsf(lo[0]), fabsf(hi[0])),
                                 fmaxf(fmaxf(fabsf(lo[1]), fabsf(hi[1])),
                                       fmaxf(fabsf(lo[2]), fabsf(hi[2]))));
        to.hi.w = (float)((double)rr * (1.0 + 1e-5) + 4.0e-7 * (double)amax);
        origin[g] = to;
        // box half extents for the near test, enlarged the same way
        const float slack = 4.0e-7f * amax;
        // ext.w: the common source mass when all are equal, else 0 (the pair
        // loops then apply it once per tile)
        // a partial tile stores -m (its padding adds exactly 0 to the
        // acceleration in the uniform form, not to the potential)
        const bool full = (t + 1) * kTileJ <= d.n;
        const float mu = uniform ? (full ? (float)m0 : -(float)m0) : 0.0f;
        ext[g] = make_float4(0.5f * ex * (1.0f + 1e-5f) + slack, 0.5f * ey * (1.0f + 1e-5f) + slack,
                             0.5f * ez * (1.0f + 1e-5f) + slack, mu);
    }
}

// ---------------------------------------------------------------------------
// Force over whole i-blocks.  items[k] = (rank, i-block), largest systems
// first; persistent CTAs claim items from a device counter.  Within an item
// the CTA streams all j-tiles of that system through the bulk-copy ring, in
// order, exactly like the single-system kernel.
// ---------------------------------------------------------------------------
// Launch shapes (threads per CTA, targets per thread); an item is one i-block
// of BLOCK * IPT targets.  Default 128 x 2; the engine takes the shape from its
// parameters (chosen by the autotuner).
// Register budget: acceleration-only launches of 128 threads are held to 6
// (one target per thread) or 5 (two) CTAs per SM, the counts at which the
// pair loop compiles without spills (as the single-system kernel).
template <int BLOCK, int IPT, bool ACC, bool POT>
struct BatchOcc {
    static constexpr int value =
        (ACC && !POT) ? (BLOCK == 128 ? (IPT == 1 ? 6 : 5) : (IPT == 1 ? 3 : 2)) : 1;
};

// v += a * (dt * fac) of one particle: fac 1 for a full kick, +-0.5 for the
// leapfrog half kicks at admission and retirement (src/base/Timestep.jl:84-93,
// 116-125), in the single-system kernels' operation order: a * dt for full
// kicks, a * fw * 0.5 * dt for half kicks.  Used by k_batch_kick and by the
// force kernel's fused kick, so both give the same bits.
__device__ __forceinline__ void kick_particle(double* __restrict__ vx, double* __restrict__ vy,
                                              double* __restrict__ vz, int64_t i, double ax,
                                              double ay, double az, const int32_t* __restrict__ sysid,
                                              const double* __restrict__ dt_slot,
                                              const double* __restrict__ fac_slot) {
    const int32_t s = sysid[i];
    if (s < 0) return;
    const double f = fac_slot[s];
    if (f == 0.0) return;
    const double dt = dt_slot[s];
    if (f == 1.0) {
        vx[i] = __dadd_rn(vx[i], __dmul_rn(ax, dt));
        vy[i] = __dadd_rn(vy[i], __dmul_rn(ay, dt));
        vz[i] = __dadd_rn(vz[i], __dmul_rn(az, dt));
    } else {
        const double fw = f > 0.0 ? 1.0 : -1.0;
        vx[i] = __dadd_rn(vx[i], __dmul_rn(__dmul_rn(__dmul_rn(ax, fw), 0.5), dt));
        vy[i] = __dadd_rn(vy[i], __dmul_rn(__dmul_rn(__dmul_rn(ay, fw), 0.5), dt));
        vz[i] = __dadd_rn(vz[i], __dmul_rn(__dmul_rn(__dmul_rn(az, fw), 0.5), dt));
    }
}

template <int LAW, bool ACC, bool POT, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK, (BatchOcc<BLOCK, IPT, ACC, POT>::value))
    k_force_batch(BatchForce f) {
    constexpr int NW = BLOCK / 32;
    constexpr int kFBt = BLOCK * IPT;
    __shared__ __align__(128) float4 buf[kStages * kTileJ];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ uint32_t done[kStages];
    __shared__ int32_t item_sh;
    __shared__ uint32_t abort_sh;
    __shared__ float2 tpx[kFBt], tpy[kFBt], tpz[kFBt];
    const int tid = threadIdx.x, lane = tid & 31;

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            done[s] = 0;
        }
        abort_sh = 0;
        fence_mbar_init();
    }
    __syncthreads();

    uint32_t vbase = 0;  // tiles streamed so far by this CTA (ring phase)
    uint32_t last_issued = 0;
    for (;;) {
        if (tid == 0) item_sh = atomicAdd(f.counter, 1);
        __syncthreads();
        const int32_t it = item_sh;
        if (it >= f.nitems || abort_sh) break;  // CTA-uniform
        const int2 ib = f.items[it];
        const SysDesc& d = f.sys[ib.x];
        if (f.nsteps_slot) {
            // a system that has made all its steps keeps its state: no force,
            // no kick (CTA-uniform: every thread reads the same words)
            const int32_t s = f.sysid[d.off];
            if (f.steps_slot[s] >= f.nsteps_slot[s]) {
                __syncthreads();  // every thread has read item_sh
                continue;
            }
        }
        const int32_t ntiles = d.ntiles;
        if (tid == 0) {
            for (int k = 0; k < kStages && k < ntiles; ++k) {
                const uint32_t v = vbase + k;
                mbar_arrive_expect_tx(&full[v % kStages], kTileJ * sizeof(float4));
                bulk_g2s(&buf[(v % kStages) * kTileJ], f.pack + (int64_t)(d.tile_off + k) * kTileJ,
                         kTileJ * sizeof(float4), &full[v % kStages]);
                last_issued = v + 1;
            }
        }
        int32_t pidx[IPT];
        float hh[IPT], h2[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int32_t slot = ib.y * kFBt + k * BLOCK + tid;
            pidx[k] = -1;
            double x = 0.0, y = 0.0, z = 0.0;
            if (slot < d.n) {
                const int32_t p = (int32_t)(d.off + f.perm[d.off + slot]);
                pidx[k] = p;
                x = f.x[p];
                y = f.y[p];
                z = f.z[p];
            }
            tpx[k * BLOCK + tid] = split_df(x);
            tpy[k * BLOCK + tid] = split_df(y);
            tpz[k * BLOCK + tid] = split_df(z);
            hh[k] = (float)d.soft[0];
            h2[k] = hh[k] * hh[k];
        }
        float sx[IPT], sy[IPT], sz[IPT], sp[IPT];
        float cx[IPT], cy[IPT], cz[IPT], cp[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            sx[k] = sy[k] = sz[k] = sp[k] = 0.0f;
            cx[k] = cy[k] = cz[k] = cp[k] = 0.0f;
        }
        bool timed_out = false;
        for (int32_t t = 0; t < ntiles; ++t) {
            const uint32_t v = vbase + t;
            const int st = (int)(v % kStages);
            const uint32_t par = (v / kStages) & 1u;
            const float4 oh = f.origin[d.tile_off + t].hi, ol = f.origin[d.tile_off + t].lo;
            float xr[IPT], yr[IPT], zr[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                xr[k] = rel_df(tpx[k * BLOCK + tid], oh.x, ol.x);
                yr[k] = rel_df(tpy[k * BLOCK + tid], oh.y, ol.y);
                zr[k] = rel_df(tpz[k * BLOCK + tid], oh.z, ol.z);
            }
            float ax[IPT], ay[IPT], az[IPT], ap[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) ax[k] = ay[k] = az[k] = ap[k] = 0.0f;
            if (!__all_sync(0xffffffffu, mbar_wait_bounded(&full[st], par, kWaitTimeoutNs))) {
                timed_out = true;
                if (lane == 0) {
                    atomicOr(f.err, DEVERR_TIMEOUT);
                    atomicExch(&abort_sh, 1u);
                }
                break;
            }
            const float4* b = &buf[st * kTileJ];
            const float4 ex = f.ext[d.tile_off + t];
            bool near = false;
            if (LAW == NB_LAW_SPLINE_G2) near = warp_near<IPT>(ex, xr, yr, zr, hh, pidx);
            // the system's last tile may be partial
            const int np2 = tile_pairs<kTileJ>(d.n - t * kTileJ);
            if (near)
                pair_loop_checked<LAW, ACC, POT, IPT>(b, xr, yr, zr, hh, h2, ax, ay, az, ap, ex.w, np2);
            else if (ex.w > 0.0f && warp_expandable<IPT>(ex, oh.w, xr, yr, zr, pidx))
                pair_loop_expand<LAW, ACC, POT, IPT>(b, xr, yr, zr, h2, ax, ay, az, ap, ex.w);
            else
                pair_loop_far<LAW, ACC, POT, IPT>(b, xr, yr, zr, h2, ax, ay, az, ap, ex.w, np2);
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                const uint32_t prev = atomicAdd(&done[st], 1u);
                if (prev == NW - 1) {
                    __threadfence_block();
                    done[st] = 0;
                    if (t + kStages < ntiles) {
                        mbar_arrive_expect_tx(&full[st], kTileJ * sizeof(float4));
                        bulk_g2s(&buf[st * kTileJ],
                                 f.pack + (int64_t)(d.tile_off + t + kStages) * kTileJ,
                                 kTileJ * sizeof(float4), &full[st]);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if (ACC) {
                    two_sum_acc(sx[k], cx[k], ax[k]);
                    two_sum_acc(sy[k], cy[k], ay[k]);
                    two_sum_acc(sz[k], cz[k], az[k]);
                }
                if (POT) two_sum_acc(sp[k], cp[k], ap[k]);
            }
        }
        if (!timed_out) {
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int32_t p = pidx[k];
                if (p < 0) continue;
                if (ACC) {
                    const double a0 = ((double)sx[k] + (double)cx[k]) * f.G;
                    const double a1 = ((double)sy[k] + (double)cy[k]) * f.G;
                    const double a2 = ((double)sz[k] + (double)cz[k]) * f.G;
                    f.ax[p] = a0;
                    f.ay[p] = a1;
                    f.az[p] = a2;
                    if (f.vx) kick_particle(f.vx, f.vy, f.vz, p, a0, a1, a2, f.sysid, f.dt_slot, f.fac_slot);
                }
                if (POT) {
                    double phi = -((double)sp[k] + (double)cp[k]);
                    if (LAW == NB_LAW_PLUMMER) phi += (double)((float)f.m[p] * rsqrt_approx(h2[k]));
                    f.pot[p] = phi * f.G;
                }
            }
        }
        vbase += (uint32_t)ntiles;
        __syncthreads();  // every warp is done with this item's tiles
    }
    if (abort_sh && tid == 0) {
        // Drain the copies that may still be in flight (at most kStages).
        for (uint32_t u = last_issued > kStages ? last_issued - kStages : 0; u < last_issued; ++u)
            (void)mbar_wait_bounded(&full[u % kStages], (u / kStages) & 1u, kWaitTimeoutNs / 8);
    }
}

bool batch_shape_ok(int block, int ipt) {
    return (block == 128 || block == 256) && (ipt == 1 || ipt == 2);
}

int batch_block_targets(int block, int ipt) { return block * ipt; }

// Dispatch over the compiled shapes: acceleration only (what the engine's step
// needs); 128 x 2 also with the potential.
template <int LAW, bool ACC, bool POT, int B, int I>
static int occ_of() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_batch<LAW, ACC, POT, B, I>, B, 0) !=
        cudaSuccess)
        return 1;
    return nb < 1 ? 1 : nb;
}

template <int LAW, bool ACC, bool POT, int B, int I>
static cudaError_t launch_of(const BatchForce& f, int grid, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(f.counter, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    k_force_batch<LAW, ACC, POT, B, I><<<grid, B, 0, s>>>(f);
    return cudaGetLastError();
}

template <int LAW>
static int occ_law(bool acc, bool pot, int block, int ipt) {
    if (!acc || pot) {
        if (block != 128 || ipt != 2) return -1;
        return acc ? occ_of<LAW, true, true, 128, 2>() : occ_of<LAW, false, true, 128, 2>();
    }
    if (block == 128) return ipt == 1 ? occ_of<LAW, true, false, 128, 1>() : occ_of<LAW, true, false, 128, 2>();
    return ipt == 1 ? occ_of<LAW, true, false, 256, 1>() : occ_of<LAW, true, false, 256, 2>();
}

template <int LAW>
static cudaError_t launch_law(const BatchForce& f, int grid, int block, int ipt, cudaStream_t s) {
    const bool acc = f.ax != nullptr, pot = f.pot != nullptr;
    if (!acc || pot) {
        if (block != 128 || ipt != 2) return cudaErrorInvalidValue;
        return acc ? launch_of<LAW, true, true, 128, 2>(f, grid, s)
                   : launch_of<LAW, false, true, 128, 2>(f, grid, s);
    }
    if (block == 128)
        return ipt == 1 ? launch_of<LAW, true, false, 128, 1>(f, grid, s)
                        : launch_of<LAW, true, false, 128, 2>(f, grid, s);
    return ipt == 1 ? launch_of<LAW, true, false, 256, 1>(f, grid, s)
                    : launch_of<LAW, true, false, 256, 2>(f, grid, s);
}

int batch_ctas_per_sm(int law, bool acc, bool pot, int block, int ipt) {
    if (!batch_shape_ok(block, ipt)) return -1;
    return law == NB_LAW_PLUMMER ? occ_law<NB_LAW_PLUMMER>(acc, pot, block, ipt)
                                 : occ_law<NB_LAW_SPLINE_G2>(acc, pot, block, ipt);
}

cudaError_t launch_force_batch(int law, const BatchForce& f, int grid, int block, int ipt,
                               cudaStream_t s) {
    const bool acc = f.ax != nullptr, pot = f.pot != nullptr;
    if (f.nitems <= 0 || grid <= 0 || (!acc && !pot)) return cudaSuccess;
    if (!batch_shape_ok(block, ipt)) return cudaErrorInvalidValue;
    return law == NB_LAW_PLUMMER ? launch_law<NB_LAW_PLUMMER>(f, grid, block, ipt, s)
                                 : launch_law<NB_LAW_SPLINE_G2>(f, grid, block, ipt, s);
}

// ---------------------------------------------------------------------------
// Integrator over the arena (FP64; built with -fmad=false in nb_integrate.cu's
// spirit: explicit round-to-nearest intrinsics keep each product and sum
// rounded as the reference's Julia expressions are).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBThreads)
    k_batch_drift(double* __restrict__ x, double* __restrict__ y, double* __restrict__ z,
                  const double* __restrict__ vx, const double* __restrict__ vy,
                  const double* __restrict__ vz, const int32_t* __restrict__ sysid,
                  const double* __restrict__ dt_slot, const double* __restrict__ fac_slot,
                  const int64_t* __restrict__ steps_slot, const int64_t* __restrict__ nsteps_slot,
                  int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
    if (i >= n) return;
    const int32_t s = sysid[i];
    if (s < 0) return;
    const double f = fac_slot[s];
    if (f == 0.0) return;
    if (nsteps_slot && steps_slot[s] >= nsteps_slot[s]) return;  // all steps made
    const double dt = __dmul_rn(dt_slot[s], f);
    x[i] = __dadd_rn(x[i], __dmul_rn(vx[i], dt));
    y[i] = __dadd_rn(y[i], __dmul_rn(vy[i], dt));
    z[i] = __dadd_rn(z[i], __dmul_rn(vz[i], dt));
}

// v += a * (dt * fac) over the arena (the admission and retirement half kicks;
// the step's full kick is fused into k_force_batch).
__global__ void __launch_bounds__(kBThreads)
    k_batch_kick(double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                 const double* __restrict__ ax, const double* __restrict__ ay,
                 const double* __restrict__ az, const int32_t* __restrict__ sysid,
                 const double* __restrict__ dt_slot, const double* __restrict__ fac_slot,
                 int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
    if (i >= n) return;
    kick_particle(vx, vy, vz, i, ax[i], ay[i], az[i], sysid, dt_slot, fac_slot);
}

__global__ void k_fill_i32(int32_t* __restrict__ a, int64_t n, int32_t v) {
    const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
    if (i < n) a[i] = v;
}

cudaError_t launch_fill_i32(int32_t* a, int64_t n, int32_t v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_fill_i32<<<(unsigned)((n + kBThreads - 1) / kBThreads), kBThreads, 0, s>>>(a, n, v);
    return cudaGetLastError();
}

cudaError_t launch_batch_large_keys(const BatchSys* bs, const int32_t* ranks, int32_t nlarge,
                                    int32_t max_n, const double* x, const double* y, const double* z,
                                    unsigned long long* box_key, uint64_t* keys, int32_t* vals,
                                    cudaStream_t s) {
    if (nlarge <= 0 || max_n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(box_key, 0xff, sizeof(unsigned long long) * 6 * (size_t)nlarge, s);
    if (e != cudaSuccess) return e;
    for (int32_t y0 = 0; y0 < nlarge; y0 += kMaxGridY) {
        const unsigned ny = (unsigned)std::min<int32_t>(kMaxGridY, nlarge - y0);
        const dim3 gbox((unsigned)((max_n + 4 * kBThreads - 1) / (4 * kBThreads)), ny);
        k_batch_large_box<<<gbox, kBThreads, 0, s>>>(bs, ranks, y0, x, y, z, box_key);
    }
    for (int32_t y0 = 0; y0 < nlarge; y0 += kMaxGridY) {
        const unsigned ny = (unsigned)std::min<int32_t>(kMaxGridY, nlarge - y0);
        const dim3 gkey((unsigned)((max_n + kBThreads - 1) / kBThreads), ny);
        k_batch_large_keys<<<gkey, kBThreads, 0, s>>>(bs, ranks, y0, box_key, x, y, z, keys, vals);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_pack(const int32_t* tile_rank, int32_t ntiles, const SysDesc* sys,
                              const double* bbox, const int32_t* perm, const double* x,
                              const double* y, const double* z, const double* m, float4* pack,
                              TileOrigin* origin, float4* ext, const int32_t* sysid,
                              const int64_t* steps_slot, const int64_t* nsteps_slot,
                              cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    k_batch_pack<<<ntiles, kTileJ, 0, s>>>(tile_rank, sys, bbox, perm, x, y, z, m, pack, origin, ext,
                                           sysid, steps_slot, nsteps_slot);
    return cudaGetLastError();
}

cudaError_t launch_batch_drift(double* x, double* y, double* z, const double* vx, const double* vy,
                               const double* vz, const int32_t* sysid, const double* dt_slot,
                               const double* fac_slot, const int64_t* steps_slot,
                               const int64_t* nsteps_slot, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_batch_drift<<<(unsigned)((n + kBThreads - 1) / kBThreads), kBThreads, 0, s>>>(
        x, y, z, vx, vy, vz, sysid, dt_slot, fac_slot, steps_slot, nsteps_slot, n);
    return cudaGetLastError();
}

cudaError_t launch_batch_kick(double* vx, double* vy, double* vz, const double* ax,
                              const double* ay, const double* az, const int32_t* sysid,
                              const double* dt_slot, const double* fac_slot, int64_t n,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_batch_kick<<<(unsigned)((n + kBThreads - 1) / kBThreads), kBThreads, 0, s>>>(
        vx, vy, vz, ax, ay, az, sysid, dt_slot, fac_slot, n);
    return cudaGetLastError();
}

}  // namespace nb
