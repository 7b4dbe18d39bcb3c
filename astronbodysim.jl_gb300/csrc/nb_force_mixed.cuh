// nb_force_mixed.cuh -- the mixed-precision direct-sum force kernels for
// sm_103a, templated on the j-tile size TJ (128, 256, 512 sources) and the
// depth NST of the shared-memory ring; nb_force_mixed_t{128,256,512}.cu
// instantiate them per tile size and nb_force_mixed.cu dispatches.
//
// Replaces compute_force_gpu_kernel (src/directsumgpu/gravity.jl:22-34), which
// reads every source from global memory once per target thread, with:
//   * a pack kernel that writes sources as FP32 float4 (x-o, y-o, z-o, m) in
//     j-tiles of TJ particles, with an FP64 origin o per tile (the centre of
//     the tile's bounding box), kept as a float pair hi + lo;
//   * a force kernel whose CTA holds BLOCK*IPT targets in registers and streams
//     every j-tile through shared memory with bulk async copies
//     (cp.async.bulk ... mbarrier::complete_tx, per CTA, no multicast) in an
//     NST-deep ring.  Each target's position is re-expressed relative to the
//     tile origin with three FP32 operations per coordinate, then the pair
//     loop runs in FP32.  Per-tile FP32 partial sums are folded into
//     (sum, carry) pairs with TwoSum.
//
// Pair law (per target softening h, src/directsum/gravity.jl:8-28):
//   r >= h : a += m d / r^3                 (fast path, branch-free)
//   r <  h : Gadget-2 spline polynomial     (rare slow path; includes j == i)
// Potential (src/directsum/potential.jl:2-27): -m/r, spline inside h, 0 at r=0.
#pragma once

#include "nb_pairs.cuh"

namespace nb {

// ---------------------------------------------------------------------------
// Pack: one CTA of TJ threads per j-tile.  Slot i of the packed array holds
// particle perm[i] (identity when perm == nullptr), in pairs: slots 2p, 2p+1 of
// a tile are stored as float4 (x0, x1, y0, y1), float4 (z0, z1, m0, m1), so
// the packed-FP32x2 pair loop evaluates two sources per instruction.  The tile
// origin is the centre of the tile's FP64 bounding box, origin.w its half
// diagonal.
// ---------------------------------------------------------------------------
template <int TJ>
__global__ void __launch_bounds__(TJ) k_pack(const double* __restrict__ x,
                                                 const double* __restrict__ y,
                                                 const double* __restrict__ z,
                                                 const double* __restrict__ m, int64_t n,
                                                 const int32_t* __restrict__ perm,
                                                 float4* __restrict__ pack,
                                                 TileOrigin* __restrict__ origin,
                                                 float4* __restrict__ ext) {
    // Each particle is split once into a double-float pair (12 FP64-pipe
    // operations, the slow pipe on this GPU).  The tile's box is reduced in
    // FP32 from the pairs relative to the tile's first particle c, the
    // common-mass test compares bit patterns, and thread 0 alone forms the
    // FP64 tile origin c + float offset and shares it.
    __shared__ float red[6][TJ / 32];
    __shared__ double cref[4];
    __shared__ float2 csplit[3];
    __shared__ TileOrigin tile_o;
    const int64_t i = (int64_t)blockIdx.x * TJ + threadIdx.x;
    const bool valid = i < n;
    double px = 0.0, py = 0.0, pz = 0.0, pm = 0.0;
    if (valid) {
        const int64_t p = perm ? (int64_t)perm[i] : i;
        px = x[p];
        py = y[p];
        pz = z[p];
        pm = m[p];
    }
    const float2 sx = split_df(px), sy = split_df(py), sz = split_df(pz);
    if (threadIdx.x == 0) {  // every tile holds at least one particle (tiles cover [0, n))
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
        for (int w = 1; w < TJ / 32; ++w) {
            a = fminf(a, red[k][w]);
            b = fminf(b, red[k + 3][w]);
        }
        lo[k] = a;
        hi[k] = -b;
    }
    const float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
    const float amax = fmaxf(fmaxf(fabsf(lo[0]), fabsf(hi[0])),
                             fmaxf(fmaxf(fabsf(lo[1]), fabsf(hi[1])), fmaxf(fabsf(lo[2]), fabsf(hi[2]))));
    if (threadIdx.x == 0) {
        // origin at the box centre; the half diagonal is enlarged to cover the
        // rounding of the FP32 relative coordinates
        const float rr = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez);
        tile_o = make_tile_origin(cref[0] + (double)(0.5f * (lo[0] + hi[0])),
                                  cref[1] + (double)(0.5f * (lo[1] + hi[1])),
                                  cref[2] + (double)(0.5f * (lo[2] + hi[2])),
                                  (double)rr * (1.0 + 1e-5) + 4.0e-7 * (double)amax);
    }
    __syncthreads();
    const TileOrigin to = tile_o;
    // ext.w: the common mass m of the tile's sources when all are equal (the
    // pair loops then apply it once per tile), else 0.  A partial tile stores
    // -m: its far padding adds exactly 0 to the acceleration in that form
    // (r^-3 underflows) but not to the potential, so the potential loops use
    // the per-pair masses there.
    const bool full = ((int64_t)blockIdx.x + 1) * TJ <= n;
    const float mu = uniform ? (full ? (float)m0 : -(float)m0) : 0.0f;
    // Sources relative to the origin by the same FP32 steps the force kernels
    // apply to targets (rel_df), so a particle's own source entry and its
    // target coordinates are bit-identical and the self pair has r = 0.
    float qx = 1e18f, qy = 1e18f, qz = 1e18f, qm = 0.0f;
    if (valid) {
        qx = rel_df(sx, to.hi.x, to.lo.x);
        qy = rel_df(sy, to.hi.y, to.lo.y);
        qz = rel_df(sz, to.hi.z, to.lo.z);
        qm = (float)pm;
    }
    // A full tile of one common mass keeps that mass in ext.w only; its mass
    // slots hold |q|^2 for the expanded far loop (pair_loop_expand).  Every
    // pair loop takes the mass of such a tile from ext.w.
    if (mu > 0.0f) qm = fmaf(qx, qx, fmaf(qy, qy, qz * qz));
    // (Zero-mass padding far away contributes exactly 0 and never takes the
    // r < h path.)  Paired layout: sources 2p and 2p+1 of the tile occupy
    // float4 (x0, x1, y0, y1) and float4 (z0, z1, m0, m1).
    float* base = reinterpret_cast<float*>(pack + (int64_t)blockIdx.x * TJ);
    const int pr = threadIdx.x >> 1, half = threadIdx.x & 1;
    base[8 * pr + half] = qx;
    base[8 * pr + 2 + half] = qy;
    base[8 * pr + 4 + half] = qz;
    base[8 * pr + 6 + half] = qm;
    if (threadIdx.x == 0) {
        origin[blockIdx.x] = to;
        // Half extents of the box for the near test, enlarged to cover the
        // rounding of the FP32 relative coordinates (the test must never
        // under-estimate them).
        const float slack = 4.0e-7f * amax;
        ext[blockIdx.x] = make_float4(0.5f * ex * (1.0f + 1e-5f) + slack, 0.5f * ey * (1.0f + 1e-5f) + slack,
                                      0.5f * ez * (1.0f + 1e-5f) + slack, mu);
    }
}


// ---------------------------------------------------------------------------
// Force kernel.
//
// CTA = BLOCK threads, IPT targets per thread (slot k*BLOCK + tid).  Targets'
// FP64 positions live in shared memory as float pairs hi + lo; per j-tile each
// thread re-expresses them relative to the tile origin (also hi + lo) with
// three FP32 operations per coordinate, so the tile loop issues no FP64
// instruction.
//
// j-tiles of TJ sources stream through an NST-stage ring.  full[s] (mbarrier, count 1 +
// transaction bytes) completes when the bulk copy of the tile has landed.
// There is no CTA-wide barrier per tile: every warp bumps done[s] after it has
// read stage s, and the last warp to do so re-arms full[s] and issues the copy
// of tile t + NST into it.  Warps may therefore run up to NST - 1
// tiles apart.  Every wait is bounded; a timed-out warp records
// DEVERR_TIMEOUT and stops, and the CTA drains its copies before exiting.
// ---------------------------------------------------------------------------
// CTAs per SM the register allocation is held to (acceleration-only launches
// of 128 threads); overridable at build time for launch-shape experiments.
#ifndef NB_MINB_IPT1
#define NB_MINB_IPT1 6
#endif
#ifndef NB_MINB_IPT2
#define NB_MINB_IPT2 5
#endif
#ifndef NB_MINB_IPT4
#define NB_MINB_IPT4 1
#endif
template <int BLOCK, int IPT, bool POT>
struct ForceOcc {
    static constexpr int value =
        (BLOCK == 128 && !POT) ? (IPT == 1 ? NB_MINB_IPT1 : (IPT == 2 ? NB_MINB_IPT2 : NB_MINB_IPT4)) : 1;
};

template <int LAW, bool ACC, bool POT, int BLOCK, int IPT, int TJ, int NST>
__global__ void __launch_bounds__(BLOCK, (ForceOcc<BLOCK, IPT, POT>::value)) k_force_mixed(Sources32 src, Targets tg, double G,
                                                       uint32_t* __restrict__ err) {
    static_assert(TJ == 128 || TJ == 256 || TJ == 512, "tile of 128, 256 or 512 sources");
    constexpr int kWarpsPerCta = BLOCK / 32;
    __shared__ __align__(128) float4 buf[NST * TJ];
    __shared__ __align__(8) uint64_t full[NST];
    __shared__ uint32_t done[NST];
    __shared__ uint32_t abort_flag;
    __shared__ float2 tpx[BLOCK * IPT], tpy[BLOCK * IPT], tpz[BLOCK * IPT];

    const int64_t ntg = tg.d_count ? (int64_t)(*tg.d_count) : tg.n;
    const int js = src.jsplit > 1 ? src.jsplit : 1;
    const int64_t blk = (int64_t)blockIdx.x / js;
    const int part = (int)(blockIdx.x % js);
    const int64_t base = blk * (BLOCK * IPT);
    if (base >= ntg) return;  // CTA-uniform
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int t_lo = (int)((int64_t)part * src.ntiles / js);
    const int ntiles = (int)((int64_t)(part + 1) * src.ntiles / js) - t_lo;  // tiles of this CTA

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            done[s] = 0;
        }
        abort_flag = 0;
        fence_mbar_init();
    }

    int32_t pidx[IPT];
    float hh[IPT], h2[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int64_t t = base + k * BLOCK + tid;
        pidx[k] = -1;
        double x = 0.0, y = 0.0, z = 0.0, h = tg.h_const;
        if (t < ntg) {
            const int32_t p = tg.idx ? tg.idx[t] : (int32_t)t;
            pidx[k] = p;
            x = tg.x[p];
            y = tg.y[p];
            z = tg.z[p];
            if (tg.type) h = tg.soft[tg.type[p] - 1];
        }
        tpx[k * BLOCK + tid] = split_df(x);
        tpy[k * BLOCK + tid] = split_df(y);
        tpz[k * BLOCK + tid] = split_df(z);
        hh[k] = (float)h;
        h2[k] = hh[k] * hh[k];
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < NST && s < ntiles; ++s) {
            mbar_arrive_expect_tx(&full[s], TJ * sizeof(float4));
            bulk_g2s(&buf[s * TJ], src.pack + (int64_t)(t_lo + s) * TJ, TJ * sizeof(float4),
                     &full[s]);
        }
    }

    float sx[IPT], sy[IPT], sz[IPT], sp[IPT];
    float cx[IPT], cy[IPT], cz[IPT], cp[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        sx[k] = sy[k] = sz[k] = sp[k] = 0.0f;
        cx[k] = cy[k] = cz[k] = cp[k] = 0.0f;
    }

    bool timed_out = false;
    for (int t = 0; t < ntiles; ++t) {
        const int s = t % NST;
        const uint32_t par = (uint32_t)(t / NST) & 1u;
        const float4 oh = src.origin[t_lo + t].hi, ol = src.origin[t_lo + t].lo;
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

        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], par, kWaitTimeoutNs));
        if (!ok || abort_flag) {
            timed_out = true;
            if (lane == 0) {
                atomicOr(err, DEVERR_TIMEOUT);
                atomicExch(&abort_flag, 1u);
            }
            break;
        }
        const float4* b = &buf[s * TJ];
        // Warp-uniform choice of the pair loop: when every target of the warp
        // lies farther than (tile radius + h) from the tile origin, no pair of
        // this tile can have r < h and the branch-free loop runs.
        const float4 ex = src.ext[t_lo + t];
        bool near = false;
        if (LAW == NB_LAW_SPLINE_G2) near = warp_near<IPT>(ex, xr, yr, zr, hh, pidx);
        if (near)
            pair_loop_checked<LAW, ACC, POT, IPT, TJ>(b, xr, yr, zr, hh, h2, ax, ay, az, ap, ex.w);
        else if (ex.w > 0.0f && warp_expandable<IPT>(ex, oh.w, xr, yr, zr, pidx))
            pair_loop_expand<LAW, ACC, POT, IPT, TJ>(b, xr, yr, zr, h2, ax, ay, az, ap, ex.w);
        else
            pair_loop_far<LAW, ACC, POT, IPT, TJ>(b, xr, yr, zr, h2, ax, ay, az, ap, ex.w);

        // Release stage s; the last warp out refills it with tile t + NST.
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t prev = atomicAdd(&done[s], 1u);
            if (prev == kWarpsPerCta - 1) {
                __threadfence_block();
                done[s] = 0;
                if (t + NST < ntiles) {
                    mbar_arrive_expect_tx(&full[s], TJ * sizeof(float4));
                    bulk_g2s(&buf[s * TJ], src.pack + (int64_t)(t_lo + t + NST) * TJ,
                             TJ * sizeof(float4), &full[s]);
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

    if (__syncthreads_or(timed_out)) {
        if (tid == 0) {
            // Drain every copy that may still be in flight before exiting.
            for (int u = 0; u < ntiles; ++u)
                (void)mbar_wait_bounded(&full[u % NST], (uint32_t)(u / NST) & 1u,
                                        kWaitTimeoutNs / 8);
        }
        return;
    }

    if (js > 1) {
        // j-split: compensated partials of this CTA's tile range
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int64_t slot = base + k * BLOCK + tid;
            float* q = src.partial + (int64_t)part * 8 * src.pstride + slot;
            q[0 * src.pstride] = sx[k];
            q[1 * src.pstride] = cx[k];
            q[2 * src.pstride] = sy[k];
            q[3 * src.pstride] = cy[k];
            q[4 * src.pstride] = sz[k];
            q[5 * src.pstride] = cz[k];
            q[6 * src.pstride] = sp[k];
            q[7 * src.pstride] = cp[k];
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int32_t p = pidx[k];
        if (p < 0) continue;
        if (ACC) {
            tg.ax[p] = ((double)sx[k] + (double)cx[k]) * G;
            tg.ay[p] = ((double)sy[k] + (double)cy[k]) * G;
            tg.az[p] = ((double)sz[k] + (double)cz[k]) * G;
        }
        if (POT) {
            // The loops accumulate +m/r; phi = -sum.
            double phi = -((double)sp[k] + (double)cp[k]);
            if (LAW == NB_LAW_PLUMMER && tg.self_mass) {
                // Remove the self pair, bit-identical to the term the loop added.
                const float mself = (float)tg.self_mass[p];
                phi += (double)(mself * rsqrt_approx(h2[k]));
            }
            tg.pot[p] = phi * G;
        }
    }
}

// Adds the j-split partials of every target in part order (deterministic).
// The compensated (sum, carry) pairs of the parts are added as double-float
// numbers in FP32 (TwoSum of the sums, carries added), about 48 bits, and
// converted to FP64 once: the slow FP64 pipe then does two conversions and
// one add per component instead of two per part.  CTAs of kJoinThreads spread
// a small target set over many SMs.
constexpr int kJoinThreads = 64;
template <int LAW, bool ACC, bool POT>
__global__ void __launch_bounds__(kJoinThreads) k_force_join(Sources32 src, Targets tg, double G) {
    const int64_t ntg = tg.d_count ? (int64_t)(*tg.d_count) : tg.n;
    const int64_t slot = (int64_t)blockIdx.x * kJoinThreads + threadIdx.x;
    if (slot >= ntg) return;
    const int32_t p = tg.idx ? tg.idx[slot] : (int32_t)slot;
    float s[4] = {0.0f, 0.0f, 0.0f, 0.0f}, c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int part = 0; part < src.jsplit; ++part) {
        const float* q = src.partial + (int64_t)part * 8 * src.pstride + slot;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            two_sum_acc(s[j], c[j], q[(2 * j) * src.pstride]);
            c[j] += q[(2 * j + 1) * src.pstride];
        }
    }
    double a[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) a[j] = (double)s[j] + (double)c[j];
    if (ACC) {
        tg.ax[p] = a[0] * G;
        tg.ay[p] = a[1] * G;
        tg.az[p] = a[2] * G;
    }
    if (POT) {
        double phi = -a[3];
        if (LAW == NB_LAW_PLUMMER && tg.self_mass) {
            const float h = (float)(tg.type ? tg.soft[tg.type[p] - 1] : tg.h_const);
            phi += (double)((float)tg.self_mass[p] * rsqrt_approx(h * h));
        }
        tg.pot[p] = phi * G;
    }
}

// Launch of one force evaluation with tiles of TJ sources (instantiated in
// nb_force_mixed_t<TJ>.cu).  Shapes: (128 | 256 threads) x (1 | 2 | 4 targets
// per thread) with the default 4-stage ring; the acceleration-only form of
// 128 x 1 and 128 x 2 also with 3 and 6 stages (6 only for tiles of up to 256
// sources: 6 x 8 KiB would pass the 48 KiB of static shared memory).  Other
// combinations use 4 stages.
template <int LAW, bool ACC, bool POT, int TJ>
cudaError_t launch_cfg_tile(const Sources32& src, const Targets& tg, double G, uint32_t* err,
                            int block, int ipt, int stages, cudaStream_t s) {
    const int64_t per = (int64_t)block * ipt;
    const int js = src.jsplit > 1 ? src.jsplit : 1;
    const int64_t grid = (tg.n + per - 1) / per * js;
    if (grid <= 0) return cudaSuccess;
    bool launched = false;
#define NB_LAUNCH(B, I, S)                                                                  \
    if (!launched && block == B && ipt == I) {                                             \
        k_force_mixed<LAW, ACC, POT, B, I, TJ, S><<<(unsigned)grid, B, 0, s>>>(src, tg, G, err); \
        launched = true;                                                                   \
    }
    if constexpr (ACC && !POT) {
        if (stages == 3) {
            NB_LAUNCH(128, 1, 3)
            NB_LAUNCH(128, 2, 3)
        }
        if constexpr (TJ <= 256) {
            if (stages == 6) {
                NB_LAUNCH(128, 1, 6)
                NB_LAUNCH(128, 2, 6)
            }
        }
    }
    NB_LAUNCH(128, 1, 4)
    NB_LAUNCH(128, 2, 4)
    NB_LAUNCH(128, 4, 4)
    NB_LAUNCH(256, 1, 4)
    NB_LAUNCH(256, 2, 4)
    if constexpr (TJ <= 256) {
        // 1024 targets' positions (24 KiB) next to a ring of 512-source tiles
        // would pass the 48 KiB of static shared memory
        NB_LAUNCH(256, 4, 4)
    }
#undef NB_LAUNCH
    if (!launched) return cudaErrorInvalidValue;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || js == 1) return e;
    k_force_join<LAW, ACC, POT><<<(unsigned)((tg.n + kJoinThreads - 1) / kJoinThreads), kJoinThreads, 0, s>>>(
        src, tg, G);
    return cudaGetLastError();
}

template <int TJ>
cudaError_t launch_force_mixed_tile(int law, bool pot, const Sources32& src, const Targets& tg,
                                    double G, uint32_t* err, int block, int ipt, int stages,
                                    cudaStream_t s) {
    const bool acc = tg.ax != nullptr;
    if (!acc && !pot) return cudaSuccess;
    if (law == NB_LAW_PLUMMER) {
        if (!acc) return launch_cfg_tile<NB_LAW_PLUMMER, false, true, TJ>(src, tg, G, err, block, ipt, stages, s);
        return pot ? launch_cfg_tile<NB_LAW_PLUMMER, true, true, TJ>(src, tg, G, err, block, ipt, stages, s)
                   : launch_cfg_tile<NB_LAW_PLUMMER, true, false, TJ>(src, tg, G, err, block, ipt, stages, s);
    }
    if (!acc) return launch_cfg_tile<NB_LAW_SPLINE_G2, false, true, TJ>(src, tg, G, err, block, ipt, stages, s);
    return pot ? launch_cfg_tile<NB_LAW_SPLINE_G2, true, true, TJ>(src, tg, G, err, block, ipt, stages, s)
               : launch_cfg_tile<NB_LAW_SPLINE_G2, true, false, TJ>(src, tg, G, err, block, ipt, stages, s);
}

template <int TJ>
cudaError_t launch_pack_tile(const double* x, const double* y, const double* z, const double* m,
                             int64_t n, const int32_t* perm, float4* pack, TileOrigin* origin,
                             float4* ext, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t ntiles = (n + TJ - 1) / TJ;
    k_pack<TJ><<<(unsigned)ntiles, TJ, 0, s>>>(x, y, z, m, n, perm, pack, origin, ext);
    return cudaGetLastError();
}

}  // namespace nb
