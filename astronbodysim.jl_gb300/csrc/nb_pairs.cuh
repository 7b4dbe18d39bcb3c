// nb_pairs.cuh -- the FP32 pair arithmetic shared by the mixed-precision force
// kernels: tile geometry, the Gadget-2 spline slow path and the two pair loops
// over one j-tile in shared memory.
#pragma once

#include "nb_internal.cuh"

namespace nb {

constexpr int kTileJ = 256;
constexpr int kStages = 4;

// Pair-loop shape: sets of split partial sums per target (consecutive source
// pairs alternate between them, so accumulating FMAs do not wait on each
// other) and source pairs per unrolled iteration.  Overridable at build time
// (-DNB_SPLIT_SUMS_IPT1=..., for launch-shape experiments).
#ifndef NB_SPLIT_SUMS_IPT1
#define NB_SPLIT_SUMS_IPT1 2
#endif
#ifndef NB_SPLIT_SUMS_IPTN
#define NB_SPLIT_SUMS_IPTN 1
#endif
#ifndef NB_PAIRS_PER_ITER
#define NB_PAIRS_PER_ITER 4
#endif
template <int IPT>
struct LoopShape {
    static constexpr int NA = IPT == 1 ? NB_SPLIT_SUMS_IPT1 : NB_SPLIT_SUMS_IPTN;
    static constexpr int UNROLL = NB_PAIRS_PER_ITER / NA > 0 ? NB_PAIRS_PER_ITER / NA : 1;
};
constexpr uint64_t kWaitTimeoutNs = 2000000000ull;  // 2 s

// ---------------------------------------------------------------------------
// Spline slow path (r < h), FP32.  Returns m*fac (to multiply d) in mr3 and the
// negated potential contribution in mp.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void spline_close(float r2, float rinv, float m, float h, float& mr3,
                                             float& mp) {
    const float hinv = 1.0f / h;
    const float hinv3 = hinv * hinv * hinv;
    const float r = (r2 > 0.0f) ? r2 * rinv : 0.0f;
    const float u = r * hinv;
    float fac, wp;
    if (u < 0.5f) {
        fac = 10.666666666667f + u * u * (32.0f * u - 38.4f);
        wp = -2.8f + u * u * (5.333333333333f + u * u * (6.4f * u - 9.6f));
    } else {
        const float u3 = u * u * u;
        fac = 21.333333333333f - 48.0f * u + 38.4f * u * u - 10.666666666667f * u3 -
              0.066666666667f / u3;
        wp = -3.2f + 0.066666666667f / u +
             u * u * (10.666666666667f + u * (-16.0f + u * (9.6f - 2.133333333333f * u)));
    }
    mr3 = m * hinv3 * fac;
    mp = (r2 > 0.0f) ? -(m * hinv * wp) : 0.0f;  // +m/r convention: phi contribution is -mp
}

// ---------------------------------------------------------------------------
// Pair loops over one j-tile in shared memory (paired layout) for IPT targets
// held in registers.
//
// pair_loop_fast: branch-free, packed FP32x2 arithmetic (fma/mul/add .f32x2):
// each instruction evaluates one target against the two sources of a pair, so
// an interaction costs 6 issue slots of FP32 math + 1 MUFU rsqrt.  Used for
// every tile in the Plummer law and for far tiles in the spline law.
// pair_loop_checked: scalar, tests r < h per pair (spline slow path, j == i).
// Both accumulate per-tile partials; pot accumulates +m/r (negated later).
// ---------------------------------------------------------------------------
// Warp-uniform choice of the pair loop: a pair of this tile can have r < h
// only for a target whose distance to the tile's box (half extents e.x, e.y,
// e.z about the tile origin, enlarged for rounding) is at most h.  When no
// target of the warp is that close, the branch-free loop runs.
template <int IPT>
__device__ __forceinline__ bool warp_near(const float4 e, const float* xr, const float* yr,
                                          const float* zr, const float* hh, const int32_t* pidx) {
    bool near = false;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const float bx = fmaxf(fabsf(xr[k]) - e.x, 0.0f);
        const float by = fmaxf(fabsf(yr[k]) - e.y, 0.0f);
        const float bz = fmaxf(fabsf(zr[k]) - e.z, 0.0f);
        const float d2 = fmaf(bx, bx, fmaf(by, by, bz * bz));
        const float lim = hh[k] * 1.0001f;
        near |= (pidx[k] >= 0) && (d2 <= lim * lim);
    }
    return __any_sync(0xffffffffu, near);
}

// Branch-free loop for far tiles.  UNI: every source of the tile has the same
// mass mu (flagged by the pack in ext.w), which is then applied once to the
// tile's partial sums instead of once per pair (one FP32 operation less per
// interaction).  Zero-mass padding (at 1e18) then adds r^-3 = 0 exactly to
// the acceleration (the product underflows) but 1e-18 per slot to the
// potential, so partial tiles take this form only without the potential.
template <int LAW, bool ACC, bool POT, int IPT, bool UNI = false, int TJ = kTileJ>
__device__ __forceinline__ void pair_loop_fast(const float4* __restrict__ b, const float* xr,
                                               const float* yr, const float* zr, const float* h2,
                                               float* ax, float* ay, float* az, float* ap,
                                               float mu = 1.0f, int np2 = TJ / 2) {
    // With one target per thread the sums are split over two sets (even and
    // odd source pairs) so that consecutive accumulating FMAs do not wait on
    // each other; with more targets per thread they are independent already.
    constexpr int NA = LoopShape<IPT>::NA;
    float2 nx[IPT], ny[IPT], nz[IPT], e2[IPT];
    float2 sx[NA][IPT], sy[NA][IPT], sz[NA][IPT], sp[NA][IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        nx[k] = make_float2(-xr[k], -xr[k]);
        ny[k] = make_float2(-yr[k], -yr[k]);
        nz[k] = make_float2(-zr[k], -zr[k]);
        e2[k] = make_float2(h2[k], h2[k]);
#pragma unroll
        for (int u = 0; u < NA; ++u) sx[u][k] = sy[u][k] = sz[u][k] = sp[u][k] = make_float2(0.0f, 0.0f);
    }
#pragma unroll (LoopShape<IPT>::UNROLL)
    for (int p = 0; p < np2; p += NA) {
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            const float4 A = b[2 * (p + u)];
            const float4 B = b[2 * (p + u) + 1];
            const float2 qx = make_float2(A.x, A.y), qy = make_float2(A.z, A.w);
            const float2 qz = make_float2(B.x, B.y), qm = make_float2(B.z, B.w);
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const float2 dx = __fadd2_rn(qx, nx[k]);
                const float2 dy = __fadd2_rn(qy, ny[k]);
                const float2 dz = __fadd2_rn(qz, nz[k]);
                float2 r2 = (LAW == NB_LAW_PLUMMER) ? __ffma2_rn(dz, dz, e2[k]) : __fmul2_rn(dz, dz);
                r2 = __ffma2_rn(dy, dy, r2);
                r2 = __ffma2_rn(dx, dx, r2);
                const float2 rinv = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
                const float2 mp = UNI ? rinv : __fmul2_rn(qm, rinv);
                if (ACC) {
                    const float2 mr3 = __fmul2_rn(__fmul2_rn(mp, rinv), rinv);
                    sx[u][k] = __ffma2_rn(dx, mr3, sx[u][k]);
                    sy[u][k] = __ffma2_rn(dy, mr3, sy[u][k]);
                    sz[u][k] = __ffma2_rn(dz, mr3, sz[u][k]);
                }
                if (POT) sp[u][k] = __fadd2_rn(sp[u][k], mp);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        float tx = 0.0f, ty = 0.0f, tz = 0.0f, tp = 0.0f;
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            tx += sx[u][k].x + sx[u][k].y;
            ty += sy[u][k].x + sy[u][k].y;
            tz += sz[u][k].x + sz[u][k].y;
            tp += sp[u][k].x + sp[u][k].y;
        }
        if (UNI) {
            tx *= mu;
            ty *= mu;
            tz *= mu;
            tp *= mu;
        }
        ax[k] += tx;
        ay[k] += ty;
        az[k] += tz;
        ap[k] += tp;
    }
}

// Far-tile loop in expanded form, for full uniform-mass tiles (the pack then
// stores |q|^2 in each source's mass slot):
//   r^2 = (|q|^2 + |x|^2 [+ h^2]) - 2 q.x            (4 FP32 operations)
//   sum_j (q_j - x) r_j^-3 = sum_j q_j r_j^-3 - x sum_j r_j^-3
// so the three differences q - x drop out of the pair loop: 10 FP32
// operations per interaction instead of 11 (the MUFU rsqrt unchanged).
// Rounding: r^2 carries about 3 ulp of |q|^2 + |x|^2, and the two sums of the
// acceleration cancel by at most (|q| + |x|) / r.  Both stay bounded when
//   |q|^2 + |x|^2 <= (R^2 + |x|^2) <= kExpandBound * d^2
// for every target of the warp, with R the tile radius (|q| <= R) and d the
// distance from the target to the tile's box (r >= d; the box is enlarged
// for rounding, so d never exceeds a true distance): the relative error of
// r^2 stays within about 3 kExpandBound ulp and the cancellation within
// sqrt(2 kExpandBound).  A target inside the box (d = 0) never qualifies.
// The box distance admits more tiles than a test on |x| alone: at N = 2^20
// (Plummer, tiles of 512) |x| >= 2.5 R (worst case 3.22) admits 76 % of the
// (warp, tile) pairs, this test with the bound 3.25 84 % and with 5 90 %.
// Bounds of 3.25, 5 and 8 gave the same force error quantiles against the
// FP64 oracle at N = 2^20 (median 3.0e-8, p99 4.8e-7, max 1.76e-5).
#ifndef NB_EXPAND_BOUND
#define NB_EXPAND_BOUND 5.0f
#endif
constexpr float kExpandBound = NB_EXPAND_BOUND;

template <int IPT>
__device__ __forceinline__ bool warp_expandable(const float4 e, float radius, const float* xr,
                                                const float* yr, const float* zr,
                                                const int32_t* pidx) {
    bool ok = true;
    const float rr = radius * radius;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const float bx = fmaxf(fabsf(xr[k]) - e.x, 0.0f);
        const float by = fmaxf(fabsf(yr[k]) - e.y, 0.0f);
        const float bz = fmaxf(fabsf(zr[k]) - e.z, 0.0f);
        const float d2 = fmaf(bx, bx, fmaf(by, by, bz * bz));
        const float x2 = fmaf(xr[k], xr[k], fmaf(yr[k], yr[k], zr[k] * zr[k]));
        ok &= (pidx[k] < 0) || (x2 + rr <= kExpandBound * d2);
    }
    return __all_sync(0xffffffffu, ok);
}

template <int LAW, bool ACC, bool POT, int IPT, int TJ = kTileJ>
__device__ __forceinline__ void pair_loop_expand(const float4* __restrict__ b, const float* xr,
                                                 const float* yr, const float* zr,
                                                 const float* h2, float* ax, float* ay, float* az,
                                                 float* ap, float mu) {
    constexpr int NA = LoopShape<IPT>::NA;
    float2 mx[IPT], my[IPT], mz[IPT], cc[IPT];
    float2 sx[NA][IPT], sy[NA][IPT], sz[NA][IPT], sw[NA][IPT], sp[NA][IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        mx[k] = make_float2(-2.0f * xr[k], -2.0f * xr[k]);
        my[k] = make_float2(-2.0f * yr[k], -2.0f * yr[k]);
        mz[k] = make_float2(-2.0f * zr[k], -2.0f * zr[k]);
        float c = fmaf(xr[k], xr[k], fmaf(yr[k], yr[k], zr[k] * zr[k]));
        if (LAW == NB_LAW_PLUMMER) c += h2[k];
        cc[k] = make_float2(c, c);
#pragma unroll
        for (int u = 0; u < NA; ++u)
            sx[u][k] = sy[u][k] = sz[u][k] = sw[u][k] = sp[u][k] = make_float2(0.0f, 0.0f);
    }
#pragma unroll (LoopShape<IPT>::UNROLL)
    for (int p = 0; p < TJ / 2; p += NA) {
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            const float4 A = b[2 * (p + u)];
            const float4 B = b[2 * (p + u) + 1];
            const float2 qx = make_float2(A.x, A.y), qy = make_float2(A.z, A.w);
            const float2 qz = make_float2(B.x, B.y), qq = make_float2(B.z, B.w);
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                float2 r2 = __fadd2_rn(qq, cc[k]);
                r2 = __ffma2_rn(qz, mz[k], r2);
                r2 = __ffma2_rn(qy, my[k], r2);
                r2 = __ffma2_rn(qx, mx[k], r2);
                const float2 rinv = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
                if (ACC) {
                    const float2 r3 = __fmul2_rn(__fmul2_rn(rinv, rinv), rinv);
                    sx[u][k] = __ffma2_rn(qx, r3, sx[u][k]);
                    sy[u][k] = __ffma2_rn(qy, r3, sy[u][k]);
                    sz[u][k] = __ffma2_rn(qz, r3, sz[u][k]);
                    sw[u][k] = __fadd2_rn(sw[u][k], r3);
                }
                if (POT) sp[u][k] = __fadd2_rn(sp[u][k], rinv);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        float tx = 0.0f, ty = 0.0f, tz = 0.0f, tw = 0.0f, tp = 0.0f;
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            tx += sx[u][k].x + sx[u][k].y;
            ty += sy[u][k].x + sy[u][k].y;
            tz += sz[u][k].x + sz[u][k].y;
            tw += sw[u][k].x + sw[u][k].y;
            tp += sp[u][k].x + sp[u][k].y;
        }
        ax[k] += fmaf(-xr[k], tw, tx) * mu;
        ay[k] += fmaf(-yr[k], tw, ty) * mu;
        az[k] += fmaf(-zr[k], tw, tz) * mu;
        ap[k] += tp * mu;
    }
}

// Source pairs of a tile the loops visit: the tile's real sources rounded up
// to 16 (the pair loops' step).  The zero-mass padding beyond them adds
// exactly 0 (its r^-3 underflows and its potential term is m r^-1 = 0), so
// stopping there leaves every sum bit-identical and saves the padding's
// share of a partial tile: about 3 % of the interactions evaluated in an
// ensemble of systems of 64 .. 8192 particles with tiles of 256.
template <int TJ>
__device__ __forceinline__ int tile_pairs(int count) {
    return count >= TJ ? TJ / 2 : (count + 15) / 16 * 8;
}

// Far-tile dispatch: the uniform-mass loop when the pack flagged the tile.
template <int LAW, bool ACC, bool POT, int IPT, int TJ = kTileJ>
__device__ __forceinline__ void pair_loop_far(const float4* __restrict__ b, const float* xr,
                                              const float* yr, const float* zr, const float* h2,
                                              float* ax, float* ay, float* az, float* ap, float mu,
                                              int np2 = TJ / 2) {
    // mu < 0: uniform but partial tile (usable for the acceleration only)
    const float m = POT ? mu : fabsf(mu);
    if (m > 0.0f)
        pair_loop_fast<LAW, ACC, POT, IPT, true, TJ>(b, xr, yr, zr, h2, ax, ay, az, ap, m, np2);
    else
        pair_loop_fast<LAW, ACC, POT, IPT, false, TJ>(b, xr, yr, zr, h2, ax, ay, az, ap, 1.0f, np2);
}

template <int LAW, bool ACC, bool POT, int IPT, bool UNI, int TJ = kTileJ>
__device__ __forceinline__ void pair_loop_checked_impl(const float4* __restrict__ b, const float* xr,
                                                       const float* yr, const float* zr,
                                                       const float* hh, const float* h2, float* ax,
                                                       float* ay, float* az, float* ap, float mu,
                                                       int np2) {
    // Two passes over the tile.  Pass 1 is the packed FP32x2 loop of
    // pair_loop_fast (uniform-mass form and split sums included) on r^2
    // clamped to at least h^2: a pair with r < h adds the bounded Newtonian
    // term of distance h, m d / h^3 (the self pair, d = 0, adds no force),
    // and the smallest unclamped r^2 of every block of 8 source pairs marks
    // the blocks that held such a pair.  Pass 2 revisits only the blocks that
    // some lane of the warp flagged and replaces, for each r < h pair, the
    // clamped term by the spline term.  Both terms are at most about m / h^2,
    // so the replacement loses nothing to cancellation.
    constexpr int NA = LoopShape<IPT>::NA;
    float2 nx[IPT], ny[IPT], nz[IPT], hc[IPT];
    float2 sx[NA][IPT], sy[NA][IPT], sz[NA][IPT], sp[NA][IPT];
    uint32_t blk = 0;  // bit q: a r < h half among source pairs 8q .. 8q + 7
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        nx[k] = make_float2(-xr[k], -xr[k]);
        ny[k] = make_float2(-yr[k], -yr[k]);
        nz[k] = make_float2(-zr[k], -zr[k]);
        hc[k] = make_float2(h2[k], h2[k]);
#pragma unroll
        for (int u = 0; u < NA; ++u) sx[u][k] = sy[u][k] = sz[u][k] = sp[u][k] = make_float2(0.0f, 0.0f);
    }
#pragma unroll 1
    for (int q = 0; q < np2 / 8; ++q) {
        float rmin[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) rmin[k] = 3e38f;
#pragma unroll
        for (int i = 0; i < 8; i += NA) {
#pragma unroll
            for (int u = 0; u < NA; ++u) {
                const int p = 8 * q + i + u;
                const float4 A = b[2 * p];
                const float4 B = b[2 * p + 1];
                const float2 qx = make_float2(A.x, A.y), qy = make_float2(A.z, A.w);
                const float2 qz = make_float2(B.x, B.y), qm = make_float2(B.z, B.w);
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const float2 dx = __fadd2_rn(qx, nx[k]);
                    const float2 dy = __fadd2_rn(qy, ny[k]);
                    const float2 dz = __fadd2_rn(qz, nz[k]);
                    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                    rmin[k] = fminf(rmin[k], fminf(r2.x, r2.y));
                    const float2 rc = make_float2(fmaxf(r2.x, hc[k].x), fmaxf(r2.y, hc[k].y));
                    const float2 rinv = make_float2(rsqrt_approx(rc.x), rsqrt_approx(rc.y));
                    const float2 mp = UNI ? rinv : __fmul2_rn(qm, rinv);
                    if (ACC) {
                        const float2 mr3 = __fmul2_rn(__fmul2_rn(mp, rinv), rinv);
                        sx[u][k] = __ffma2_rn(dx, mr3, sx[u][k]);
                        sy[u][k] = __ffma2_rn(dy, mr3, sy[u][k]);
                        sz[u][k] = __ffma2_rn(dz, mr3, sz[u][k]);
                    }
                    if (POT) sp[u][k] = __fadd2_rn(sp[u][k], mp);
                }
            }
        }
        bool f = false;
#pragma unroll
        for (int k = 0; k < IPT; ++k) f |= rmin[k] < h2[k];
        blk |= (uint32_t)f << q;
    }
    // Fold the split sums (and the common mass) into one set.
    float2 tx[IPT], ty[IPT], tz[IPT], tp[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        tx[k] = sx[0][k];
        ty[k] = sy[0][k];
        tz[k] = sz[0][k];
        tp[k] = sp[0][k];
#pragma unroll
        for (int u = 1; u < NA; ++u) {
            tx[k] = __fadd2_rn(tx[k], sx[u][k]);
            ty[k] = __fadd2_rn(ty[k], sy[u][k]);
            tz[k] = __fadd2_rn(tz[k], sz[u][k]);
            tp[k] = __fadd2_rn(tp[k], sp[u][k]);
        }
        if (UNI) {
            const float2 m2 = make_float2(mu, mu);
            tx[k] = __fmul2_rn(tx[k], m2);
            ty[k] = __fmul2_rn(ty[k], m2);
            tz[k] = __fmul2_rn(tz[k], m2);
            tp[k] = __fmul2_rn(tp[k], m2);
        }
    }
    for (uint32_t wb = __reduce_or_sync(0xffffffffu, blk); wb != 0u; wb &= wb - 1u) {
        const int q0 = 8 * (__ffs(wb) - 1);
#pragma unroll 1
        for (int p = q0; p < q0 + 8; ++p) {
            const float4 A = b[2 * p];
            const float4 B = b[2 * p + 1];
            const float2 qx = make_float2(A.x, A.y), qy = make_float2(A.z, A.w);
            const float2 qz = make_float2(B.x, B.y), qm = make_float2(B.z, B.w);
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const float2 dx = __fadd2_rn(qx, nx[k]);
                const float2 dy = __fadd2_rn(qy, ny[k]);
                const float2 dz = __fadd2_rn(qz, nz[k]);
                const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                const bool cx = r2.x < h2[k], cy = r2.y < h2[k];
                if (__any_sync(0xffffffffu, cx | cy)) {
                    // the clamped Newtonian term pass 1 added: m r_h^-3 d and m r_h^-1
                    const float rh = rsqrt_approx(h2[k]);
                    if (cx) {
                        const float m = UNI ? mu : qm.x;
                        float mr3, mp;
                        spline_close(r2.x, rsqrt_approx(r2.x), m, hh[k], mr3, mp);
                        const float mrh = m * rh;
                        const float d3 = mr3 - (mrh * rh) * rh;
                        tx[k].x = fmaf(dx.x, d3, tx[k].x);
                        ty[k].x = fmaf(dy.x, d3, ty[k].x);
                        tz[k].x = fmaf(dz.x, d3, tz[k].x);
                        tp[k].x += mp - mrh;
                    }
                    if (cy) {
                        const float m = UNI ? mu : qm.y;
                        float mr3, mp;
                        spline_close(r2.y, rsqrt_approx(r2.y), m, hh[k], mr3, mp);
                        const float mrh = m * rh;
                        const float d3 = mr3 - (mrh * rh) * rh;
                        tx[k].y = fmaf(dx.y, d3, tx[k].y);
                        ty[k].y = fmaf(dy.y, d3, ty[k].y);
                        tz[k].y = fmaf(dz.y, d3, tz[k].y);
                        tp[k].y += mp - mrh;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        ax[k] += tx[k].x + tx[k].y;
        ay[k] += ty[k].x + ty[k].y;
        az[k] += tz[k].x + tz[k].y;
        ap[k] += tp[k].x + tp[k].y;
    }
}

// Near-tile loop: the uniform-mass form when the pack flagged the tile.
template <int LAW, bool ACC, bool POT, int IPT, int TJ = kTileJ>
__device__ __forceinline__ void pair_loop_checked(const float4* __restrict__ b, const float* xr,
                                                  const float* yr, const float* zr,
                                                  const float* hh, const float* h2, float* ax,
                                                  float* ay, float* az, float* ap, float mu,
                                                  int np2 = TJ / 2) {
    const float m = POT ? mu : fabsf(mu);
    if (m > 0.0f)
        pair_loop_checked_impl<LAW, ACC, POT, IPT, true, TJ>(b, xr, yr, zr, hh, h2, ax, ay, az, ap, m, np2);
    else
        pair_loop_checked_impl<LAW, ACC, POT, IPT, false, TJ>(b, xr, yr, zr, hh, h2, ax, ay, az, ap, 1.0f,
                                                              np2);
}

}  // namespace nb
