// nb_force_fp64.cu -- plain FP64 direct-sum force (the reference's Float64 form).
//
// Built with -fmad=false so every a*b+c rounds twice, as Julia evaluates the
// pair expressions of src/directsum/gravity.jl:8-28 and
// src/directsum/potential.jl:2-27; sqrt and division are IEEE-rounded.  Each
// pair term is therefore the same double the CPU computes; the per-target sum
// is compensated (TwoSum), so the result differs from the CPU's pairwise sum
// (src/directsum/gravity.jl:45) only by that sum's own rounding.
//
// Sources are staged through shared memory in tiles of kTile (x, y, z, m);
// one target per thread.
#include "nb_internal.cuh"

namespace nb {

constexpr int kTile = 128;

template <int LAW>
__device__ __forceinline__ void pair_force64(double px, double py, double pz, dvec4 q, double G,
                                             double h, double h_inv, double h3_inv, double& fx,
                                             double& fy, double& fz) {
    const double dx = q.x - px, dy = q.y - py, dz = q.z - pz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    double fac;
    if (LAW == NB_LAW_PLUMMER) {
        const double r2e = r2 + h * h;
        fac = q.w / (r2e * sqrt(r2e));
    } else {
        const double r = sqrt(r2);
        if (r >= h) {
            fac = q.w / (r2 * r);
        } else {
            const double u = r * h_inv;
            if (u < 0.5)
                fac = q.w * h3_inv * (10.666666666667 + u * u * (32.0 * u - 38.4));
            else
                fac = q.w * h3_inv *
                      (21.333333333333 - 48.0 * u + 38.4 * (u * u) - 10.666666666667 * (u * u * u) -
                       0.066666666667 / (u * u * u));
        }
    }
    fx = dx * fac * G;
    fy = dy * fac * G;
    fz = dz * fac * G;
}

template <int LAW>
__device__ __forceinline__ double pair_pot64(double px, double py, double pz, dvec4 q, double G,
                                             double h, double h_inv) {
    const double dx = q.x - px, dy = q.y - py, dz = q.z - pz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double r = sqrt(r2);
    double pot;
    if (LAW == NB_LAW_PLUMMER) {
        pot = -q.w / sqrt(r2 + h * h) * G;
    } else if (r >= h) {
        pot = -q.w / r * G;
    } else {
        const double u = r * h_inv;
        double wp;
        if (u < 0.5)
            wp = -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6));
        else
            wp = -3.2 + 0.066666666667 / u +
                 u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)));
        pot = q.w * h_inv * wp * G;
    }
    if (r == 0.0) pot = pot * 0.0;
    return pot;
}

template <int LAW, bool ACC, bool POT>
__global__ void __launch_bounds__(kTile) k_force_fp64(Sources64 src, Targets tg, double G) {
    __shared__ dvec4 sj[kTile];
    const int64_t ntg = tg.d_count ? (int64_t)(*tg.d_count) : tg.n;
    const int64_t base = (int64_t)blockIdx.x * kTile;
    if (base >= ntg) return;
    const int64_t t = base + threadIdx.x;
    int32_t p = -1;
    double px = 0.0, py = 0.0, pz = 0.0, h = tg.h_const;
    if (t < ntg) {
        p = tg.idx ? tg.idx[t] : (int32_t)t;
        px = tg.x[p];
        py = tg.y[p];
        pz = tg.z[p];
        if (tg.type) h = tg.soft[tg.type[p] - 1];
    }
    const double h_inv = 1.0 / h;
    const double h3_inv = h_inv * h_inv * h_inv;
    double sx = 0.0, sy = 0.0, sz = 0.0, sp = 0.0;
    double cx = 0.0, cy = 0.0, cz = 0.0, cp = 0.0;
    for (int64_t j0 = 0; j0 < src.n; j0 += kTile) {
        __syncthreads();
        const int64_t jj = j0 + threadIdx.x;
        if (jj < src.n) sj[threadIdx.x] = make_dvec4(src.x[jj], src.y[jj], src.z[jj], src.m[jj]);
        __syncthreads();
        const int cnt = (int)((src.n - j0) < kTile ? (src.n - j0) : kTile);
        for (int j = 0; j < cnt; ++j) {
            const dvec4 q = sj[j];
            if (ACC) {
                double fx, fy, fz;
                pair_force64<LAW>(px, py, pz, q, G, h, h_inv, h3_inv, fx, fy, fz);
                two_sum_acc(sx, cx, fx);
                two_sum_acc(sy, cy, fy);
                two_sum_acc(sz, cz, fz);
            }
            if (POT) two_sum_acc(sp, cp, pair_pot64<LAW>(px, py, pz, q, G, h, h_inv));
        }
    }
    if (p < 0) return;
    if (ACC) {
        tg.ax[p] = sx + cx;
        tg.ay[p] = sy + cy;
        tg.az[p] = sz + cz;
    }
    if (POT) tg.pot[p] = sp + cp;
}

template <int LAW>
static cudaError_t launch_law(bool acc, bool pot, const Sources64& src, const Targets& tg,
                              double G, cudaStream_t s) {
    const int64_t grid = (tg.n + kTile - 1) / kTile;
    if (grid <= 0) return cudaSuccess;
    if (acc && pot)
        k_force_fp64<LAW, true, true><<<(unsigned)grid, kTile, 0, s>>>(src, tg, G);
    else if (acc)
        k_force_fp64<LAW, true, false><<<(unsigned)grid, kTile, 0, s>>>(src, tg, G);
    else if (pot)
        k_force_fp64<LAW, false, true><<<(unsigned)grid, kTile, 0, s>>>(src, tg, G);
    return cudaGetLastError();
}

cudaError_t launch_force_fp64(int law, bool pot, const Sources64& src, const Targets& tg,
                              double G, uint32_t* /*err*/, cudaStream_t s) {
    const bool acc = tg.ax != nullptr;
    if (law == NB_LAW_PLUMMER) return launch_law<NB_LAW_PLUMMER>(acc, pot, src, tg, G, s);
    return launch_law<NB_LAW_SPLINE_G2>(acc, pot, src, tg, G, s);
}

}  // namespace nb
