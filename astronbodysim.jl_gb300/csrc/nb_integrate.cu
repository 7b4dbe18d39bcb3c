// nb_integrate.cu -- leapfrog kick/drift, power-of-two timestep bins, device
// time line and FP64 diagnostics.  HBM-bound elementwise kernels.
//
// Built with -fmad=false: every update rounds each product and sum the way the
// reference's Julia expressions do, so given the same accelerations the
// velocities, positions and integer bins are bit-identical to the CPU path
// (src/base/Timestep.jl).
#include "nb_internal.cuh"

namespace nb {

constexpr int kBlock = 128;  // small CTAs spread small systems over more SMs (FP64 work)

static inline unsigned grid_for(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

// src/base/Timestep.jl:1-23 (CPU) and src/directsumgpu/timestep.jl:1-26 (GPU).
// Returns the power-of-two integer step; sets error bits like the CPU path's
// error() calls.
__device__ __forceinline__ int64_t get_timestep(double ax, double ay, double az, double h,
                                                const TimeCfg& c, uint32_t* err) {
    const double ac = sqrt(ax * ax + ay * ay + az * az);
    double dt;
    if (c.criterion == NB_CRIT_ETA_SQRT_EPS)
        dt = c.eta * sqrt(h / ac);
    else
        dt = sqrt(2 * c.eta * h / ac);
    if (dt > c.max_step) dt = c.max_step;
    if (dt < c.min_step) atomicOr(err, DEVERR_MINSTEP);
    const double ti_step = dt / c.time_interval;
    if (!(ti_step > 0)) atomicOr(err, DEVERR_TISTEP);
    int64_t ti_min = c.time_base;
    while (ti_min > 0 && (double)ti_min > ti_step) ti_min >>= 1;
    if (ti_min == 0) atomicOr(err, DEVERR_TISTEP);
    return ti_min;
}

// Active list: particles with Ti_endstep == system_time_int
// (src/directsum/gravity.jl:95-96), compacted in slot order (perm order when
// perm is given) by count -> exclusive scan -> scatter, so the list is the
// same on every run and consecutive entries are spatially close.
__device__ __forceinline__ bool slot_active(const int64_t* __restrict__ ti_end, int64_t n,
                                            const int32_t* __restrict__ perm, int64_t now,
                                            int64_t slot, int32_t& i) {
    i = 0;
    if (slot >= n) return false;
    i = perm ? perm[slot] : (int32_t)slot;
    return ti_end[i] == now;
}

__global__ void __launch_bounds__(kBlock) k_active_count(const int64_t* __restrict__ ti_end,
                                                         int64_t n, const int32_t* __restrict__ perm,
                                                         const Clock* __restrict__ clk,
                                                         uint32_t* __restrict__ counts) {
    int32_t i;
    const bool act = slot_active(ti_end, n, perm, clk->t_int,
                                 (int64_t)blockIdx.x * kBlock + threadIdx.x, i);
    const int c = __syncthreads_count(act);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
}

__global__ void __launch_bounds__(kBlock) k_active_scatter(const int64_t* __restrict__ ti_end,
                                                           int64_t n, const int32_t* __restrict__ perm,
                                                           Clock* clk, const uint32_t* __restrict__ offs,
                                                           int32_t* __restrict__ list) {
    __shared__ uint32_t wcount[kBlock / 32];
    int32_t i;
    const bool act = slot_active(ti_end, n, perm, clk->t_int,
                                 (int64_t)blockIdx.x * kBlock + threadIdx.x, i);
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wcount[warp] = __popc(mask);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
        if (w < warp) before += wcount[w];
        total += wcount[w];
    }
    const uint32_t base = offs[blockIdx.x];
    if (act) list[base + before + __popc(mask & ((1u << lane) - 1u))] = i;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) clk->n_active = (int32_t)(base + total);
}

int64_t active_scratch_words(int64_t n) { return (n + kBlock - 1) / kBlock + 1; }

cudaError_t launch_active_list(const int64_t* ti_end, int64_t n, const int32_t* perm, Clock* clk,
                               int32_t* list, uint32_t* scratch, cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(&clk->n_active, 0, sizeof(int32_t), s);
    const unsigned g = grid_for(n);
    k_active_count<<<g, kBlock, 0, s>>>(ti_end, n, perm, clk, scratch);
    cudaError_t e = launch_exclusive_scan(scratch, (int64_t)g, s);
    if (e != cudaSuccess) return e;
    k_active_scatter<<<g, kBlock, 0, s>>>(ti_end, n, perm, clk, scratch, list);
    return cudaGetLastError();
}

// src/base/Timestep.jl:29-39
__global__ void k_init_timesteps(const double* __restrict__ ax, const double* __restrict__ ay,
                                 const double* __restrict__ az, const int32_t* __restrict__ type,
                                 int64_t* __restrict__ ti_end, int64_t n, TimeCfg c, Clock* clk) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    if (!c.adaptive) {
        ti_end[i] = 0;
        return;
    }
    ti_end[i] = get_timestep(ax[i], ay[i], az[i], c.soft[type[i] - 1], c, &clk->err);
}

cudaError_t launch_init_timesteps(const double* ax, const double* ay, const double* az,
                                  const int32_t* type, int64_t* /*ti_beg*/, int64_t* ti_end,
                                  int64_t n, TimeCfg cfg, Clock* clk, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_init_timesteps<<<grid_for(n), kBlock, 0, s>>>(ax, ay, az, type, ti_end, n, cfg, clk);
    return cudaGetLastError();
}

// src/base/Timestep.jl:105-125
__global__ void k_half_kick(double* __restrict__ vx, double* __restrict__ vy,
                            double* __restrict__ vz, const double* __restrict__ ax,
                            const double* __restrict__ ay, const double* __restrict__ az,
                            const int64_t* __restrict__ ti_beg, const int64_t* __restrict__ ti_end,
                            int64_t n, TimeCfg c, double fw) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    if (c.adaptive) {
        const double d = (double)(ti_end[i] - ti_beg[i]);
        vx[i] = vx[i] + ax[i] * fw * 0.5 * d * c.time_interval;
        vy[i] = vy[i] + ay[i] * fw * 0.5 * d * c.time_interval;
        vz[i] = vz[i] + az[i] * fw * 0.5 * d * c.time_interval;
    } else {
        vx[i] = vx[i] + ax[i] * fw * 0.5 * c.dt;
        vy[i] = vy[i] + ay[i] * fw * 0.5 * c.dt;
        vz[i] = vz[i] + az[i] * fw * 0.5 * c.dt;
    }
}

cudaError_t launch_half_kick(double* vx, double* vy, double* vz, const double* ax,
                             const double* ay, const double* az, const int64_t* ti_beg,
                             const int64_t* ti_end, int64_t n, TimeCfg cfg, int forward,
                             cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_half_kick<<<grid_for(n), kBlock, 0, s>>>(vx, vy, vz, ax, ay, az, ti_beg, ti_end, n, cfg,
                                               (double)forward);
    return cudaGetLastError();
}

// src/base/Timestep.jl:47-93 (advance_and_find_timestep)
__global__ void k_kick(double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                       const double* __restrict__ ax, const double* __restrict__ ay,
                       const double* __restrict__ az, const int32_t* __restrict__ type,
                       int64_t* __restrict__ ti_beg, int64_t* __restrict__ ti_end, int64_t n,
                       TimeCfg c, Clock* clk) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    if (!c.adaptive) {
        vx[i] = vx[i] + ax[i] * c.dt;
        vy[i] = vy[i] + ay[i] * c.dt;
        vz[i] = vz[i] + az[i] * c.dt;
        return;
    }
    const int64_t now = clk->t_int;
    const int64_t te = ti_end[i];
    if (te != now) return;
    const int64_t TB = c.time_base;
    const double a_x = ax[i], a_y = ay[i], a_z = az[i];
    int64_t ti_step = get_timestep(a_x, a_y, a_z, c.soft[type[i] - 1], c, &clk->err);
    if (now == TB) ti_step = 0;
    if (TB - now < ti_step) ti_step = TB - now;
    const int64_t tb = ti_beg[i];
    const double tstart = (double)(tb + te) / 2;
    const double tend = (double)te + 0.5 * (double)ti_step;
    const double dt = (tend - tstart) * c.time_interval;
    vx[i] = vx[i] + a_x * dt;
    vy[i] = vy[i] + a_y * dt;
    vz[i] = vz[i] + a_z * dt;
    ti_beg[i] = te;
    ti_end[i] = te + ti_step;
    if (!(isfinite(a_x) && isfinite(a_y) && isfinite(a_z))) atomicOr(&clk->err, DEVERR_NONFINITE);
}

cudaError_t launch_kick(double* vx, double* vy, double* vz, const double* ax, const double* ay,
                        const double* az, const int32_t* type, int64_t* ti_beg, int64_t* ti_end,
                        int64_t n, TimeCfg cfg, Clock* clk, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_kick<<<grid_for(n), kBlock, 0, s>>>(vx, vy, vz, ax, ay, az, type, ti_beg, ti_end, n, cfg,
                                          clk);
    return cudaGetLastError();
}

// postprocessing_force (src/directsumgpu/gravity.jl:64-79; CPU
// src/base/PostProcessing/Force.jl:33-47), for the particles that received a
// force (Ti_endstep == t_int, or all with constant steps):
//   background field: point mass a += -GM / (r.r) * r / |r| (the attractor of
//     test/Local-Timestep.jl:746), or pseudo-Newtonian a += -GM / (|r| - r_g)^2
//     * r / |r| (src/tools/BlackHole.jl:41-60), r = x - centre;
//   then Milgrom (1983): a *= nu(|a| / ACC0, n),
//     nu(y, n) = (0.5 (1 + sqrt(1 + 4 y^-n)))^(1/n) (src/mond/milgrom1983.jl:6-8, 36-51).
// A particle with a = 0 keeps a = 0 under MOND (the limit of a nu(a)); the
// reference's expression gives 0 * Inf = NaN there.
__global__ void k_postprocess(double* __restrict__ ax, double* __restrict__ ay,
                              double* __restrict__ az, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              const int64_t* __restrict__ ti_end, int64_t n, const Clock* clk,
                              int active_only, PostCfg c) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    if (active_only && ti_end[i] != clk->t_int) return;
    double a0 = ax[i], a1 = ay[i], a2 = az[i];
    if (c.bg_kind != NB_BG_NONE) {
        const double rx = x[i] - c.cx, ry = y[i] - c.cy, rz = z[i] - c.cz;
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double r = sqrt(r2);
        double f;
        if (c.bg_kind == NB_BG_POINT_MASS) {
            f = -c.gm / r2;
        } else {
            const double d = r - c.rg;
            f = -c.gm / (d * d);
        }
        a0 = a0 + f * (rx / r);
        a1 = a1 + f * (ry / r);
        a2 = a2 + f * (rz / r);
    }
    if (c.mond == NB_MOND_MILGROM1983) {
        const double an = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
        if (an > 0.0) {
            const double yy = an / c.acc0;
            const double nu = pow(0.5 * (1.0 + sqrt(1.0 + 4.0 * pow(yy, -c.nu_index))), 1.0 / c.nu_index);
            a0 = a0 * nu;
            a1 = a1 * nu;
            a2 = a2 * nu;
        }
    }
    ax[i] = a0;
    ay[i] = a1;
    az[i] = a2;
}

cudaError_t launch_postprocess(double* ax, double* ay, double* az, const double* x, const double* y,
                               const double* z, const int64_t* ti_end, int64_t n, const Clock* clk,
                               int active_only, PostCfg c, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_postprocess<<<grid_for(n), kBlock, 0, s>>>(ax, ay, az, x, y, z, ti_end, n, clk, active_only, c);
    return cudaGetLastError();
}

// src/base/Timestep.jl:135-144 -- min over Ti_endstep and TimeBase.
__global__ void k_min_reset(Clock* clk, int64_t time_base) { clk->min_endstep = time_base; }

__global__ void k_min_endstep(const int64_t* __restrict__ ti_end, int64_t n, Clock* clk) {
    __shared__ long long red[kBlock / 32];
    long long v = LLONG_MAX;
    for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBlock)
        v = min(v, (long long)ti_end[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBlock / 32; ++w) v = min(v, red[w]);
        atomicMin(reinterpret_cast<long long*>(&clk->min_endstep), v);
    }
}

cudaError_t launch_min_endstep(const int64_t* ti_end, int64_t n, int64_t time_base, Clock* clk,
                               cudaStream_t s) {
    k_min_reset<<<1, 1, 0, s>>>(clk, time_base);
    if (n > 0) {
        int64_t g = (n + kBlock - 1) / kBlock;
        if (g > 1216) g = 1216;
        k_min_endstep<<<(unsigned)g, kBlock, 0, s>>>(ti_end, n, clk);
    }
    return cudaGetLastError();
}

// check_sync_point_local (src/base/Timestep.jl:146-157): counts the particles
// with Ti_endstep > min_endstep (the value of the last find_min_endstep); all
// of them are past it exactly at a full synchronisation point.
__global__ void k_sync_count(const int64_t* __restrict__ ti_end, int64_t n, const Clock* clk,
                             unsigned long long* count) {
    __shared__ unsigned long long red[kBlock / 32];
    const int64_t m = clk->min_endstep;
    unsigned long long c = 0;
    for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBlock)
        c += ti_end[i] > m ? 1ull : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBlock / 32; ++w) c += red[w];
        atomicAdd(count, c);
    }
}

cudaError_t launch_sync_count(const int64_t* ti_end, int64_t n, const Clock* clk,
                              unsigned long long* count, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || n <= 0) return e;
    int64_t g = (n + kBlock - 1) / kBlock;
    if (g > 1216) g = 1216;
    k_sync_count<<<(unsigned)g, kBlock, 0, s>>>(ti_end, n, clk, count);
    return cudaGetLastError();
}

// Clock advance before a drift (single thread).
//   mode 0: adaptive, to min_endstep       (src/directsum/timestep.jl:1-20)
//   mode 1: adaptive, to t_int_arg
//   mode 2: constant, to t_float + dt      (src/base/Timestep.jl:197-215)
//   mode 3: constant, to t_float_arg
__global__ void k_clock_advance(Clock* clk, TimeCfg c, int mode, int64_t t_int_arg,
                                double t_float_arg) {
    if (mode == 0 || mode == 1) {
        const int64_t next = mode == 0 ? clk->min_endstep : t_int_arg;
        clk->last_t_int = clk->t_int;
        clk->t_int = next;
        clk->t_float = c.time_begin + (double)clk->t_int * c.time_interval;
        clk->dt_drift = (double)(clk->t_int - clk->last_t_int) * c.time_interval;
    } else {
        const double next = mode == 2 ? clk->t_float + c.dt : t_float_arg;
        clk->last_t_float = clk->t_float;
        clk->t_float = next;
        clk->dt_drift = clk->t_float - clk->last_t_float;
    }
}

// src/base/Timestep.jl:169-191
__global__ void k_drift(double* __restrict__ x, double* __restrict__ y, double* __restrict__ z,
                        const double* __restrict__ vx, const double* __restrict__ vy,
                        const double* __restrict__ vz, int64_t n, const Clock* __restrict__ clk) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    const double dt = clk->dt_drift;
    x[i] = x[i] + vx[i] * dt;
    y[i] = y[i] + vy[i] * dt;
    z[i] = z[i] + vz[i] * dt;
}

cudaError_t launch_drift(double* x, double* y, double* z, const double* vx, const double* vy,
                         const double* vz, int64_t n, TimeCfg cfg, Clock* clk, int mode,
                         int64_t t_int_arg, double t_float_arg, cudaStream_t s) {
    k_clock_advance<<<1, 1, 0, s>>>(clk, cfg, mode, t_int_arg, t_float_arg);
    if (n > 0) k_drift<<<grid_for(n), kBlock, 0, s>>>(x, y, z, vx, vy, vz, n, clk);
    return cudaGetLastError();
}

// find_next_sync_point_and_drift with snapshots (src/base/Timestep.jl:197-215
// constant, :224-245 adaptive), one event per graph replay (single thread).
// The step ends at t_float + dt (constant) or at min_endstep (adaptive); while
// the next output time is at or before that end, the reference drifts to the
// output time, writes the snapshot and moves the output time on by
// BetweenSnapshots.  Here the clock advances to that output time, the
// condition of the force/kick branch is 0, and at_output stops further
// replays until the host has written the snapshot and cleared it; the next
// replay continues the same step (mid_step) towards the next output or the
// step's end.  The clock arithmetic is the reference's: t_float = Begin +
// t_int * TimeInterval and drift interval (t_int - last) * TimeInterval for
// adaptive steps, drift interval t_float - last_t_float for constant steps.
__global__ void k_clock_plan(Clock* clk, TimeCfg c, cudaGraphConditionalHandle cond) {
    if (clk->at_output) {
        clk->drift_skip = 1;
        cudaGraphSetConditional(cond, 0u);
        return;
    }
    clk->drift_skip = 0;
    bool stop;
    if (c.adaptive) {
        const int64_t target = clk->mid_step ? clk->step_target_int : clk->min_endstep;
        stop = c.outputs_on && clk->next_out_int <= target;
        const int64_t next = stop ? clk->next_out_int : target;
        if (stop) {
            clk->step_target_int = target;
            clk->next_out_int += c.between_int;
        }
        clk->last_t_int = clk->t_int;
        clk->t_int = next;
        clk->t_float = c.time_begin + (double)clk->t_int * c.time_interval;
        clk->dt_drift = (double)(clk->t_int - clk->last_t_int) * c.time_interval;
    } else {
        const double target = clk->mid_step ? clk->step_target_float : clk->t_float + c.dt;
        stop = c.outputs_on && clk->next_out_float <= target;
        const double next = stop ? clk->next_out_float : target;
        if (stop) {
            clk->step_target_float = target;
            clk->next_out_float += c.between_float;
        }
        clk->last_t_float = clk->t_float;
        clk->t_float = next;
        clk->dt_drift = clk->t_float - clk->last_t_float;
    }
    clk->mid_step = stop ? 1 : 0;
    clk->at_output = stop ? 1 : 0;
    if (stop) clk->outputs += 1;
    cudaGraphSetConditional(cond, stop ? 0u : 1u);
}

// k_drift of a replay planned by k_clock_plan (no-op when drift_skip is set).
__global__ void k_drift_gated(double* __restrict__ x, double* __restrict__ y,
                              double* __restrict__ z, const double* __restrict__ vx,
                              const double* __restrict__ vy, const double* __restrict__ vz,
                              int64_t n, const Clock* __restrict__ clk) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n || clk->drift_skip) return;
    const double dt = clk->dt_drift;
    x[i] = x[i] + vx[i] * dt;
    y[i] = y[i] + vy[i] * dt;
    z[i] = z[i] + vz[i] * dt;
}

cudaError_t launch_plan_and_drift(double* x, double* y, double* z, const double* vx,
                                  const double* vy, const double* vz, int64_t n, TimeCfg cfg,
                                  Clock* clk, cudaGraphConditionalHandle cond, cudaStream_t s) {
    k_clock_plan<<<1, 1, 0, s>>>(clk, cfg, cond);
    if (n > 0) k_drift_gated<<<grid_for(n), kBlock, 0, s>>>(x, y, z, vx, vy, vz, n, clk);
    return cudaGetLastError();
}

__global__ void k_clock_end_step(Clock* clk, int adaptive, int64_t n) {
    if (!adaptive) clk->last_t_float = clk->t_float;  // src/run.jl:164
    const double targets = adaptive ? (double)clk->n_active : (double)n;
    clk->interactions += targets * (double)n;
    clk->steps += 1;
}

cudaError_t launch_clock_end_step(Clock* clk, int adaptive, int64_t n, cudaStream_t s) {
    k_clock_end_step<<<1, 1, 0, s>>>(clk, adaptive, n);
    return cudaGetLastError();
}

// src/base/Potential.jl:5-24
__global__ void k_remove_self_potential(double* __restrict__ pot, const double* __restrict__ m,
                                        const int32_t* __restrict__ type, int64_t n, TimeCfg c,
                                        double G) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    pot[i] = pot[i] + G * m[i] / (c.soft[type[i] - 1] / 2.8);
}

cudaError_t launch_remove_self_potential(double* pot, const double* m, const int32_t* type,
                                         int64_t n, TimeCfg cfg, double G, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_remove_self_potential<<<grid_for(n), kBlock, 0, s>>>(pot, m, type, n, cfg, G);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 diagnostics (src/base/Energy.jl:13-101): per-block partials into
// scratch, then one block sums the partials in a fixed order.  Deterministic.
// ---------------------------------------------------------------------------
constexpr int kDiagBlock = 256;
constexpr int kDiagQ = 8;

__global__ void __launch_bounds__(kDiagBlock)
    k_diag_partial(const double* __restrict__ x, const double* __restrict__ y,
                   const double* __restrict__ z, const double* __restrict__ vx,
                   const double* __restrict__ vy, const double* __restrict__ vz,
                   const double* __restrict__ m, const double* __restrict__ pot, int64_t n,
                   double* __restrict__ partial) {
    __shared__ double red[kDiagQ][kDiagBlock / 32];
    double q[kDiagQ];
#pragma unroll
    for (int k = 0; k < kDiagQ; ++k) q[k] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kDiagBlock + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kDiagBlock) {
        const double mi = m[i], px = x[i], py = y[i], pz = z[i];
        const double ux = vx[i], uy = vy[i], uz = vz[i];
        const double hm = 0.5 * mi;
        q[0] += (hm * ux) * ux + (hm * uy) * uy + (hm * uz) * uz;
        q[1] += pot ? pot[i] * mi : 0.0;
        q[2] += ux * mi;
        q[3] += uy * mi;
        q[4] += uz * mi;
        q[5] += mi * (py * uz - pz * uy);
        q[6] += mi * (pz * ux - px * uz);
        q[7] += mi * (px * uy - py * ux);
    }
#pragma unroll
    for (int k = 0; k < kDiagQ; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q[k] += __shfl_xor_sync(0xffffffffu, q[k], o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < kDiagQ; ++k) red[k][threadIdx.x >> 5] = q[k];
    }
    __syncthreads();
    if (threadIdx.x < kDiagQ) {
        double s = 0.0;
        for (int w = 0; w < kDiagBlock / 32; ++w) s += red[threadIdx.x][w];
        partial[(int64_t)blockIdx.x * kDiagQ + threadIdx.x] = s;
    }
}

__global__ void k_diag_final(const double* __restrict__ partial, int64_t nblocks,
                             double* __restrict__ out8) {
    // One warp per quantity, compensated sum over the partials in fixed order.
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= kDiagQ) return;
    double s = 0.0, c = 0.0;
    for (int64_t b = lane; b < nblocks; b += 32) two_sum_acc(s, c, partial[b * kDiagQ + k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double so = __shfl_xor_sync(0xffffffffu, s, o);
        const double co = __shfl_xor_sync(0xffffffffu, c, o);
        two_sum_acc(s, c, so);
        c += co;
    }
    if (lane == 0) out8[k] = (k == 1 ? 0.5 : 1.0) * (s + c);
}

int64_t diag_scratch_doubles(int64_t n) {
    int64_t g = (n + kDiagBlock - 1) / kDiagBlock;
    if (g > 1216) g = 1216;
    if (g < 1) g = 1;
    return g * kDiagQ;
}

cudaError_t launch_diag(const double* x, const double* y, const double* z, const double* vx,
                        const double* vy, const double* vz, const double* m, const double* pot,
                        int64_t n, double* scratch, int64_t scratch_blocks, double* out8,
                        cudaStream_t s) {
    int64_t g = scratch_blocks;
    if (g < 1) g = 1;
    k_diag_partial<<<(unsigned)g, kDiagBlock, 0, s>>>(x, y, z, vx, vy, vz, m, pot, n, scratch);
    k_diag_final<<<1, 32 * kDiagQ, 0, s>>>(scratch, g, out8);
    return cudaGetLastError();
}

}  // namespace nb
