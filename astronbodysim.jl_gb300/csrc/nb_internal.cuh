// nb_internal.cuh -- device-side layout, kernel argument blocks and PTX helpers
// shared by the translation units of libnbody_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nbody_gb300.h"

namespace nb {

// 32-byte aligned FP64 quadruple (tile origins, staged FP64 sources).
struct __align__(32) dvec4 {
    double x, y, z, w;
};
__host__ __device__ __forceinline__ dvec4 make_dvec4(double x, double y, double z, double w) {
    return dvec4{x, y, z, w};
}

// FP64 tile origin (or target position) held as an unevaluated sum of two
// floats, v = hi + lo with lo = fl(v - hi).  x - o then costs three FP32
// operations, (x.hi - o.hi) + (x.lo - o.lo), within about one FP32 ulp of the
// FP64 difference rounded once, so the force kernels' per-tile re-origin
// needs no FP64 instruction.  hi.w carries the tile's half diagonal.
struct __align__(16) TileOrigin {
    float4 hi;
    float4 lo;
};
__device__ __forceinline__ float2 split_df(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ TileOrigin make_tile_origin(double x, double y, double z, double w) {
    const float2 a = split_df(x), b = split_df(y), c = split_df(z);
    TileOrigin o;
    o.hi = make_float4(a.x, b.x, c.x, (float)w);
    o.lo = make_float4(a.y, b.y, c.y, 0.0f);
    return o;
}
// FP32 coordinate of a split position t relative to a split origin (oh, ol).
__device__ __forceinline__ float rel_df(float2 t, float oh, float ol) {
    return __fadd_rn(__fsub_rn(t.x, oh), __fsub_rn(t.y, ol));
}

// Device error word bits (read back by the host after synchronising calls).
enum : uint32_t {
    DEVERR_NONFINITE = 1u,  // NaN/Inf acceleration
    DEVERR_MINSTEP = 2u,    // dt < MinStep   (src/base/Timestep.jl:9-11)
    DEVERR_TISTEP = 4u,     // ti_step <= 0   (src/base/Timestep.jl:13-16)
    DEVERR_TIMEOUT = 8u,    // bounded mbarrier wait gave up
};

// Device-resident time line (TimeInfo) and per-step scalars.
struct Clock {
    int64_t t_int;          // system_time_int
    int64_t last_t_int;     // last_system_time_int
    int64_t min_endstep;    // find_min_endstep result
    double t_float;         // system_time_float
    double last_t_float;    // last_system_time_float
    double dt_drift;        // interval of the pending drift
    int32_t n_active;       // active particles at t_int
    uint32_t err;           // DEVERR_* bits
    double interactions;    // sum over steps of (targets x sources)
    int64_t steps;          // steps taken through the step graph
    // Snapshot schedule (TimeInfo.next_output_time_int / _float,
    // src/base/Config.jl:732-733, 749-750) and the state of a step that
    // stopped at an output time inside it (find_next_sync_point_and_drift,
    // src/base/Timestep.jl:197-245).
    int64_t next_out_int;     // next output time on the integer time line
    double next_out_float;    // next output time (constant steps)
    int64_t step_target_int;  // end of the step being split (adaptive)
    double step_target_float; // end of the step being split (constant)
    int32_t mid_step;         // 1: positions sit at an output time inside a step
    int32_t at_output;        // 1: stopped at an output, waiting for the host
    int32_t drift_skip;       // 1: the gated drift of this replay does nothing
    int32_t pad;
    int64_t outputs;          // output stops so far
};

// Timestep configuration passed by value.
struct TimeCfg {
    int32_t adaptive;
    int32_t criterion;
    double dt;
    double eta;
    double min_step;
    double max_step;
    int64_t time_base;
    double time_interval;
    double time_begin;
    double soft[6];
    // Snapshot interval (TimeConfig.BetweenSnapshots / BetweenSnapshotsInt,
    // src/base/Config.jl:392-394, 436-439); outputs_on 0 = no output stops.
    int32_t outputs_on;
    int32_t pad;
    double between_float;
    int64_t between_int;
};

// Targets of a force evaluation.  Target slot t maps to particle idx[t]
// (identity when idx == nullptr); positions and outputs are indexed by the
// particle index.  The number of targets is *d_count when d_count != nullptr,
// else n.
struct Targets {
    const double* x;
    const double* y;
    const double* z;
    const int32_t* type;  // softening table index 1..6; nullptr -> h_const
    const int32_t* idx;
    const int32_t* d_count;
    int64_t n;
    double soft[6];
    double h_const;
    double* ax;
    double* ay;
    double* az;
    double* pot;  // nullptr -> no potential
    // Plummer law only: targets are also sources at the same FP32 position
    // (the self pair contributes -m/h to the potential and is removed).
    const double* self_mass;
};

// Packed FP32 sources for the mixed kernel: j-tiles of tile_j particles,
// float4 (x - o, y - o, z - o, m) with an FP64 origin o per tile.
struct Sources32 {
    const float4* pack;
    const TileOrigin* origin;
    const float4* ext;  // per tile: half extents of the box (x, y, z) and half diagonal
    int32_t ntiles;
    int32_t tile_j;
    // j-split: each i-block's tiles are shared by jsplit CTAs, which write
    // compensated partials (partial[(part * 8 + q) * pstride + slot]) that
    // k_force_join adds in part order.  jsplit 1: no partials.
    int32_t jsplit;
    int32_t pad;
    float* partial;
    int64_t pstride;
};

// FP64 sources.
struct Sources64 {
    const double* x;
    const double* y;
    const double* z;
    const double* m;
    int64_t n;
};

// One independent system of a work-list force evaluation (device memory).
struct SysDesc {
    int64_t off;       // first particle: index into the SoA arrays and into perm
    int64_t ubase;     // first work unit of the system
    int32_t n;         // particles (targets and sources)
    int32_t tile_off;  // first packed j-tile
    int32_t ntiles;    // ceil(n / 256) j-tiles
    int32_t nblocks;   // ceil(n / 256) i-blocks of targets
    double soft[6];    // softening by particle type
};

// Persistent work-list force over nsys systems (nb_force_worklist.cu).
struct WorkList {
    const SysDesc* sys;
    int32_t nsys;
    int32_t grid;              // persistent CTAs; also the fix-up's partition
    int64_t units;             // sum over systems of nblocks * ntiles
    const int32_t* active;     // one system only: targets = active[0 .. *d_count)
    const int32_t* d_count;
    const int32_t* perm;       // otherwise target slot q of system s is particle perm[off + q]
    const float4* pack;
    const TileOrigin* origin;
    const float4* ext;
    const double* x;
    const double* y;
    const double* z;
    const double* m;
    const int32_t* type;       // nullptr -> soft[0]
    double* ax;                // nullptr -> potential only
    double* ay;
    double* az;
    double* pot;               // nullptr -> no potential
    float* partial;            // worklist_partial_bytes(grid)
    double G;
    uint32_t* err;
    int32_t block_cyclic;      // one system: CTA c takes whole i-blocks c, c + grid, ...
    int32_t pad;
};

cudaError_t launch_force_worklist(int law, const WorkList& w, cudaStream_t s);
int worklist_ctas_per_sm(int law, bool acc, bool pot);
size_t worklist_partial_bytes(int64_t grid);
int worklist_block_targets();

// Many-system engine (nb_batch.cu, nb_engine.cu).
struct BatchSys {
    int64_t aoff;  // first arena particle
    int64_t soff;  // first sorted slot
    int32_t n;
    int32_t slot;
};

struct BatchForce {
    const SysDesc* sys;   // by rank; off = first sorted slot
    const int2* items;    // (rank, i-block), largest systems first
    // sys[r].off is the system's first arena particle and perm its
    // arena-relative Morton order: slot q is particle off + perm[off + q]
    int32_t nitems;
    int32_t pad;
    int32_t* counter;     // claim counter, zeroed by the launch
    const int32_t* perm;  // sorted slot -> arena particle
    const float4* pack;
    const TileOrigin* origin;
    const float4* ext;
    const double* x;
    const double* y;
    const double* z;
    const double* m;
    double* ax;
    double* ay;
    double* az;
    double* pot;
    double G;
    uint32_t* err;
    // Optional kick fused into the epilogue (the engine's step): with vx set,
    // each target's velocity takes v += a * dt_slot[s] * fac_slot[s] exactly
    // as k_batch_kick would apply it right after the force (s = sysid[p]).
    double* vx;
    double* vy;
    double* vz;
    const int32_t* sysid;
    const double* dt_slot;
    const double* fac_slot;
    // Optional per-slot gate (the engine's step): a system whose own step
    // count has reached its target (steps_slot[s] >= nsteps_slot[s]) is
    // skipped, so it stays where its last step left it.
    const int64_t* steps_slot;
    const int64_t* nsteps_slot;
};

cudaError_t launch_force_batch(int law, const BatchForce& f, int grid, int block, int ipt,
                               cudaStream_t s);
cudaError_t launch_fill_i32(int32_t* a, int64_t n, int32_t v, cudaStream_t s);
int batch_ctas_per_sm(int law, bool acc, bool pot, int block, int ipt);
bool batch_shape_ok(int block, int ipt);
int batch_block_targets(int block, int ipt);
// Morton order of the systems too large for the shared-memory sort ("large"
// systems, listed by rank in ranks[0 .. nlarge)): their particles only, at
// compact offsets BatchSys::soff (0 .. nl), are keyed (large index << 42 |
// 14-bit-per-axis Morton code over the system's box) and radix-sorted.  The
// boxes are reduced with atomics on order-preserving integer images of the
// coordinates into box_key (6 per large system, reset to all ones first).
// Grids are (chunks of the largest system) x nlarge.
cudaError_t launch_batch_large_keys(const BatchSys* bs, const int32_t* ranks, int32_t nlarge,
                                    int32_t max_n, const double* x, const double* y, const double* z,
                                    unsigned long long* box_key, uint64_t* keys, int32_t* vals,
                                    cudaStream_t s);
cudaError_t launch_batch_pack(const int32_t* tile_rank, int32_t ntiles, const SysDesc* sys,
                              const double* bbox, const int32_t* perm, const double* x,
                              const double* y, const double* z, const double* m, float4* pack,
                              TileOrigin* origin, float4* ext, const int32_t* sysid,
                              const int64_t* steps_slot, const int64_t* nsteps_slot,
                              cudaStream_t s);
int batch_small_sort_limit();
cudaError_t prepare_batch_sort_small();
cudaError_t launch_batch_sort_small(const BatchSys* bs, int32_t nrank, int32_t max_small_n,
                                    const int64_t* steps_slot, const int64_t* nsteps_slot,
                                    int32_t every, int32_t force_all, const double* x,
                                    const double* y, const double* z, double* bbox, int32_t* lperm,
                                    cudaStream_t s);
cudaError_t launch_batch_perm_to_local(const BatchSys* bs, const int32_t* ranks, int32_t nlarge,
                                       int32_t max_n, const int32_t* perm, int32_t* lperm,
                                       cudaStream_t s);
cudaError_t launch_batch_tick(const BatchSys* bs, int32_t nrank, int64_t* steps_slot,
                              const int64_t* nsteps_slot, cudaStream_t s);
cudaError_t launch_batch_drift(double* x, double* y, double* z, const double* vx, const double* vy,
                               const double* vz, const int32_t* sysid, const double* dt_slot,
                               const double* fac_slot, const int64_t* steps_slot,
                               const int64_t* nsteps_slot, int64_t n, cudaStream_t s);
cudaError_t launch_batch_kick(double* vx, double* vy, double* vz, const double* ax,
                              const double* ay, const double* az, const int32_t* sysid,
                              const double* dt_slot, const double* fac_slot, int64_t n,
                              cudaStream_t s);

// Launch helpers implemented in the .cu files.
cudaError_t launch_pack(const double* x, const double* y, const double* z, const double* m,
                        int64_t n, const int32_t* perm, int tile_j, float4* pack,
                        TileOrigin* origin, float4* ext, cudaStream_t s);
// Morton-order permutation of the particles (nb_sort.cu); scratch of
// sort_scratch_bytes(n) bytes.
size_t sort_scratch_bytes(int64_t n);
cudaError_t launch_morton_sort(const double* x, const double* y, const double* z, int64_t n,
                               void* scratch, int32_t* perm, cudaStream_t s);
uint64_t* sort_keys_buffer(void* scratch, int64_t n);
cudaError_t launch_sort_keys(void* scratch, int64_t n, int32_t* vals, int passes, cudaStream_t s);
// Tile sizes of the packed sources: 128, 256 or 512 (src.tile_j); stages:
// depth of the force kernel's shared-memory ring (3, 4, 6; see
// nb_force_mixed.cuh for the combinations compiled).
cudaError_t launch_force_mixed(int law, bool pot, const Sources32& src, const Targets& tg,
                               double G, uint32_t* err, int block, int ipt, cudaStream_t s,
                               int stages = 4);
bool tile_size_ok(int tile_j);
cudaError_t launch_force_fp64(int law, bool pot, const Sources64& src, const Targets& tg,
                              double G, uint32_t* err, cudaStream_t s);

// Integrator kernels (nb_integrate.cu).
// Active list (Ti_endstep == t_int); slots are scanned in perm order when perm
// is given, so consecutive list entries stay spatially close.
cudaError_t launch_active_list(const int64_t* ti_end, int64_t n, const int32_t* perm, Clock* clk,
                               int32_t* list, uint32_t* scratch, cudaStream_t s);
int64_t active_scratch_words(int64_t n);
cudaError_t launch_exclusive_scan(uint32_t* counts, int64_t len, cudaStream_t s);
cudaError_t launch_init_timesteps(const double* ax, const double* ay, const double* az,
                                  const int32_t* type, int64_t* ti_beg, int64_t* ti_end, int64_t n,
                                  TimeCfg cfg, Clock* clk, cudaStream_t s);
cudaError_t launch_half_kick(double* vx, double* vy, double* vz, const double* ax,
                             const double* ay, const double* az, const int64_t* ti_beg,
                             const int64_t* ti_end, int64_t n, TimeCfg cfg, int forward,
                             cudaStream_t s);
// Particles with Ti_endstep > clk->min_endstep, counted into *count.
cudaError_t launch_sync_count(const int64_t* ti_end, int64_t n, const Clock* clk,
                              unsigned long long* count, cudaStream_t s);

// Force post-processing (background field, then Milgrom MOND); see nb_params.
struct PostCfg {
    int32_t bg_kind;
    int32_t mond;
    double gm;
    double cx, cy, cz;
    double rg;
    double acc0;
    double nu_index;
};
cudaError_t launch_postprocess(double* ax, double* ay, double* az, const double* x, const double* y,
                               const double* z, const int64_t* ti_end, int64_t n, const Clock* clk,
                               int active_only, PostCfg c, cudaStream_t s);

cudaError_t launch_kick(double* vx, double* vy, double* vz, const double* ax, const double* ay,
                        const double* az, const int32_t* type, int64_t* ti_beg, int64_t* ti_end,
                        int64_t n, TimeCfg cfg, Clock* clk, cudaStream_t s);
cudaError_t launch_min_endstep(const int64_t* ti_end, int64_t n, int64_t time_base, Clock* clk,
                               cudaStream_t s);
// mode 0: drift to clk->min_endstep (adaptive); 1: to t_int_arg; 2: float t + dt (const step);
// 3: to t_float_arg.
cudaError_t launch_drift(double* x, double* y, double* z, const double* vx, const double* vy,
                         const double* vz, int64_t n, TimeCfg cfg, Clock* clk, int mode,
                         int64_t t_int_arg, double t_float_arg, cudaStream_t s);
cudaError_t launch_clock_end_step(Clock* clk, int adaptive, int64_t n, cudaStream_t s);
// One event of find_next_sync_point_and_drift (src/base/Timestep.jl:197-245):
// the clock advances to the next output time when it falls inside the step
// (setting at_output and the graph condition to 0), else to the step's end
// (condition 1: force and kick follow); then the gated drift.  A replay that
// finds at_output still set does nothing.
cudaError_t launch_plan_and_drift(double* x, double* y, double* z, const double* vx,
                                  const double* vy, const double* vz, int64_t n, TimeCfg cfg,
                                  Clock* clk, cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t launch_diag(const double* x, const double* y, const double* z, const double* vx,
                        const double* vy, const double* vz, const double* m, const double* pot,
                        int64_t n, double* scratch, int64_t scratch_blocks, double* out8,
                        cudaStream_t s);
int64_t diag_scratch_doubles(int64_t n);
cudaError_t launch_remove_self_potential(double* pot, const double* m, const int32_t* type,
                                         int64_t n, TimeCfg cfg, double G, cudaStream_t s);

// ---------------------------------------------------------------------------
// PTX helpers (sm_90+ mbarrier / bulk async copy).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after ~timeout_ns of wall time (globaltimer, read
// after every try_wait, each of which suspends for at most a system-defined
// slice) or an iteration cap, whichever comes first.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t timeout_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > timeout_ns) return false;
    }
    return false;
}

// Bulk global->shared copy completing on an mbarrier (no multicast).
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Approximate reciprocal (MUFU), flushing subnormals; used for r^-2 so that
// m r^-3 = (m r^-1) * r^-2 costs one FP32 multiply after the two MUFU ops.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Knuth TwoSum accumulation: (s, c) += v with the rounding error of s + v
// carried in c.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float v) {
    float t = s + v;
    float bp = t - s;
    float e = (s - (t - bp)) + (v - bp);
    s = t;
    c += e;
}

__device__ __forceinline__ void two_sum_acc(double& s, double& c, double v) {
    double t = __dadd_rn(s, v);
    double bp = __dadd_rn(t, -s);
    double e = __dadd_rn(__dadd_rn(s, -__dadd_rn(t, -bp)), __dadd_rn(v, -bp));
    s = t;
    c = __dadd_rn(c, e);
}

}  // namespace nb
