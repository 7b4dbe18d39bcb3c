// nb_api.cu -- the C ABI of libnbody_gb300.so: handle life cycle, uploads,
// downloads, and the DirectSum-on-GPU operations of AstroNbodySim.jl
// (src/directsumgpu/gravity.jl, src/directsumgpu/timestep.jl) re-expressed as
// launches of this library's kernels on the handle's stream.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nb_internal.cuh"

using nb::Clock;
using nb::TimeCfg;

struct nb_handle {
    nb_params p{};
    TimeCfg tc{};
    int dev = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int64_t n = 0;
    int64_t cap = 0;
    void* arena = nullptr;
    double *x = nullptr, *y = nullptr, *z = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr;
    double *pot = nullptr, *m = nullptr;
    int32_t* type = nullptr;
    int64_t *ti_beg = nullptr, *ti_end = nullptr;
    int32_t* active = nullptr;
    int32_t* perm = nullptr;
    uint32_t* act_scratch = nullptr;
    void* sort_scratch = nullptr;
    float4* pack = nullptr;
    nb::TileOrigin* origin = nullptr;
    float4* ext = nullptr;
    int32_t ntiles = 0;
    double* diag_scratch = nullptr;
    int64_t diag_blocks = 0;
    double* diag_out = nullptr;
    Clock* clk = nullptr;
    void* probe = nullptr;
    size_t probe_bytes = 0;
    // Step graphs: [0] re-orders the sources (Morton sort) before the pack,
    // [1] packs in the order of the last sort.  The host replays [0] every
    // resort steps (and whenever the order is not valid) and [1] otherwise.
    cudaGraphExec_t step_exec = nullptr;
    cudaGraphExec_t step_exec_nosort = nullptr;
    cudaGraphExec_t out_exec = nullptr;  // step graph that stops at output times
    cudaGraphExec_t out_exec_nosort = nullptr;
    int resort = 16;                      // steps between Morton sorts in the step graphs
    bool perm_valid = false;              // perm holds an order of the current particles
    int64_t host_steps = 0;               // steps completed by step graphs (device clock)
    double between = 0.0;                 // BetweenSnapshots (0: no output stops)
    int block = 128;
    int ipt = 2;
    bool worklist = false;     // persistent work-list kernel forced (block == -1)
    bool auto_cfg = true;      // kernel and shape chosen per N
    int wl_mode = 0;           // 0: even unit split, 1: block-cyclic whole blocks
    int nsm = 0;
    int wl_occ[2][3] = {};     // CTAs per SM of k_force_worklist [law][acc, acc+pot, pot]
    nb::SysDesc* sysdesc = nullptr;
    float* partial = nullptr;
    size_t partial_bytes = 0;
    int jsplit = 1;
    int tj = 256;               // sources per packed j-tile (128, 256, 512)
    int stages = 4;             // depth of the force kernel's copy ring
    int jalloc = 1;             // j-split the arena's partial buffer holds
    float* jpartial = nullptr;  // j-split partials (arena)
    int64_t jstride = 0;
    std::string err;
};

namespace {

constexpr int kTileJ = 256;
// Built-in launch rule (the autotuner's choices on GB300, both laws, rounded
// to four size classes): the direct grid of 128-thread CTAs with each
// i-block's tiles split over several CTAs --
//   N <  2^15: one target per thread, j-split 4, tiles of 128;
//   N >= 2^15: one target per thread, j-split 8, tiles of 256;
//   N >= 2^16: two targets per thread, j-split 8, tiles of 256;
//   N >= 2^17: the same with tiles of 512 (N = 2^20: 345 ms per force against
//              367 ms with tiles of 256).
constexpr int kAutoJsplitMax = 8;
constexpr int64_t kAutoTile256From = 1 << 15;
constexpr int64_t kAutoIpt2From = 1 << 16;
constexpr int64_t kAutoTile512From = 1 << 17;

int auto_jsplit(int64_t n) { return n >= kAutoTile256From ? 8 : 4; }
int auto_tile(int64_t n) { return n >= kAutoTile512From ? 512 : (n >= kAutoTile256From ? 256 : 128); }

// Reason the last nb_create on this thread failed (there is no handle to hold it).
thread_local std::string g_create_err;

int fail(nb_handle* h, int code, const char* fmt, ...) {
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

#define NB_CK(call)                                                                            \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(h, e_ == cudaErrorMemoryAllocation ? NB_ERR_OOM : NB_ERR_CUDA,       \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

TimeCfg make_timecfg(const nb_params& p, double between) {
    TimeCfg c{};
    c.adaptive = p.adaptive;
    c.criterion = p.criterion;
    c.dt = p.dt;
    c.eta = p.eta;
    c.min_step = p.min_step;
    c.max_step = p.max_step;
    c.time_base = p.time_base;
    c.time_interval = (p.time_end - p.time_begin) / (double)p.time_base;
    c.time_begin = p.time_begin;
    for (int k = 0; k < 6; ++k) c.soft[k] = p.softening[k];
    // BetweenSnapshotsInt = floor(BetweenSnapshots / TimeInterval) for adaptive
    // steps, 0 for constant steps (src/base/Config.jl:436-439)
    c.between_float = between;
    c.between_int = p.adaptive ? (int64_t)std::floor(between / c.time_interval) : 0;
    c.outputs_on = between > 0.0 ? 1 : 0;
    return c;
}

// TimeInfo at construction (src/base/Config.jl:742-761): t = Begin, first
// output at Begin + BetweenSnapshots (integer line: BetweenSnapshotsInt).
Clock initial_clock(const nb_params& p, const TimeCfg& tc) {
    Clock c{};
    c.t_float = p.time_begin;
    c.last_t_float = p.time_begin;
    c.next_out_int = tc.between_int;
    c.next_out_float = p.time_begin + tc.between_float;
    return c;
}

int check_params(nb_handle* h, const nb_params* p) {
    if (!(p->law == NB_LAW_SPLINE_G2 || p->law == NB_LAW_PLUMMER))
        return fail(h, NB_ERR_INVALID_ARG, "law must be NB_LAW_SPLINE_G2 or NB_LAW_PLUMMER");
    if (!(p->precision == NB_PREC_FP64 || p->precision == NB_PREC_MIXED))
        return fail(h, NB_ERR_INVALID_ARG, "precision must be NB_PREC_FP64 or NB_PREC_MIXED");
    if (!(p->criterion == NB_CRIT_REF || p->criterion == NB_CRIT_ETA_SQRT_EPS))
        return fail(h, NB_ERR_INVALID_ARG, "unknown timestep criterion");
    for (int k = 0; k < 6; ++k)
        if (!(p->softening[k] > 0.0) || !std::isfinite(p->softening[k]))
            return fail(h, NB_ERR_INVALID_ARG, "softening[%d] must be finite and > 0", k);
    if (!p->adaptive && !(p->dt > 0.0))
        return fail(h, NB_ERR_INVALID_ARG, "constant timestep needs dt > 0");
    if (p->adaptive) {
        if (p->time_base <= 0 || (p->time_base & (p->time_base - 1)) != 0)
            return fail(h, NB_ERR_INVALID_ARG, "time_base must be a power of two");
        if (!(p->time_end > p->time_begin))
            return fail(h, NB_ERR_INVALID_ARG, "time_end must exceed time_begin");
        if (!(p->eta > 0.0)) return fail(h, NB_ERR_INVALID_ARG, "eta must be > 0");
    }
    const int b = p->block, i = p->i_per_thread;
    if (b != 0 && b != -1 && b != 128 && b != 256)
        return fail(h, NB_ERR_INVALID_ARG, "block must be 0 (auto), -1 (work list), 128 or 256");
    if (i != 0 && i != 1 && i != 2 && i != 4)
        return fail(h, NB_ERR_INVALID_ARG, "i_per_thread must be 1, 2 or 4");
    if (p->bg_kind < NB_BG_NONE || p->bg_kind > NB_BG_PSEUDO_NEWTONIAN || !std::isfinite(p->bg_gm) ||
        !std::isfinite(p->bg_rg) || !std::isfinite(p->bg_center[0]) ||
        !std::isfinite(p->bg_center[1]) || !std::isfinite(p->bg_center[2]))
        return fail(h, NB_ERR_INVALID_ARG, "bad background field parameters");
    if (p->mond != NB_MOND_NONE &&
        (p->mond != NB_MOND_MILGROM1983 || !(p->mond_acc0 > 0.0) || !std::isfinite(p->mond_acc0) ||
         !(p->mond_nu_index > 0.0) || !std::isfinite(p->mond_nu_index)))
        return fail(h, NB_ERR_INVALID_ARG, "MOND needs ACC0 > 0 and MOND_nuIndex > 0");
    if (p->j_split < 0 || p->j_split > 8)
        return fail(h, NB_ERR_INVALID_ARG, "j_split must be 0..8");
    if (p->tile_j != 0 && !nb::tile_size_ok(p->tile_j))
        return fail(h, NB_ERR_INVALID_ARG, "tile_j must be 0 (auto), 128, 256 or 512");
    if (p->block == -1 && p->tile_j != 0 && p->tile_j != kTileJ)
        return fail(h, NB_ERR_INVALID_ARG, "the work-list kernel takes tiles of %d sources", kTileJ);
    if (p->stages != 0 && p->stages != 3 && p->stages != 4 && p->stages != 6)
        return fail(h, NB_ERR_INVALID_ARG, "stages must be 0 (auto), 3, 4 or 6");
    if (p->resort_every < 0 || p->resort_every > (1 << 20))
        return fail(h, NB_ERR_INVALID_ARG, "resort_every must be 0 (auto) or 1..2^20");
    if (p->algorithm != NB_ALG_LEAPFROG && p->algorithm != NB_ALG_EULER)
        return fail(h, NB_ERR_INVALID_ARG, "algorithm must be NB_ALG_LEAPFROG or NB_ALG_EULER");
    return NB_OK;
}

void drop_graph(nb_handle* h) {
    h->perm_valid = false;  // the next step graph replay sorts first
    if (h->step_exec) {
        cudaGraphExecDestroy(h->step_exec);
        h->step_exec = nullptr;
    }
    if (h->out_exec) {
        cudaGraphExecDestroy(h->out_exec);
        h->out_exec = nullptr;
    }
    if (h->step_exec_nosort) {
        cudaGraphExecDestroy(h->step_exec_nosort);
        h->step_exec_nosort = nullptr;
    }
    if (h->out_exec_nosort) {
        cudaGraphExecDestroy(h->out_exec_nosort);
        h->out_exec_nosort = nullptr;
    }
}

int sync_and_check(nb_handle* h) {
    NB_CK(cudaStreamSynchronize(h->stream));
    uint32_t e = 0;
    NB_CK(cudaMemcpy(&e, &h->clk->err, sizeof e, cudaMemcpyDeviceToHost));
    if (e) {
        NB_CK(cudaMemset(&h->clk->err, 0, sizeof e));
        if (e & nb::DEVERR_TIMEOUT)
            return fail(h, NB_ERR_TIMEOUT, "device wait timed out (error bits 0x%x)", e);
        return fail(h, NB_ERR_NUMERIC,
                    "numeric error (bits 0x%x: 1=non-finite acc, 2=dt<MinStep, 4=bad integer step)",
                    e);
    }
    return NB_OK;
}

nb::Targets particle_targets(nb_handle* h, bool want_acc, bool want_pot) {
    nb::Targets t{};
    t.x = h->x;
    t.y = h->y;
    t.z = h->z;
    t.type = h->type;
    t.idx = nullptr;
    t.d_count = nullptr;
    t.n = h->n;
    for (int k = 0; k < 6; ++k) t.soft[k] = h->p.softening[k];
    t.h_const = h->p.softening[0];
    t.ax = want_acc ? h->ax : nullptr;
    t.ay = want_acc ? h->ay : nullptr;
    t.az = want_acc ? h->az : nullptr;
    t.pot = want_pot ? h->pot : nullptr;
    t.self_mass = h->m;
    return t;
}

// Enqueue one force evaluation on stream s (no synchronisation).  With
// active_only the targets are the particles with Ti_endstep == t_int
// (src/directsum/gravity.jl:95-96); the list is built on the device.
// sort = false packs the sources in the order of the last sort (perm must
// hold a valid order; any order gives the same forces to FP32 round-off).
cudaError_t enqueue_force(nb_handle* h, const nb::Targets& tg, cudaStream_t s, bool active_only,
                          bool sort = true) {
    const bool pot = tg.pot != nullptr;
    const bool particles = tg.x == h->x;
    nb::Targets t2 = tg;
    cudaError_t e;
    if (h->p.precision == NB_PREC_FP64) {
        if (active_only) {
            e = nb::launch_active_list(h->ti_end, h->n, nullptr, h->clk, h->active, h->act_scratch, s);
            if (e != cudaSuccess) return e;
            t2.idx = h->active;
            t2.d_count = &h->clk->n_active;
        }
        nb::Sources64 src{h->x, h->y, h->z, h->m, h->n};
        return nb::launch_force_fp64(h->p.law, pot, src, t2, h->p.G, &h->clk->err, s);
    }
    // Morton order of the sources keeps every j-tile compact, so the FP32
    // coordinates relative to its origin stay small.
    if (sort) {
        e = nb::launch_morton_sort(h->x, h->y, h->z, h->n, h->sort_scratch, h->perm, s);
        if (e != cudaSuccess) return e;
    }
    e = nb::launch_pack(h->x, h->y, h->z, h->m, h->n, h->perm, h->tj, h->pack, h->origin, h->ext, s);
    if (e != cudaSuccess) return e;
    // Built-in choice (the size classes of auto_tile / auto_jsplit above):
    // the direct grid with each i-block's tiles split over 4 or 8
    // CTAs, whose compensated partials are joined in order.  The split keeps
    // the grid several waves deep at small N and its last wave short at large
    // N.
    bool use_wl = h->worklist;
    int blk = h->block, ipt = h->ipt;
    int js = h->jsplit;
    if (h->auto_cfg) {
        use_wl = false;
        blk = 128;
        ipt = h->n >= kAutoIpt2From ? 2 : 1;
        js = auto_jsplit(h->n);
    }
    if (particles && use_wl) {
        if (active_only) {
            e = nb::launch_active_list(h->ti_end, h->n, h->perm, h->clk, h->active, h->act_scratch, s);
            if (e != cudaSuccess) return e;
        }
        const bool acc = tg.ax != nullptr;
        const int variant = acc ? (pot ? 1 : 0) : 2;
        const int64_t bt = nb::worklist_block_targets();
        const int64_t nblocks = (h->n + bt - 1) / bt;
        nb::WorkList w{};
        w.sys = h->sysdesc;
        w.nsys = 1;
        w.units = nblocks * (int64_t)h->ntiles;
        int64_t grid = (int64_t)h->wl_occ[h->p.law][variant] * h->nsm;
        w.block_cyclic = h->wl_mode == 1 ? 1 : 0;
        if (!active_only && grid > (w.block_cyclic ? nblocks : w.units))
            grid = w.block_cyclic ? nblocks : w.units;
        w.grid = (int32_t)grid;
        w.active = active_only ? h->active : nullptr;
        w.d_count = active_only ? &h->clk->n_active : nullptr;
        w.perm = active_only ? nullptr : h->perm;
        w.pack = h->pack;
        w.origin = h->origin;
        w.ext = h->ext;
        w.x = h->x;
        w.y = h->y;
        w.z = h->z;
        w.m = h->m;
        w.type = h->type;
        w.ax = tg.ax;
        w.ay = tg.ay;
        w.az = tg.az;
        w.pot = tg.pot;
        w.partial = h->partial;
        w.G = h->p.G;
        w.err = &h->clk->err;
        return nb::launch_force_worklist(h->p.law, w, s);
    }
    if (particles) {
        // Targets are visited in the same Morton order, so the targets of a
        // warp are close together and most j-tiles take the branch-free loop.
        if (active_only) {
            e = nb::launch_active_list(h->ti_end, h->n, h->perm, h->clk, h->active, h->act_scratch, s);
            if (e != cudaSuccess) return e;
            t2.idx = h->active;
            t2.d_count = &h->clk->n_active;
        } else {
            t2.idx = h->perm;
        }
    }
    nb::Sources32 src{h->pack, h->origin, h->ext, h->ntiles, h->tj};
    if (particles && js > 1 && js <= h->jalloc) {
        src.jsplit = js;
        src.partial = h->jpartial;
        src.pstride = h->jstride;
    }
    return nb::launch_force_mixed(h->p.law, pot, src, t2, h->p.G, &h->clk->err, blk, ipt, s,
                                  h->stages);
}

// Force post-processing of the particles that received a force (no-op when
// neither a background field nor MOND is configured).
cudaError_t enqueue_post(nb_handle* h, cudaStream_t s, bool active_only) {
    if (h->p.bg_kind == NB_BG_NONE && h->p.mond == NB_MOND_NONE) return cudaSuccess;
    nb::PostCfg c{};
    c.bg_kind = h->p.bg_kind;
    c.mond = h->p.mond;
    c.gm = h->p.bg_gm;
    c.cx = h->p.bg_center[0];
    c.cy = h->p.bg_center[1];
    c.cz = h->p.bg_center[2];
    c.rg = h->p.bg_rg;
    c.acc0 = h->p.mond_acc0;
    c.nu_index = h->p.mond_nu_index;
    return nb::launch_postprocess(h->ax, h->ay, h->az, h->x, h->y, h->z, h->ti_end, h->n, h->clk,
                                  active_only ? 1 : 0, c, s);
}

// Enqueue step(sim, DirectSum, GPU): drift -> force(active) -> kick.
cudaError_t enqueue_step(nb_handle* h, cudaStream_t s, bool sort) {
    cudaError_t e;
    const bool adaptive = h->p.adaptive != 0;
    if (adaptive) {
        e = nb::launch_min_endstep(h->ti_end, h->n, h->p.time_base, h->clk, s);
        if (e != cudaSuccess) return e;
        e = nb::launch_drift(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->n, h->tc, h->clk, 0, 0, 0.0,
                             s);
        if (e != cudaSuccess) return e;
    } else {
        e = nb::launch_drift(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->n, h->tc, h->clk, 2, 0, 0.0,
                             s);
        if (e != cudaSuccess) return e;
    }
    e = enqueue_force(h, particle_targets(h, true, false), s, adaptive, sort);
    if (e != cudaSuccess) return e;
    e = enqueue_post(h, s, adaptive);
    if (e != cudaSuccess) return e;
    e = nb::launch_kick(h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->type, h->ti_beg, h->ti_end,
                        h->n, h->tc, h->clk, s);
    if (e != cudaSuccess) return e;
    return nb::launch_clock_end_step(h->clk, h->p.adaptive, h->n, s);
}

// The step graph with snapshot stops (find_next_sync_point_and_drift with
// outputs, src/base/Timestep.jl:197-245): [min end step] -> plan -> gated
// drift -> IF(condition){force, post-processing, kick, clock}.  The plan
// kernel sets the condition, so a replay either completes a step or stops the
// time line at an output time inside it; the IF body is skipped on the device
// without a host round trip.
cudaError_t capture_output_graph(nb_handle* h, cudaGraphExec_t* out, bool sort) {
    *out = nullptr;
    cudaStream_t s = h->own_stream;
    const bool adaptive = h->p.adaptive != 0;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle cond = 0;
    e = cudaGraphConditionalHandleCreate(&cond, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return e;
    }
    e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return e;
    }
    cudaGraph_t body = nullptr;
    if (adaptive) e = nb::launch_min_endstep(h->ti_end, h->n, h->p.time_base, h->clk, s);
    if (e == cudaSuccess)
        e = nb::launch_plan_and_drift(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->n, h->tc, h->clk,
                                      cond, s);
    if (e == cudaSuccess) {
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &deps, nullptr, &ndeps);
        if (e == cudaSuccess) {
            cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
            cp.conditional.handle = cond;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t node = nullptr;
            e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp);
            if (e == cudaSuccess) {
                body = cp.conditional.phGraph_out[0];
                e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                        cudaStreamSetCaptureDependencies);
            }
        }
    }
    cudaGraph_t g2 = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &g2);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) {
        // the IF body: the rest of step(sim, DirectSum, GPU)
        e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            e = enqueue_force(h, particle_targets(h, true, false), s, adaptive, sort);
            if (e == cudaSuccess) e = enqueue_post(h, s, adaptive);
            if (e == cudaSuccess)
                e = nb::launch_kick(h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->type, h->ti_beg,
                                    h->ti_end, h->n, h->tc, h->clk, s);
            if (e == cudaSuccess) e = nb::launch_clock_end_step(h->clk, h->p.adaptive, h->n, s);
            cudaGraph_t b2 = nullptr;
            e2 = cudaStreamEndCapture(s, &b2);
            if (e == cudaSuccess) e = e2;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) *out = nullptr;
    return e;
}

int ensure_capacity(nb_handle* h, int64_t n) {
    const int js_need = h->auto_cfg ? kAutoJsplitMax : h->jsplit;
    if (n <= h->cap && h->arena && js_need <= h->jalloc) return NB_OK;
    drop_graph(h);
    if (h->arena) {
        cudaFree(h->arena);
        h->arena = nullptr;
        h->cap = 0;
    }
    // room for every tile size: tile records for tiles of 128, padded sources
    // for tiles of 512
    const int64_t ntiles = (n + 127) / 128;
    const int64_t npad = (n + 511) / 512 * 512;
    const int64_t dblocks = nb::diag_scratch_doubles(n);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t d = sizeof(double) * (size_t)n;
    size_t o_x = take(d), o_y = take(d), o_z = take(d), o_vx = take(d), o_vy = take(d),
           o_vz = take(d), o_ax = take(d), o_ay = take(d), o_az = take(d), o_pot = take(d),
           o_m = take(d);
    size_t o_type = take(sizeof(int32_t) * (size_t)n);
    size_t o_tb = take(sizeof(int64_t) * (size_t)n), o_te = take(sizeof(int64_t) * (size_t)n);
    size_t o_act = take(sizeof(int32_t) * (size_t)n);
    size_t o_perm = take(sizeof(int32_t) * (size_t)n);
    // j-split partials: jsplit x 8 floats per target slot (slots padded to 1024)
    const int64_t jstride = (n + 1023) / 1024 * 1024;
    size_t o_jp = take(js_need > 1 ? sizeof(float) * 8 * (size_t)js_need * jstride : 0);
    size_t o_acts = take(sizeof(uint32_t) * (size_t)nb::active_scratch_words(n));
    size_t o_sort = take(nb::sort_scratch_bytes(n));
    size_t o_pack = take(sizeof(float4) * (size_t)npad);
    size_t o_orig = take(sizeof(nb::TileOrigin) * (size_t)ntiles);
    size_t o_ext = take(sizeof(float4) * (size_t)ntiles);
    size_t o_ds = take(sizeof(double) * (size_t)dblocks);
    size_t o_do = take(sizeof(double) * 8);
    void* a = nullptr;
    NB_CK(cudaMalloc(&a, off));
    char* b = static_cast<char*>(a);
    h->arena = a;
    h->cap = n;
    h->x = (double*)(b + o_x);
    h->y = (double*)(b + o_y);
    h->z = (double*)(b + o_z);
    h->vx = (double*)(b + o_vx);
    h->vy = (double*)(b + o_vy);
    h->vz = (double*)(b + o_vz);
    h->ax = (double*)(b + o_ax);
    h->ay = (double*)(b + o_ay);
    h->az = (double*)(b + o_az);
    h->pot = (double*)(b + o_pot);
    h->m = (double*)(b + o_m);
    h->type = (int32_t*)(b + o_type);
    h->ti_beg = (int64_t*)(b + o_tb);
    h->ti_end = (int64_t*)(b + o_te);
    h->active = (int32_t*)(b + o_act);
    h->perm = (int32_t*)(b + o_perm);
    h->jpartial = js_need > 1 ? (float*)(b + o_jp) : nullptr;
    h->jalloc = js_need;
    h->jstride = jstride;
    h->act_scratch = (uint32_t*)(b + o_acts);
    h->sort_scratch = (void*)(b + o_sort);
    h->pack = (float4*)(b + o_pack);
    h->origin = (nb::TileOrigin*)(b + o_orig);
    h->ext = (float4*)(b + o_ext);
    h->diag_scratch = (double*)(b + o_ds);
    h->diag_blocks = dblocks / 8;
    h->diag_out = (double*)(b + o_do);
    h->ntiles = (int32_t)((n + h->tj - 1) / h->tj);
    return NB_OK;
}

// The single-system descriptor of the work-list force (particles, tiles,
// softening table).
int upload_sysdesc(nb_handle* h) {
    nb::SysDesc d{};
    const int64_t bt = nb::worklist_block_targets();
    d.off = 0;
    d.ubase = 0;
    d.n = (int32_t)h->n;
    d.tile_off = 0;
    d.ntiles = h->ntiles;
    d.nblocks = (int32_t)((h->n + bt - 1) / bt);
    for (int k = 0; k < 6; ++k) d.soft[k] = h->p.softening[k];
    NB_CK(cudaMemcpy(h->sysdesc, &d, sizeof d, cudaMemcpyHostToDevice));
    return NB_OK;
}

// Launch-shape choice of nb_params (block, i_per_thread, j_split).
void apply_tuning(nb_handle* h, const nb_params& p) {
    h->block = p.block > 0 ? p.block : 128;
    h->ipt = p.i_per_thread ? p.i_per_thread : 2;
    h->jsplit = p.j_split > 1 ? p.j_split : 1;
    h->tj = p.tile_j ? p.tile_j : kTileJ;
    h->stages = p.stages ? p.stages : 4;
    h->resort = p.resort_every ? p.resort_every : 16;
    h->worklist = p.block == -1;
    h->auto_cfg = p.block == 0 && p.i_per_thread == 0;
}

// Checkpoint image: this header, then x, y, z, vx, vy, vz, ax, ay, az, pot, m
// (FP64, n each), type (int32, n, padded to 8 bytes), Ti_begstep, Ti_endstep
// (int64, n each).  The parameters carry the time-integration algorithm and
// the clock the snapshot schedule, so a restored run keeps both.
struct CkptHeader {
    char magic[8];
    int64_t version;
    int64_t n;
    int64_t bytes;
    int64_t params_size;
    int64_t clock_size;
    nb_params p;
    double between;  // BetweenSnapshots (0: no output stops)
    // Source order of the step graphs: the step count that sets the phase of
    // their re-sorts, or -1 when the image holds no valid order (the
    // permutation block after the bins then carries no meaning).
    int64_t order_steps;
    Clock clk;
};
constexpr char kCkptMagic[8] = {'N', 'B', 'G', 'B', '3', '0', '0', 'C'};
constexpr int64_t kCkptVersion = 3;

// Header, 11 FP64 arrays, types, two int64 bin arrays, the Morton permutation.
int64_t ckpt_bytes(int64_t n) {
    return (int64_t)sizeof(CkptHeader) + 11 * 8 * n + 2 * (int64_t)align_up(4 * (size_t)n, 8) +
           16 * n;
}

int require_particles(nb_handle* h) {
    if (h->n <= 0) return fail(h, NB_ERR_STATE, "no particles uploaded");
    return NB_OK;
}

int use_device(nb_handle* h) {
    NB_CK(cudaSetDevice(h->dev));
    return NB_OK;
}

}  // namespace

extern "C" {

const char* nb_version(void) { return "nbody_gb300 0.1.0 (sm_103a)"; }

void nb_default_params(nb_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->G = 1.0;
    for (int k = 0; k < 6; ++k) p->softening[k] = 1.0e-4;
    p->law = NB_LAW_SPLINE_G2;
    p->precision = NB_PREC_MIXED;
    p->adaptive = 1;
    p->criterion = NB_CRIT_REF;
    p->dt = 0.0;
    p->eta = 0.025;
    p->min_step = 1.0e-8;
    p->max_step = INFINITY;
    p->time_base = (int64_t)1 << 30;
    p->time_begin = 0.0;
    p->time_end = 0.1;
    p->device = 0;
    p->mond_nu_index = 2.0;
}

int nb_create(const nb_params* p, nb_handle** out) {
    g_create_err.clear();
    if (!p || !out) {
        g_create_err = "nb_create: null parameter or output pointer";
        return NB_ERR_INVALID_ARG;
    }
    *out = nullptr;
    nb_handle* h = new (std::nothrow) nb_handle();
    if (!h) return NB_ERR_OOM;
    int rc = check_params(h, p);
    if (rc) {
        g_create_err = h->err;
        delete h;
        return rc;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || p->device < 0 || p->device >= ndev) {
        g_create_err = "nb_create: device " + std::to_string(p->device) + " not available (" +
                       std::to_string(ndev) + " CUDA devices)";
        delete h;
        return NB_ERR_CUDA;
    }
    h->p = *p;
    h->tc = make_timecfg(*p, 0.0);
    h->dev = p->device;
    if (cudaSetDevice(h->dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&h->clk, sizeof(Clock)) != cudaSuccess) {
        if (h->own_stream) cudaStreamDestroy(h->own_stream);
        delete h;
        return NB_ERR_CUDA;
    }
    h->stream = h->own_stream;
    Clock c = initial_clock(*p, h->tc);
    cudaMemcpy(h->clk, &c, sizeof c, cudaMemcpyHostToDevice);
    // Work-list force: persistent grid = CTAs per SM x SMs for each variant;
    // the partial-sum scratch is sized for the largest grid.
    // block == -1: persistent work-list kernel; block/ipt given: direct grid with
    // that shape; 0/0: chosen per particle count in enqueue_force.
    apply_tuning(h, *p);
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->dev);
    int occ_max = 0;
    for (int law = 0; law < 2; ++law)
        for (int v = 0; v < 3; ++v) {
            h->wl_occ[law][v] = nb::worklist_ctas_per_sm(law, v != 2, v != 0);
            if (h->wl_occ[law][v] < 1) h->wl_occ[law][v] = 1;
            if (h->wl_occ[law][v] > occ_max) occ_max = h->wl_occ[law][v];
        }
    if (const char* ev = std::getenv("NBODY_GB300_WL_MODE")) h->wl_mode = std::atoi(ev) == 1 ? 1 : 0;
    // Tuning override: CTAs per SM of the persistent work-list grid.
    if (const char* ev = std::getenv("NBODY_GB300_WL_CTAS_PER_SM")) {
        const int o = std::atoi(ev);
        if (o >= 1 && o <= 32) {
            for (int law = 0; law < 2; ++law)
                for (int v = 0; v < 3; ++v) h->wl_occ[law][v] = o;
            if (o > occ_max) occ_max = o;
        }
    }
    h->partial_bytes = nb::worklist_partial_bytes((int64_t)occ_max * h->nsm);
    if (cudaMalloc(&h->partial, h->partial_bytes) != cudaSuccess ||
        cudaMalloc(&h->sysdesc, sizeof(nb::SysDesc)) != cudaSuccess) {
        if (h->partial) cudaFree(h->partial);
        cudaFree(h->clk);
        cudaStreamDestroy(h->own_stream);
        delete h;
        return NB_ERR_OOM;
    }
    *out = h;
    return NB_OK;
}

int nb_destroy(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    cudaSetDevice(h->dev);
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graph(h);
    if (h->arena) cudaFree(h->arena);
    if (h->probe) cudaFree(h->probe);
    if (h->clk) cudaFree(h->clk);
    if (h->partial) cudaFree(h->partial);
    if (h->sysdesc) cudaFree(h->sysdesc);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return NB_OK;
}

int nb_set_stream(nb_handle* h, void* stream) {
    if (!h) return NB_ERR_INVALID_ARG;
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    return NB_OK;
}

int nb_get_stream(nb_handle* h, void** stream) {
    if (!h || !stream) return NB_ERR_INVALID_ARG;
    *stream = h->stream;
    return NB_OK;
}

int nb_upload(nb_handle* h, int64_t n, const double* x, const double* y, const double* z,
              const double* vx, const double* vy, const double* vz, const double* m,
              const int32_t* type) {
    if (!h) return NB_ERR_INVALID_ARG;
    if (n < 0 || n > (int64_t)0x7fffffff) return fail(h, NB_ERR_INVALID_ARG, "bad particle count %lld", (long long)n);
    if (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m))
        return fail(h, NB_ERR_INVALID_ARG, "null particle array");
    if (type)
        for (int64_t i = 0; i < n; ++i)
            if (type[i] < 1 || type[i] > 6)
                return fail(h, NB_ERR_INVALID_ARG, "type[%lld]=%d outside 1..6", (long long)i, type[i]);
    int rc = use_device(h);
    if (rc) return rc;
    const int64_t n_old = h->n;
    const int tj_old = h->tj;
    if (n > 0) {
        if (h->auto_cfg && h->p.tile_j == 0) h->tj = auto_tile(n);
        rc = ensure_capacity(h, n);  // drops the step graphs when it re-lays the arena out
        if (rc) return rc;
    }
    h->n = n;
    // tiles of this upload (the arena may hold more from a larger earlier one)
    h->ntiles = (int32_t)((n + h->tj - 1) / h->tj);
    // The step graphs hold the arena's pointers and the particle and tile
    // counts, not the data: they stay valid for an upload of the same size.
    // The source order of the old particles does not carry over.
    if (n != n_old || h->tj != tj_old)
        drop_graph(h);
    else
        h->perm_valid = false;
    if (n == 0) return NB_OK;
    const size_t d = sizeof(double) * (size_t)n;
    cudaStream_t s = h->stream;
    NB_CK(cudaMemcpyAsync(h->x, x, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->y, y, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->z, z, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->vx, vx, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->vy, vy, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->vz, vz, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(h->m, m, d, cudaMemcpyHostToDevice, s));
    if (type) {
        NB_CK(cudaMemcpyAsync(h->type, type, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
    } else {
        // Default particle type 1.
        std::vector<int32_t> ones((size_t)n, 1);
        NB_CK(cudaMemcpy(h->type, ones.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice));
    }
    NB_CK(cudaMemsetAsync(h->ax, 0, d, s));
    NB_CK(cudaMemsetAsync(h->ay, 0, d, s));
    NB_CK(cudaMemsetAsync(h->az, 0, d, s));
    NB_CK(cudaMemsetAsync(h->pot, 0, d, s));
    NB_CK(cudaMemsetAsync(h->ti_beg, 0, sizeof(int64_t) * (size_t)n, s));
    NB_CK(cudaMemsetAsync(h->ti_end, 0, sizeof(int64_t) * (size_t)n, s));
    Clock c = initial_clock(h->p, h->tc);
    NB_CK(cudaMemcpyAsync(h->clk, &c, sizeof c, cudaMemcpyHostToDevice, s));
    NB_CK(cudaStreamSynchronize(s));
    return upload_sysdesc(h);
}

int nb_download(nb_handle* h, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                double* ax, double* ay, double* az, double* pot, int64_t* ti_begstep,
                int64_t* ti_endstep) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    if (h->n == 0) return NB_OK;
    const size_t d = sizeof(double) * (size_t)h->n;
    cudaStream_t s = h->stream;
    struct {
        void* dst;
        const void* src;
        size_t bytes;
    } cp[] = {{x, h->x, d},   {y, h->y, d},   {z, h->z, d},   {vx, h->vx, d},
              {vy, h->vy, d}, {vz, h->vz, d}, {ax, h->ax, d}, {ay, h->ay, d},
              {az, h->az, d}, {pot, h->pot, d},
              {ti_begstep, h->ti_beg, sizeof(int64_t) * (size_t)h->n},
              {ti_endstep, h->ti_end, sizeof(int64_t) * (size_t)h->n}};
    for (auto& c : cp)
        if (c.dst) NB_CK(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, s));
    NB_CK(cudaStreamSynchronize(s));
    return NB_OK;
}

int nb_upload_acc(nb_handle* h, const double* ax, const double* ay, const double* az) {
    if (!h || !ax || !ay || !az) return fail(h, NB_ERR_INVALID_ARG, "null acceleration array");
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    const size_t d = sizeof(double) * (size_t)h->n;
    NB_CK(cudaMemcpyAsync(h->ax, ax, d, cudaMemcpyHostToDevice, h->stream));
    NB_CK(cudaMemcpyAsync(h->ay, ay, d, cudaMemcpyHostToDevice, h->stream));
    NB_CK(cudaMemcpyAsync(h->az, az, d, cudaMemcpyHostToDevice, h->stream));
    NB_CK(cudaStreamSynchronize(h->stream));
    return NB_OK;
}

int nb_upload_bins(nb_handle* h, const int64_t* ti_begstep, const int64_t* ti_endstep) {
    if (!h || !ti_begstep || !ti_endstep) return fail(h, NB_ERR_INVALID_ARG, "null bin array");
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    const size_t d = sizeof(int64_t) * (size_t)h->n;
    NB_CK(cudaMemcpyAsync(h->ti_beg, ti_begstep, d, cudaMemcpyHostToDevice, h->stream));
    NB_CK(cudaMemcpyAsync(h->ti_end, ti_endstep, d, cudaMemcpyHostToDevice, h->stream));
    NB_CK(cudaStreamSynchronize(h->stream));
    return NB_OK;
}

int nb_set_softening(nb_handle* h, const double soft[6]) {
    if (!h || !soft) return NB_ERR_INVALID_ARG;
    for (int k = 0; k < 6; ++k)
        if (!(soft[k] > 0.0) || !std::isfinite(soft[k]))
            return fail(h, NB_ERR_INVALID_ARG, "softening[%d] must be finite and > 0", k);
    for (int k = 0; k < 6; ++k) h->p.softening[k] = soft[k];
    h->tc = make_timecfg(h->p, h->between);
    drop_graph(h);
    if (h->n > 0) {
        int rc = use_device(h);
        if (rc) return rc;
        return upload_sysdesc(h);
    }
    return NB_OK;
}

int nb_compute_force(nb_handle* h, int flags) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    const bool adaptive = h->p.adaptive != 0;
    NB_CK(enqueue_force(h, particle_targets(h, true, (flags & NB_FORCE_POT) != 0), h->stream,
                        adaptive));
    NB_CK(enqueue_post(h, h->stream, adaptive));
    return sync_and_check(h);
}

int nb_compute_potential(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    NB_CK(enqueue_force(h, particle_targets(h, false, true), h->stream, false));
    return sync_and_check(h);
}

int nb_remove_self_potential(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    NB_CK(nb::launch_remove_self_potential(h->pot, h->m, h->type, h->n, h->tc, h->p.G, h->stream));
    return sync_and_check(h);
}

int nb_force_at_points(nb_handle* h, int64_t n, const double* px, const double* py,
                       const double* pz, double soft, double* ax, double* ay, double* az,
                       double* pot) {
    if (!h) return NB_ERR_INVALID_ARG;
    if (n < 0 || n > (int64_t)0x7fffffff || (n > 0 && (!px || !py || !pz)))
        return fail(h, NB_ERR_INVALID_ARG, "bad probe arrays");
    if (!(soft > 0.0) || !std::isfinite(soft))
        return fail(h, NB_ERR_INVALID_ARG, "softening must be finite and > 0");
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    if (n == 0) return NB_OK;
    const size_t d = sizeof(double) * (size_t)n;
    const size_t need = 7 * align_up(d, 256);
    if (need > h->probe_bytes) {
        if (h->probe) cudaFree(h->probe);
        h->probe = nullptr;
        h->probe_bytes = 0;
        NB_CK(cudaMalloc(&h->probe, need));
        h->probe_bytes = need;
    }
    char* b = static_cast<char*>(h->probe);
    const size_t st = align_up(d, 256);
    double* dx = (double*)(b + 0 * st);
    double* dy = (double*)(b + 1 * st);
    double* dz = (double*)(b + 2 * st);
    double* oax = (double*)(b + 3 * st);
    double* oay = (double*)(b + 4 * st);
    double* oaz = (double*)(b + 5 * st);
    double* opot = (double*)(b + 6 * st);
    cudaStream_t s = h->stream;
    NB_CK(cudaMemcpyAsync(dx, px, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(dy, py, d, cudaMemcpyHostToDevice, s));
    NB_CK(cudaMemcpyAsync(dz, pz, d, cudaMemcpyHostToDevice, s));
    nb::Targets t{};
    t.x = dx;
    t.y = dy;
    t.z = dz;
    t.type = nullptr;
    t.idx = nullptr;
    t.d_count = nullptr;
    t.n = n;
    for (int k = 0; k < 6; ++k) t.soft[k] = soft;
    t.h_const = soft;
    const bool want_acc = ax || ay || az;
    t.ax = want_acc ? oax : nullptr;
    t.ay = want_acc ? oay : nullptr;
    t.az = want_acc ? oaz : nullptr;
    t.pot = pot ? opot : nullptr;
    t.self_mass = nullptr;
    NB_CK(enqueue_force(h, t, s, false));
    if (ax) NB_CK(cudaMemcpyAsync(ax, oax, d, cudaMemcpyDeviceToHost, s));
    if (ay) NB_CK(cudaMemcpyAsync(ay, oay, d, cudaMemcpyDeviceToHost, s));
    if (az) NB_CK(cudaMemcpyAsync(az, oaz, d, cudaMemcpyDeviceToHost, s));
    if (pot) NB_CK(cudaMemcpyAsync(pot, opot, d, cudaMemcpyDeviceToHost, s));
    return sync_and_check(h);
}

int nb_init_timesteps(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    NB_CK(nb::launch_init_timesteps(h->ax, h->ay, h->az, h->type, h->ti_beg, h->ti_end, h->n, h->tc,
                                    h->clk, h->stream));
    return sync_and_check(h);
}

int nb_half_kick(nb_handle* h, int forward) {
    if (!h || (forward != 1 && forward != -1)) return fail(h, NB_ERR_INVALID_ARG, "forward must be +1 or -1");
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    NB_CK(nb::launch_half_kick(h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->ti_beg, h->ti_end, h->n,
                               h->tc, forward, h->stream));
    return sync_and_check(h);
}

int nb_kick(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    NB_CK(nb::launch_kick(h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->type, h->ti_beg, h->ti_end,
                          h->n, h->tc, h->clk, h->stream));
    return sync_and_check(h);
}

int nb_find_min_endstep(nb_handle* h, int64_t* min_endstep) {
    if (!h || !min_endstep) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    NB_CK(nb::launch_min_endstep(h->ti_end, h->n, h->p.time_base, h->clk, h->stream));
    NB_CK(cudaMemcpyAsync(min_endstep, &h->clk->min_endstep, sizeof(int64_t),
                          cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

int nb_check_sync_point(nb_handle* h, int32_t* sync) {
    if (!h || !sync) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    // the diagnostics' 8-double output slot serves as the counter
    unsigned long long* count = reinterpret_cast<unsigned long long*>(h->diag_out);
    NB_CK(nb::launch_sync_count(h->ti_end, h->n, h->clk, count, h->stream));
    unsigned long long c = 0;
    NB_CK(cudaMemcpyAsync(&c, count, sizeof c, cudaMemcpyDeviceToHost, h->stream));
    rc = sync_and_check(h);
    if (rc) return rc;
    *sync = c == (unsigned long long)h->n ? 1 : 0;
    return NB_OK;
}

int nb_drift_to_int(nb_handle* h, int64_t t_int) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    NB_CK(nb::launch_drift(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->n, h->tc, h->clk, 1, t_int, 0.0,
                           h->stream));
    return sync_and_check(h);
}

int nb_drift_to_float(nb_handle* h, double t_float) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    NB_CK(nb::launch_drift(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->n, h->tc, h->clk, 3, 0,
                           t_float, h->stream));
    return sync_and_check(h);
}

// Replays of the output-aware step graph until `nsteps` steps are complete;
// with stop_at_output the call returns at the first output time reached
// (*at_output = 1), otherwise it continues through output times (the drift
// is still split there).  *done = complete steps.
// The step graphs that skip the sort read perm: give it an order of the
// current particles first when none is known (after nb_create, nb_upload,
// nb_checkpoint_load or a parameter change).
static int ensure_order(nb_handle* h) {
    if (h->perm_valid || h->p.precision == NB_PREC_FP64) return NB_OK;
    NB_CK(nb::launch_morton_sort(h->x, h->y, h->z, h->n, h->sort_scratch, h->perm, h->stream));
    h->perm_valid = true;
    return NB_OK;
}

static int step_with_outputs(nb_handle* h, int64_t nsteps, bool stop_at_output, int64_t* done,
                      int32_t* at_output) {
    *done = 0;
    *at_output = 0;
    if (!h->out_exec || !h->out_exec_nosort) {
        NB_CK(cudaStreamSynchronize(h->stream));
        cudaError_t e = capture_output_graph(h, &h->out_exec, true);
        if (e == cudaSuccess) e = capture_output_graph(h, &h->out_exec_nosort, false);
        if (e != cudaSuccess)
            return fail(h, NB_ERR_CUDA, "output step graph capture failed: %s", cudaGetErrorString(e));
    }
    // Replays after an output stop are no-ops on the device, so the host reads
    // the clock between chunks instead of after every step.
    struct {
        int64_t steps;
        int32_t at_output;
    } st;
    Clock c{};
    NB_CK(cudaStreamSynchronize(h->stream));
    NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
    const int64_t steps0 = c.steps;
    st.steps = c.steps;
    st.at_output = c.at_output;
    while (st.steps - steps0 < nsteps) {
        if (st.at_output) {
            // the host has seen this output: resume the step
            NB_CK(cudaMemsetAsync(&h->clk->at_output, 0, sizeof(int32_t), h->stream));
        }
        int64_t chunk = nsteps - (st.steps - steps0);
        if (chunk > 32) chunk = 32;
        int rc0 = ensure_order(h);
        if (rc0) return rc0;
        for (int64_t k = 0; k < chunk; ++k) {
            // Replay k performs step st.steps + k until one stops at an output
            // time; the rest of the chunk is then skipped on the device and
            // the next chunk starts from the device's count again.
            const bool sort = (st.steps + k) % h->resort == 0;
            NB_CK(cudaGraphLaunch(sort ? h->out_exec : h->out_exec_nosort, h->stream));
        }
        int rc = sync_and_check(h);
        if (rc) return rc;
        NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
        st.steps = c.steps;
        st.at_output = c.at_output;
        if (st.at_output && stop_at_output) break;
    }
    *done = st.steps - steps0;
    *at_output = st.at_output;
    h->host_steps = st.steps;
    return NB_OK;
}

int nb_step(nb_handle* h, int64_t nsteps) {
    if (!h || nsteps < 0) return fail(h, NB_ERR_INVALID_ARG, "nsteps must be >= 0");
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    if (nsteps == 0) return NB_OK;
    if (h->tc.outputs_on) {
        int64_t done = 0;
        int32_t at = 0;
        return step_with_outputs(h, nsteps, false, &done, &at);
    }
    if (!h->step_exec || !h->step_exec_nosort) {
        // Capture one step (with and without the sort) on the handle's own
        // (non-default) stream; the graphs are then launched on whatever
        // stream the handle currently uses.
        NB_CK(cudaStreamSynchronize(h->stream));
        for (int variant = 0; variant < 2; ++variant) {
            cudaGraph_t g = nullptr;
            NB_CK(cudaStreamBeginCapture(h->own_stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue_step(h, h->own_stream, variant == 0);
            cudaError_t e2 = cudaStreamEndCapture(h->own_stream, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return fail(h, NB_ERR_CUDA, "step capture failed: %s",
                            cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            cudaGraphExec_t* dst = variant == 0 ? &h->step_exec : &h->step_exec_nosort;
            e = cudaGraphInstantiate(dst, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                *dst = nullptr;
                return fail(h, NB_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
            }
        }
    }
    int rc0 = ensure_order(h);
    if (rc0) return rc0;
    for (int64_t k = 0; k < nsteps; ++k) {
        const bool sort = h->host_steps % h->resort == 0;
        NB_CK(cudaGraphLaunch(sort ? h->step_exec : h->step_exec_nosort, h->stream));
        h->host_steps += 1;
    }
    return sync_and_check(h);
}

int nb_step_until_output(nb_handle* h, int64_t max_steps, int64_t* steps_done,
                         int32_t* at_output) {
    if (!h || max_steps < 0 || !steps_done || !at_output)
        return fail(h, NB_ERR_INVALID_ARG, "max_steps must be >= 0 and the outputs non-NULL");
    *steps_done = 0;
    *at_output = 0;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    if (max_steps == 0) return NB_OK;
    if (!h->tc.outputs_on) {
        rc = nb_step(h, max_steps);
        if (rc) return rc;
        *steps_done = max_steps;
        return NB_OK;
    }
    return step_with_outputs(h, max_steps, true, steps_done, at_output);
}

int nb_set_snapshot_interval(nb_handle* h, double between) {
    if (!h) return NB_ERR_INVALID_ARG;
    if (!(between >= 0.0) || !std::isfinite(between))
        return fail(h, NB_ERR_INVALID_ARG, "BetweenSnapshots must be finite and >= 0");
    const TimeCfg tc = make_timecfg(h->p, between);
    if (tc.outputs_on && h->p.adaptive && tc.between_int <= 0)
        return fail(h, NB_ERR_INVALID_ARG,
                    "BetweenSnapshots %.17g is below TimeInterval %.17g: BetweenSnapshotsInt would be 0",
                    between, tc.time_interval);
    int rc = use_device(h);
    if (rc) return rc;
    Clock c{};
    NB_CK(cudaStreamSynchronize(h->stream));
    NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
    if (c.mid_step)
        return fail(h, NB_ERR_STATE, "the time line is stopped at an output time inside a step");
    drop_graph(h);
    h->between = between;
    h->tc = tc;
    const Clock c0 = initial_clock(h->p, tc);
    c.next_out_int = c0.next_out_int;
    c.next_out_float = c0.next_out_float;
    NB_CK(cudaMemcpy(h->clk, &c, sizeof c, cudaMemcpyHostToDevice));
    return NB_OK;
}

int nb_get_output_time(nb_handle* h, int64_t* next_int, double* next_float, int32_t* at_output,
                       int64_t* outputs) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    Clock c{};
    NB_CK(cudaStreamSynchronize(h->stream));
    NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
    if (next_int) *next_int = c.next_out_int;
    if (next_float) *next_float = c.next_out_float;
    if (at_output) *at_output = c.at_output;
    if (outputs) *outputs = c.outputs;
    return NB_OK;
}

int nb_run_begin(nb_handle* h) {
    int rc = nb_compute_force(h, 0);
    if (rc) return rc;
    rc = nb_init_timesteps(h);
    if (rc) return rc;
    if (h->p.algorithm == NB_ALG_EULER) return NB_OK;
    return nb_half_kick(h, +1);
}

int nb_run_end(nb_handle* h) {
    if (!h) return NB_ERR_INVALID_ARG;
    if (h->p.algorithm == NB_ALG_EULER) return NB_OK;
    return nb_half_kick(h, -1);
}

int nb_get_time(nb_handle* h, int64_t* t_int, double* t_float) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    Clock c{};
    NB_CK(cudaStreamSynchronize(h->stream));
    NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
    if (t_int) *t_int = c.t_int;
    if (t_float) *t_float = c.t_float;
    return NB_OK;
}

int nb_get_counters(nb_handle* h, int64_t* steps, double* interactions) {
    if (!h) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    Clock c{};
    NB_CK(cudaStreamSynchronize(h->stream));
    NB_CK(cudaMemcpy(&c, h->clk, sizeof c, cudaMemcpyDeviceToHost));
    if (steps) *steps = c.steps;
    if (interactions) *interactions = c.interactions;
    return NB_OK;
}

int nb_diagnostics(nb_handle* h, int with_potential, nb_diag* out) {
    if (!h || !out) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    rc = require_particles(h);
    if (rc) return rc;
    if (with_potential) NB_CK(enqueue_force(h, particle_targets(h, false, true), h->stream, false));
    NB_CK(nb::launch_diag(h->x, h->y, h->z, h->vx, h->vy, h->vz, h->m, h->pot, h->n,
                          h->diag_scratch, h->diag_blocks, h->diag_out, h->stream));
    double o[8];
    NB_CK(cudaMemcpyAsync(o, h->diag_out, sizeof o, cudaMemcpyDeviceToHost, h->stream));
    rc = sync_and_check(h);
    if (rc) return rc;
    out->kinetic = o[0];
    out->potential = o[1];
    for (int k = 0; k < 3; ++k) {
        out->momentum[k] = o[2 + k];
        out->angular_momentum[k] = o[5 + k];
    }
    return NB_OK;
}

int nb_active_count(nb_handle* h, int64_t* count) {
    if (!h || !count) return NB_ERR_INVALID_ARG;
    int rc = use_device(h);
    if (rc) return rc;
    if (h->n == 0) {
        *count = 0;
        return NB_OK;
    }
    NB_CK(nb::launch_active_list(h->ti_end, h->n, nullptr, h->clk, h->active, h->act_scratch, h->stream));
    int32_t c = 0;
    NB_CK(cudaMemcpyAsync(&c, &h->clk->n_active, sizeof c, cudaMemcpyDeviceToHost, h->stream));
    NB_CK(cudaStreamSynchronize(h->stream));
    *count = c;
    return NB_OK;
}

int nb_checkpoint_size(nb_handle* h, int64_t* bytes) {
    if (!h || !bytes) return NB_ERR_INVALID_ARG;
    *bytes = ckpt_bytes(h->n);
    return NB_OK;
}

int nb_checkpoint_save(nb_handle* h, void* buf, int64_t bytes) {
    if (!h || !buf) return fail(h, NB_ERR_INVALID_ARG, "null checkpoint buffer");
    const int64_t n = h->n;
    if (bytes < ckpt_bytes(n))
        return fail(h, NB_ERR_INVALID_ARG, "checkpoint buffer of %lld bytes, need %lld",
                    (long long)bytes, (long long)ckpt_bytes(n));
    int rc = use_device(h);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    NB_CK(cudaStreamSynchronize(s));
    CkptHeader hd{};
    std::memcpy(hd.magic, kCkptMagic, sizeof hd.magic);
    hd.version = kCkptVersion;
    hd.n = n;
    hd.bytes = ckpt_bytes(n);
    hd.params_size = (int64_t)sizeof(nb_params);
    hd.clock_size = (int64_t)sizeof(Clock);
    hd.p = h->p;
    hd.between = h->between;
    hd.order_steps = h->perm_valid ? h->host_steps : -1;
    NB_CK(cudaMemcpy(&hd.clk, h->clk, sizeof(Clock), cudaMemcpyDeviceToHost));
    char* b = static_cast<char*>(buf);
    std::memcpy(b, &hd, sizeof hd);
    size_t off = sizeof hd;
    if (n > 0) {
        const double* arrs[11] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->pot, h->m};
        const size_t d = sizeof(double) * (size_t)n;
        for (const double* a : arrs) {
            NB_CK(cudaMemcpyAsync(b + off, a, d, cudaMemcpyDeviceToHost, s));
            off += d;
        }
        NB_CK(cudaMemcpyAsync(b + off, h->type, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        off += align_up(4 * (size_t)n, 8);
        NB_CK(cudaMemcpyAsync(b + off, h->ti_beg, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        off += sizeof(int64_t) * (size_t)n;
        NB_CK(cudaMemcpyAsync(b + off, h->ti_end, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        off += sizeof(int64_t) * (size_t)n;
        if (h->perm_valid)
            NB_CK(cudaMemcpyAsync(b + off, h->perm, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        else
            std::memset(b + off, 0, align_up(4 * (size_t)n, 8));
        NB_CK(cudaStreamSynchronize(s));
    }
    return NB_OK;
}

int nb_checkpoint_load(nb_handle* h, const void* buf, int64_t bytes) {
    if (!h || !buf) return fail(h, NB_ERR_INVALID_ARG, "null checkpoint buffer");
    if (bytes < (int64_t)sizeof(CkptHeader))
        return fail(h, NB_ERR_INVALID_ARG, "checkpoint image too short");
    CkptHeader hd;
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, kCkptMagic, sizeof hd.magic) != 0 || hd.version != kCkptVersion ||
        hd.params_size != (int64_t)sizeof(nb_params) || hd.clock_size != (int64_t)sizeof(Clock))
        return fail(h, NB_ERR_INVALID_ARG, "not a checkpoint image of this library version");
    const int64_t n = hd.n;
    if (n < 0 || n > (int64_t)0x7fffffff || hd.bytes != ckpt_bytes(n) || bytes < hd.bytes)
        return fail(h, NB_ERR_INVALID_ARG, "checkpoint image size does not match its particle count");
    nb_params p = hd.p;
    p.device = h->dev;  // the image moves to this handle's device
    int rc = check_params(h, &p);
    if (rc) return rc;
    if (!(hd.between >= 0.0) || !std::isfinite(hd.between))
        return fail(h, NB_ERR_INVALID_ARG, "checkpoint image has a bad snapshot interval");
    const char* b = static_cast<const char*>(buf);
    const int32_t* type = reinterpret_cast<const int32_t*>(b + sizeof hd + 11 * 8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i)
        if (type[i] < 1 || type[i] > 6)
            return fail(h, NB_ERR_INVALID_ARG, "checkpoint type[%lld]=%d outside 1..6", (long long)i, type[i]);
    // A saved source order is used only if it is a permutation of 0..n-1
    // (the pack gathers through it); otherwise the next step re-sorts.
    bool order_ok = hd.order_steps >= 0 && n > 0;
    if (order_ok) {
        const int32_t* pm = reinterpret_cast<const int32_t*>(
            b + sizeof hd + 11 * 8 * (size_t)n + align_up(4 * (size_t)n, 8) + 16 * (size_t)n);
        std::vector<unsigned char> seen((size_t)n, 0);
        for (int64_t i = 0; i < n && order_ok; ++i) {
            const int32_t v = pm[i];
            if (v < 0 || v >= n || seen[(size_t)v]) order_ok = false;
            else seen[(size_t)v] = 1;
        }
    }
    rc = use_device(h);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    NB_CK(cudaStreamSynchronize(s));
    drop_graph(h);
    h->p = p;
    h->between = hd.between;
    h->tc = make_timecfg(p, hd.between);
    apply_tuning(h, p);
    // ensure_capacity re-lays the arena out when the j-split needs more room
    if (n > 0) {
        if (h->auto_cfg && h->p.tile_j == 0) h->tj = auto_tile(n);
        rc = ensure_capacity(h, n);
        if (rc) return rc;
    }
    h->n = n;
    h->ntiles = (int32_t)((n + h->tj - 1) / h->tj);
    NB_CK(cudaMemcpy(h->clk, &hd.clk, sizeof(Clock), cudaMemcpyHostToDevice));
    if (n == 0) return NB_OK;
    size_t off = sizeof hd;
    double* arrs[11] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->ax, h->ay, h->az, h->pot, h->m};
    const size_t d = sizeof(double) * (size_t)n;
    for (double* a : arrs) {
        NB_CK(cudaMemcpyAsync(a, b + off, d, cudaMemcpyHostToDevice, s));
        off += d;
    }
    NB_CK(cudaMemcpyAsync(h->type, b + off, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
    off += align_up(4 * (size_t)n, 8);
    NB_CK(cudaMemcpyAsync(h->ti_beg, b + off, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, s));
    off += sizeof(int64_t) * (size_t)n;
    NB_CK(cudaMemcpyAsync(h->ti_end, b + off, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, s));
    off += sizeof(int64_t) * (size_t)n;
    if (order_ok) {
        // the saved order lets the step graphs continue bit-identically
        NB_CK(cudaMemcpyAsync(h->perm, b + off, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
    }
    NB_CK(cudaStreamSynchronize(s));
    h->perm_valid = order_ok;
    h->host_steps = order_ok ? hd.order_steps : 0;
    return upload_sysdesc(h);
}

const char* nb_last_error(nb_handle* h) {
    if (!h) return g_create_err.empty() ? "null handle" : g_create_err.c_str();
    return h->err.c_str();
}

}  // extern "C"
