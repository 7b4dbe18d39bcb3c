// nb_engine.cu -- many-system engine: resident arena, footprint admission,
// continuous batching, CUDA-graph steps (C ABI in include/nbody_gb300.h).
//
// Host-side bookkeeping:
//   * the particle arena [0, max_particles) is handed out in contiguous ranges
//     by a first-fit free list; a request is admitted (FIFO) when a range of its
//     size and a system slot are free -- admission by memory footprint;
//   * running systems are ranked in slot order; the rank tables (SysDesc,
//     BatchSys, tile -> rank, (rank, i-block) work items largest first) are
//     rebuilt whenever the set of running systems changes, and the step graph
//     is re-captured then;
//   * a step advances every running system by one KDK step; nb_engine_run
//     replays the graph up to max_steps_per_call times; a per-slot gate on
//     the device holds each system once it has made its step count, so none
//     overshoots, and the call then retires finished systems and admits
//     queued ones.
// Each system follows run(sim) (src/run.jl:76-87, 101-173): force and +1/2
// kick on admission, nsteps x (drift, force, kick), -1/2 kick on retirement.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "nb_internal.cuh"

namespace {

constexpr int kTile = 256;
// Systems are put in Morton order at admission and every 64 of their own
// steps (measured on the 4096-system ensemble: 2363, 2379 and 2383 G
// interactions/s for every 16, 32 and 64 steps); any order gives correct
// forces, a fresher one only keeps the tiles compact.
#ifndef NB_ENGINE_RESORT_EVERY
#define NB_ENGINE_RESORT_EVERY 64
#endif
constexpr int kResortEvery = NB_ENGINE_RESORT_EVERY;

struct Request {
    int64_t id = 0;
    int64_t n = 0;
    std::vector<double> in;   // x, y, z, vx, vy, vz, m (n each)
    std::vector<double> out;  // x, y, z, vx, vy, vz after retirement
    double soft = 0.0;
    double dt = 0.0;
    int64_t nsteps = 0;
    int64_t steps_done = 0;
    int32_t state = NB_REQ_QUEUED;
    int32_t slot = -1;
    int64_t aoff = -1;
    // suspended state: in = x, y, z, vx, vy, vz, m, ax, ay, az (n each), order = lperm
    bool resumed = false;
    std::vector<int32_t> order;
};

}  // namespace

struct nb_engine {
    nb_engine_params p{};
    int dev = 0;
    cudaStream_t stream = nullptr;
    int nsm = 0;
    int occ_acc = 1, occ_pot = 1;
    int fblock = 128, fipt = 2;  // batch force launch shape
    std::string err;

    // device arena
    void* arena = nullptr;
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr, *pot = nullptr, *m = nullptr;
    int32_t* sysid = nullptr;
    int32_t* perm = nullptr;    // global radix-sort result (sorted slot -> arena particle)
    int32_t* lperm = nullptr;   // per-system Morton order, arena-relative
    int64_t* steps_slot = nullptr;
    int64_t* nsteps_slot = nullptr;  // target own-step count of each running slot (0 otherwise)
    void* sort_scratch = nullptr;
    float4* pack = nullptr;
    nb::TileOrigin* origin = nullptr;
    float4* ext = nullptr;
    int32_t* tile_rank = nullptr;
    nb::SysDesc* sysdesc = nullptr;
    nb::BatchSys* batchsys = nullptr;
    int32_t* rank_of_slot = nullptr;
    double* bbox = nullptr;
    double* dt_slot = nullptr;
    double* fac_step = nullptr;
    double* fac_once = nullptr;
    int2* items = nullptr;
    int2* items_new = nullptr;
    int32_t* counter = nullptr;
    uint32_t* derr = nullptr;
    int64_t tile_cap = 0;
    int64_t item_cap = 0;

    // host bookkeeping
    std::map<int64_t, int64_t> free_ranges;  // offset -> size
    std::vector<int64_t> slot_req;           // slot -> request id (-1 free)
    std::unordered_map<int64_t, Request> reqs;
    std::deque<int64_t> queue;
    int64_t next_id = 1;
    int64_t high_water = 0;
    bool dirty = true;
    int32_t nrank = 0;
    int32_t ntiles_total = 0;
    int32_t nitems = 0;
    int32_t max_small_n = 0;   // largest system ordered in shared memory
    // systems too large for the shared-memory sort ("large"): their ranks,
    // particle count and largest size; they are radix-sorted every step
    int32_t nlarge = 0;
    int64_t nl_particles = 0;
    int32_t max_large_n = 0;
    int32_t* large_ranks = nullptr;        // device, max_systems
    unsigned long long* box_key = nullptr;  // device, 6 per large system
    cudaGraphExec_t graph = nullptr;        // step graph without the per-slot gate
    cudaGraphExec_t graph_gated = nullptr;  // with it, for chunks some system finishes inside
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    nb_engine_stats stats{};
    std::vector<int64_t> finished;  // ids retired since the last nb_engine_drain_done
    bool inflight = false;           // a chunk of steps launched by nb_engine_run_async
    int64_t inflight_k = 0;          // its step count
};

namespace {

int efail(nb_engine* e, int code, const char* fmt, ...) {
    if (e) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        e->err = buf;
    }
    return code;
}

#define NE_CK(call)                                                                            \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return efail(e, e_ == cudaErrorMemoryAllocation ? NB_ERR_OOM : NB_ERR_CUDA,      \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

int64_t ntiles_of(int64_t n) { return (n + kTile - 1) / kTile; }

// First-fit allocation of a particle range; -1 when no free range is large enough.
int64_t alloc_range(nb_engine* e, int64_t n) {
    for (auto it = e->free_ranges.begin(); it != e->free_ranges.end(); ++it) {
        if (it->second >= n) {
            const int64_t off = it->first, sz = it->second;
            e->free_ranges.erase(it);
            if (sz > n) e->free_ranges[off + n] = sz - n;
            return off;
        }
    }
    return -1;
}

void free_range(nb_engine* e, int64_t off, int64_t n) {
    auto it = e->free_ranges.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != e->free_ranges.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        e->free_ranges.erase(nx);
    }
    if (it != e->free_ranges.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            e->free_ranges.erase(it);
        }
    }
}

void drop_graph(nb_engine* e) {
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    if (e->graph_gated) {
        cudaGraphExecDestroy(e->graph_gated);
        e->graph_gated = nullptr;
    }
}

int check_err(nb_engine* e) {
    uint32_t bits = 0;
    NE_CK(cudaMemcpyAsync(&bits, e->derr, sizeof bits, cudaMemcpyDeviceToHost, e->stream));
    NE_CK(cudaStreamSynchronize(e->stream));
    if (bits) {
        NE_CK(cudaMemset(e->derr, 0, sizeof bits));
        if (bits & nb::DEVERR_TIMEOUT) return efail(e, NB_ERR_TIMEOUT, "device wait timed out");
        return efail(e, NB_ERR_NUMERIC, "numeric error bits 0x%x", bits);
    }
    return NB_OK;
}

// Rebuild the rank tables of the running systems and upload them.
int rebuild(nb_engine* e) {
    std::vector<int32_t> slots;
    for (int32_t s = 0; s < (int32_t)e->slot_req.size(); ++s)
        if (e->slot_req[s] >= 0 && e->reqs[e->slot_req[s]].state == NB_REQ_RUNNING) slots.push_back(s);
    const int32_t R = (int32_t)slots.size();
    std::vector<nb::SysDesc> sd(R);
    std::vector<nb::BatchSys> bs(R);
    std::vector<int32_t> ros(e->p.max_systems, -1);
    std::vector<int32_t> trank;
    std::vector<double> fstep(e->p.max_systems, 0.0), dts(e->p.max_systems, 0.0);
    std::vector<int64_t> nst(e->p.max_systems, 0);
    int64_t soff = 0, toff = 0, hw = 0;
    std::vector<int32_t> lranks;
    int32_t max_large = 0;
    for (int32_t r = 0; r < R; ++r) {
        const Request& q = e->reqs[e->slot_req[slots[r]]];
        const int64_t nt = ntiles_of(q.n);
        nb::SysDesc d{};
        d.off = q.aoff;
        d.ubase = 0;
        d.n = (int32_t)q.n;
        d.tile_off = (int32_t)toff;
        d.ntiles = (int32_t)nt;
        const int32_t bt = nb::batch_block_targets(e->fblock, e->fipt);
        d.nblocks = (int32_t)((q.n + bt - 1) / bt);
        for (int k = 0; k < 6; ++k) d.soft[k] = q.soft;
        sd[r] = d;
        // sorted-slot offset: compact over the large systems (the only ones
        // the radix sort orders); unused by the others
        const bool large = q.n > nb::batch_small_sort_limit();
        bs[r] = nb::BatchSys{q.aoff, large ? soff : 0, (int32_t)q.n, slots[r]};
        if (large) {
            lranks.push_back(r);
            max_large = std::max<int32_t>(max_large, (int32_t)q.n);
            soff += q.n;
        }
        ros[slots[r]] = r;
        for (int64_t t = 0; t < nt; ++t) trank.push_back(r);
        fstep[slots[r]] = 1.0;
        dts[slots[r]] = q.dt;
        nst[slots[r]] = q.nsteps;
        toff += nt;
        hw = std::max(hw, q.aoff + q.n);
    }
    // Work items: (rank, i-block), systems with the most j-tiles first.
    std::vector<int32_t> order(R);
    for (int32_t r = 0; r < R; ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return sd[a].ntiles > sd[b].ntiles; });
    std::vector<int2> items;
    for (int32_t r : order)
        for (int32_t b = 0; b < sd[r].nblocks; ++b) items.push_back(make_int2(r, b));
    if (toff > e->tile_cap) return efail(e, NB_ERR_STATE, "tile capacity exceeded");
    if ((int64_t)items.size() > e->item_cap) return efail(e, NB_ERR_STATE, "work-item capacity exceeded");
    if (R > 0) {
        NE_CK(cudaMemcpy(e->sysdesc, sd.data(), sizeof(nb::SysDesc) * R, cudaMemcpyHostToDevice));
        NE_CK(cudaMemcpy(e->batchsys, bs.data(), sizeof(nb::BatchSys) * R, cudaMemcpyHostToDevice));
        NE_CK(cudaMemcpy(e->tile_rank, trank.data(), sizeof(int32_t) * toff, cudaMemcpyHostToDevice));
        NE_CK(cudaMemcpy(e->items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
    }
    NE_CK(cudaMemcpy(e->rank_of_slot, ros.data(), sizeof(int32_t) * ros.size(), cudaMemcpyHostToDevice));
    NE_CK(cudaMemcpy(e->fac_step, fstep.data(), sizeof(double) * fstep.size(), cudaMemcpyHostToDevice));
    NE_CK(cudaMemcpy(e->dt_slot, dts.data(), sizeof(double) * dts.size(), cudaMemcpyHostToDevice));
    NE_CK(cudaMemcpy(e->nsteps_slot, nst.data(), sizeof(int64_t) * nst.size(), cudaMemcpyHostToDevice));
    e->nrank = R;
    e->ntiles_total = (int32_t)toff;
    e->nitems = (int32_t)items.size();
    e->high_water = hw;
    e->max_small_n = 0;
    for (int32_t r = 0; r < R; ++r)
        if (sd[r].n <= nb::batch_small_sort_limit()) e->max_small_n = std::max(e->max_small_n, sd[r].n);
    e->nlarge = (int32_t)lranks.size();
    e->nl_particles = soff;
    e->max_large_n = max_large;
    if (!lranks.empty())
        NE_CK(cudaMemcpy(e->large_ranks, lranks.data(), sizeof(int32_t) * lranks.size(),
                         cudaMemcpyHostToDevice));
    e->dirty = false;
    drop_graph(e);
    return NB_OK;
}

nb::BatchForce force_args(nb_engine* e, const int2* items, int32_t nitems) {
    nb::BatchForce f{};
    f.sys = e->sysdesc;
    f.items = items;
    f.nitems = nitems;
    f.counter = e->counter;
    f.perm = e->lperm;
    f.pack = e->pack;
    f.origin = e->origin;
    f.ext = e->ext;
    f.x = e->x;
    f.y = e->y;
    f.z = e->z;
    f.m = e->m;
    f.ax = e->ax;
    f.ay = e->ay;
    f.az = e->az;
    f.pot = nullptr;
    f.G = e->p.G;
    f.err = e->derr;
    return f;
}

// Sort + pack of all running systems (enqueue only).  Systems of at most
// batch_small_sort_limit() particles are re-ordered in shared memory, one CTA
// each, at admission (force_all) and every kResortEvery of their own steps;
// larger systems are ordered every step by the global radix sort over the
// arena, which runs only when such a system is resident.  Tile origins and
// radii are recomputed from the current positions every step.
// gate: inside the step graph, skip the systems that have made all their
// steps (at admission every new system is ordered and packed).
cudaError_t enqueue_sort_pack(nb_engine* e, cudaStream_t s, bool force_all, bool gate) {
    const int64_t* nsteps = gate ? e->nsteps_slot : nullptr;
    cudaError_t r = cudaSuccess;
    if (e->nlarge > 0) {
        // the large systems' particles only; digits up to the large index bits
        const int64_t nl = e->nl_particles;
        int bits = 42, v = e->nlarge - 1;
        while (v > 0) {
            ++bits;
            v >>= 1;
        }
        const int passes = ((bits + 7) / 8 + 1) / 2 * 2;  // 8-bit digits, an even count
        r = nb::launch_batch_large_keys(e->batchsys, e->large_ranks, e->nlarge, e->max_large_n, e->x,
                                        e->y, e->z, e->box_key, nb::sort_keys_buffer(e->sort_scratch, nl),
                                        e->perm, s);
        if (r != cudaSuccess) return r;
        r = nb::launch_sort_keys(e->sort_scratch, nl, e->perm, passes, s);
        if (r != cudaSuccess) return r;
        r = nb::launch_batch_perm_to_local(e->batchsys, e->large_ranks, e->nlarge, e->max_large_n,
                                           e->perm, e->lperm, s);
        if (r != cudaSuccess) return r;
    }
    r = nb::launch_batch_sort_small(e->batchsys, e->nrank, e->max_small_n, e->steps_slot, nsteps,
                                    kResortEvery, force_all ? 1 : 0, e->x, e->y, e->z, e->bbox,
                                    e->lperm, s);
    if (r != cudaSuccess) return r;
    return nb::launch_batch_pack(e->tile_rank, e->ntiles_total, e->sysdesc, e->bbox, e->lperm, e->x,
                                 e->y, e->z, e->m, e->pack, e->origin, e->ext, e->sysid,
                                 e->steps_slot, nsteps, s);
}

// One KDK step of every running system (enqueue only).  gated: hold the
// systems that have made all their steps (a chunk that some system finishes
// inside); without it every running system steps (and no kernel reads the
// step counts).
cudaError_t enqueue_step(nb_engine* e, cudaStream_t s, bool gated) {
    const int64_t* nsteps = gated ? e->nsteps_slot : nullptr;
    cudaError_t r = nb::launch_batch_drift(e->x, e->y, e->z, e->vx, e->vy, e->vz, e->sysid, e->dt_slot,
                                           e->fac_step, e->steps_slot, nsteps, e->high_water, s);
    if (r != cudaSuccess) return r;
    r = enqueue_sort_pack(e, s, false, gated);
    if (r != cudaSuccess) return r;
    // force with the step's kick fused into its epilogue: every target of the
    // work items is a particle of a running system, and those are exactly
    // the particles the kick moves (fac_step 1)
    nb::BatchForce f = force_args(e, e->items, e->nitems);
    f.vx = e->vx;
    f.vy = e->vy;
    f.vz = e->vz;
    f.sysid = e->sysid;
    f.dt_slot = e->dt_slot;
    f.fac_slot = e->fac_step;
    f.steps_slot = e->steps_slot;
    f.nsteps_slot = nsteps;
    r = nb::launch_force_batch(e->p.law, f, e->occ_acc * e->nsm, e->fblock, e->fipt, s);
    if (r != cudaSuccess) return r;
    return nb::launch_batch_tick(e->batchsys, e->nrank, e->steps_slot, nsteps, s);
}

// Admit queued requests (FIFO) while a slot and a particle range are free;
// returns the slots admitted.
int admit(nb_engine* e, std::vector<int32_t>& admitted) {
    while (!e->queue.empty()) {
        Request& q = e->reqs[e->queue.front()];
        int32_t slot = -1;
        for (int32_t s = 0; s < (int32_t)e->slot_req.size(); ++s)
            if (e->slot_req[s] < 0) {
                slot = s;
                break;
            }
        if (slot < 0) break;
        const int64_t off = alloc_range(e, q.n);
        if (off < 0) break;  // head of the queue waits for space (FIFO)
        const size_t d = sizeof(double) * (size_t)q.n;
        const double* in = q.in.data();
        double* dst[10] = {e->x, e->y, e->z, e->vx, e->vy, e->vz, e->m, e->ax, e->ay, e->az};
        const int narr = q.resumed ? 10 : 7;
        for (int k = 0; k < narr; ++k)
            NE_CK(cudaMemcpyAsync(dst[k] + off, in + (size_t)k * q.n, d, cudaMemcpyHostToDevice, e->stream));
        if (q.resumed) {
            // own Morton order and step count, so the re-ordering schedule continues
            NE_CK(cudaMemcpyAsync(e->lperm + off, q.order.data(), sizeof(int32_t) * (size_t)q.n,
                                  cudaMemcpyHostToDevice, e->stream));
            NE_CK(cudaMemcpyAsync(e->steps_slot + slot, &q.steps_done, sizeof(int64_t),
                                  cudaMemcpyHostToDevice, e->stream));
        } else {
            NE_CK(cudaMemsetAsync(e->ax + off, 0, d, e->stream));
            NE_CK(cudaMemsetAsync(e->ay + off, 0, d, e->stream));
            NE_CK(cudaMemsetAsync(e->az + off, 0, d, e->stream));
            NE_CK(cudaMemsetAsync(e->steps_slot + slot, 0, sizeof(int64_t), e->stream));
        }
        NE_CK(nb::launch_fill_i32(e->sysid + off, q.n, slot, e->stream));
        NE_CK(cudaStreamSynchronize(e->stream));
        q.aoff = off;
        q.slot = slot;
        q.state = NB_REQ_RUNNING;
        q.in.clear();
        q.in.shrink_to_fit();
        q.order.clear();
        q.order.shrink_to_fit();
        e->slot_req[slot] = q.id;
        e->queue.pop_front();
        if (!q.resumed) admitted.push_back(slot);  // a resumed system needs no start-up
        q.resumed = false;
        e->dirty = true;
    }
    return NB_OK;
}

// Kick the given slots by fac (+0.5 on admission, -0.5 on retirement).
int half_kick(nb_engine* e, const std::vector<int32_t>& slots, double fac) {
    std::vector<double> f(e->p.max_systems, 0.0);
    for (int32_t s : slots) f[s] = fac;
    NE_CK(cudaMemcpy(e->fac_once, f.data(), sizeof(double) * f.size(), cudaMemcpyHostToDevice));
    NE_CK(nb::launch_batch_kick(e->vx, e->vy, e->vz, e->ax, e->ay, e->az, e->sysid, e->dt_slot,
                                e->fac_once, e->high_water, e->stream));
    return check_err(e);
}

// Force on the newly admitted systems only (their items), then +1/2 kick.
int start_systems(nb_engine* e, const std::vector<int32_t>& slots) {
    if (slots.empty()) return NB_OK;
    std::vector<int32_t> ros(e->p.max_systems);
    NE_CK(cudaMemcpy(ros.data(), e->rank_of_slot, sizeof(int32_t) * ros.size(), cudaMemcpyDeviceToHost));
    std::vector<nb::SysDesc> sd(e->nrank);
    NE_CK(cudaMemcpy(sd.data(), e->sysdesc, sizeof(nb::SysDesc) * sd.size(), cudaMemcpyDeviceToHost));
    std::vector<int32_t> ranks;
    for (int32_t s : slots) ranks.push_back(ros[s]);
    std::stable_sort(ranks.begin(), ranks.end(),
                     [&](int32_t a, int32_t b) { return sd[a].ntiles > sd[b].ntiles; });
    std::vector<int2> items;
    for (int32_t r : ranks)
        for (int32_t b = 0; b < sd[r].nblocks; ++b) items.push_back(make_int2(r, b));
    NE_CK(cudaMemcpy(e->items_new, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
    // New systems have step count 0, so they are due for ordering; the others
    // keep their order (their schedule must not depend on admissions).
    NE_CK(enqueue_sort_pack(e, e->stream, false, false));
    NE_CK(nb::launch_force_batch(e->p.law, force_args(e, e->items_new, (int32_t)items.size()),
                                 e->occ_acc * e->nsm, e->fblock, e->fipt, e->stream));
    return half_kick(e, slots, 0.5);
}

// Retire systems whose step count is reached: -1/2 kick, download, free.
int retire(nb_engine* e) {
    std::vector<int32_t> fin;
    for (int32_t s = 0; s < (int32_t)e->slot_req.size(); ++s) {
        if (e->slot_req[s] < 0) continue;
        Request& q = e->reqs[e->slot_req[s]];
        if (q.state == NB_REQ_RUNNING && q.steps_done >= q.nsteps) fin.push_back(s);
    }
    if (fin.empty()) return NB_OK;
    int rc = half_kick(e, fin, -0.5);
    if (rc) return rc;
    for (int32_t s : fin) {
        Request& q = e->reqs[e->slot_req[s]];
        q.out.resize((size_t)6 * q.n);
        const size_t d = sizeof(double) * (size_t)q.n;
        const double* src[6] = {e->x, e->y, e->z, e->vx, e->vy, e->vz};
        for (int k = 0; k < 6; ++k)
            NE_CK(cudaMemcpyAsync(q.out.data() + (size_t)k * q.n, src[k] + q.aoff, d,
                                  cudaMemcpyDeviceToHost, e->stream));
        NE_CK(nb::launch_fill_i32(e->sysid + q.aoff, q.n, -1, e->stream));
        NE_CK(cudaStreamSynchronize(e->stream));
        free_range(e, q.aoff, q.n);
        q.state = NB_REQ_DONE;
        e->slot_req[s] = -1;
        e->stats.done += 1;
        e->finished.push_back(q.id);
        e->dirty = true;
    }
    return NB_OK;
}

// Admission and start-up before a chunk of steps: retire finished systems,
// admit queued ones, rebuild the rank tables, start the admitted systems.
int prepare_chunk(nb_engine* e) {
    int rc = retire(e);  // systems submitted with nsteps == 0 or finished earlier
    if (rc) return rc;
    std::vector<int32_t> admitted;
    rc = admit(e, admitted);
    if (rc) return rc;
    if (e->dirty) {
        rc = rebuild(e);
        if (rc) return rc;
    }
    return start_systems(e, admitted);
}

// Launch up to max_steps engine steps (at most max_steps_per_call, and no more
// than the running system with the most steps left needs) as graph replays
// between two events; *k is the step count (0: nothing to run).  A system that
// makes its last step inside the chunk is held where it is by the step graph's
// per-slot gate (steps_slot >= nsteps_slot: no drift, force, kick or count)
// until the chunk ends and retires it, so chunks need not stop at the first
// system to finish.  No synchronisation.
int launch_chunk(nb_engine* e, int64_t max_steps, int64_t* k_out) {
    *k_out = 0;
    if (e->nrank == 0) return NB_OK;
    int64_t need = 0, least = INT64_MAX;
    for (int32_t s = 0; s < (int32_t)e->slot_req.size(); ++s) {
        if (e->slot_req[s] < 0) continue;
        const Request& q = e->reqs[e->slot_req[s]];
        if (q.state != NB_REQ_RUNNING) continue;
        need = std::max<int64_t>(need, q.nsteps - q.steps_done);
        least = std::min<int64_t>(least, q.nsteps - q.steps_done);
    }
    const int64_t k = std::min<int64_t>(std::min<int64_t>(max_steps, e->p.max_steps_per_call), need);
    if (k <= 0) return NB_OK;
    // the gate is needed only when some system finishes inside the chunk
    const bool gated = least < k;
    cudaGraphExec_t* exec = gated ? &e->graph_gated : &e->graph;
    if (!*exec) {
        cudaGraph_t g = nullptr;
        NE_CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t r1 = enqueue_step(e, e->stream, gated);
        cudaError_t r2 = cudaStreamEndCapture(e->stream, &g);
        if (r1 != cudaSuccess || r2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return efail(e, NB_ERR_CUDA, "engine step capture failed: %s",
                         cudaGetErrorString(r1 != cudaSuccess ? r1 : r2));
        }
        cudaError_t r3 = cudaGraphInstantiate(exec, g, 0);
        cudaGraphDestroy(g);
        if (r3 != cudaSuccess) {
            *exec = nullptr;
            return efail(e, NB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(r3));
        }
    }
    NE_CK(cudaEventRecord(e->ev0, e->stream));
    for (int64_t i = 0; i < k; ++i) NE_CK(cudaGraphLaunch(*exec, e->stream));
    NE_CK(cudaEventRecord(e->ev1, e->stream));
    *k_out = k;
    return NB_OK;
}

// Wait for a launched chunk of k steps, account it and retire the systems it
// finished.
int complete_chunk(nb_engine* e, int64_t k) {
    int rc = check_err(e);
    if (rc) return rc;
    float ms = 0.0f;
    NE_CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    e->stats.gpu_ms += ms;
    e->stats.engine_steps += k;
    for (int32_t s = 0; s < (int32_t)e->slot_req.size(); ++s) {
        if (e->slot_req[s] < 0) continue;
        Request& q = e->reqs[e->slot_req[s]];
        if (q.state != NB_REQ_RUNNING) continue;
        const int64_t adv = std::min<int64_t>(k, q.nsteps - q.steps_done);  // the gate stops it there
        q.steps_done += adv;
        e->stats.interactions += (double)adv * (double)q.n * (double)q.n;
    }
    return retire(e);
}

// Completes the chunk an nb_engine_run_async call left running, if any.
int finish_inflight(nb_engine* e) {
    if (!e->inflight) return NB_OK;
    e->inflight = false;
    return complete_chunk(e, e->inflight_k);
}

}  // namespace

extern "C" {

int nb_engine_create(const nb_engine_params* p, nb_engine** out) {
    if (!p || !out) return NB_ERR_INVALID_ARG;
    *out = nullptr;
    if (p->max_particles <= 0 || p->max_particles > 0x7fffffffLL || p->max_systems <= 0 ||
        (p->law != NB_LAW_SPLINE_G2 && p->law != NB_LAW_PLUMMER) ||
        !nb::batch_shape_ok(p->block > 0 ? p->block : 128, p->i_per_thread > 0 ? p->i_per_thread : 2))
        return NB_ERR_INVALID_ARG;
    nb_engine* e = new (std::nothrow) nb_engine();
    if (!e) return NB_ERR_OOM;
    e->p = *p;
    if (e->p.max_steps_per_call <= 0) e->p.max_steps_per_call = 64;
    e->dev = p->device;
    if (cudaSetDevice(e->dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete e;
        return NB_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->dev);
    e->fblock = p->block > 0 ? p->block : 128;
    e->fipt = p->i_per_thread > 0 ? p->i_per_thread : 2;
    e->occ_acc = nb::batch_ctas_per_sm(p->law, true, false, e->fblock, e->fipt);
    nb::prepare_batch_sort_small();
    const int64_t P = p->max_particles, S = p->max_systems;
    e->tile_cap = P / kTile + S;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = al256(off + bytes);
        return o;
    };
    const size_t dP = sizeof(double) * (size_t)P;
    size_t o_d[11];
    for (int k = 0; k < 11; ++k) o_d[k] = take(dP);
    size_t o_sys = take(sizeof(int32_t) * P), o_perm = take(sizeof(int32_t) * P);
    size_t o_lperm = take(sizeof(int32_t) * P), o_steps = take(sizeof(int64_t) * S);
    size_t o_nsteps = take(sizeof(int64_t) * S);
    size_t o_sort = take(nb::sort_scratch_bytes(P));
    size_t o_pack = take(sizeof(float4) * kTile * (size_t)e->tile_cap);
    size_t o_orig = take(sizeof(nb::TileOrigin) * (size_t)e->tile_cap);
    size_t o_ext = take(sizeof(float4) * (size_t)e->tile_cap);
    size_t o_trank = take(sizeof(int32_t) * (size_t)e->tile_cap);
    size_t o_sd = take(sizeof(nb::SysDesc) * S), o_bs = take(sizeof(nb::BatchSys) * S);
    size_t o_ros = take(sizeof(int32_t) * S), o_bbox = take(sizeof(double) * 6 * S);
    size_t o_dt = take(sizeof(double) * S), o_fs = take(sizeof(double) * S);
    size_t o_fo = take(sizeof(double) * S);
    size_t o_lr = take(sizeof(int32_t) * S), o_bk = take(sizeof(unsigned long long) * 6 * S);
    // work items: at most one per i-block of the smallest block (128 targets) per system
    e->item_cap = P / 128 + S;
    size_t o_it = take(sizeof(int2) * (size_t)e->item_cap), o_itn = take(sizeof(int2) * (size_t)e->item_cap);
    size_t o_cnt = take(sizeof(int32_t) * 4), o_err = take(sizeof(uint32_t) * 4);
    if (cudaMalloc(&e->arena, off) != cudaSuccess) {
        cudaStreamDestroy(e->stream);
        delete e;
        return NB_ERR_OOM;
    }
    char* b = static_cast<char*>(e->arena);
    double** dp[11] = {&e->x, &e->y, &e->z, &e->vx, &e->vy, &e->vz, &e->ax, &e->ay, &e->az, &e->pot, &e->m};
    for (int k = 0; k < 11; ++k) *dp[k] = (double*)(b + o_d[k]);
    e->sysid = (int32_t*)(b + o_sys);
    e->perm = (int32_t*)(b + o_perm);
    e->lperm = (int32_t*)(b + o_lperm);
    e->steps_slot = (int64_t*)(b + o_steps);
    e->nsteps_slot = (int64_t*)(b + o_nsteps);
    e->sort_scratch = b + o_sort;
    e->pack = (float4*)(b + o_pack);
    e->origin = (nb::TileOrigin*)(b + o_orig);
    e->ext = (float4*)(b + o_ext);
    e->tile_rank = (int32_t*)(b + o_trank);
    e->sysdesc = (nb::SysDesc*)(b + o_sd);
    e->batchsys = (nb::BatchSys*)(b + o_bs);
    e->rank_of_slot = (int32_t*)(b + o_ros);
    e->bbox = (double*)(b + o_bbox);
    e->dt_slot = (double*)(b + o_dt);
    e->fac_step = (double*)(b + o_fs);
    e->fac_once = (double*)(b + o_fo);
    e->large_ranks = (int32_t*)(b + o_lr);
    e->box_key = (unsigned long long*)(b + o_bk);
    e->items = (int2*)(b + o_it);
    e->items_new = (int2*)(b + o_itn);
    e->counter = (int32_t*)(b + o_cnt);
    e->derr = (uint32_t*)(b + o_err);
    cudaMemset(e->derr, 0, sizeof(uint32_t));
    nb::launch_fill_i32(e->sysid, P, -1, e->stream);
    cudaStreamSynchronize(e->stream);
    e->free_ranges[0] = P;
    e->slot_req.assign(S, -1);
    cudaEventCreate(&e->ev0);
    cudaEventCreate(&e->ev1);
    if (cudaGetLastError() != cudaSuccess) {
        cudaFree(e->arena);
        cudaStreamDestroy(e->stream);
        delete e;
        return NB_ERR_CUDA;
    }
    *out = e;
    return NB_OK;
}

int nb_engine_destroy(nb_engine* e) {
    if (!e) return NB_ERR_INVALID_ARG;
    cudaSetDevice(e->dev);
    cudaStreamSynchronize(e->stream);
    e->inflight = false;
    drop_graph(e);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    cudaFree(e->arena);
    cudaStreamDestroy(e->stream);
    delete e;
    return NB_OK;
}

int nb_batch_submit(nb_engine* e, int64_t n, const double* x, const double* y, const double* z,
                    const double* vx, const double* vy, const double* vz, const double* m,
                    double softening, double dt, int64_t nsteps, int64_t* id) {
    if (!e || !id) return NB_ERR_INVALID_ARG;
    if (n <= 0 || !x || !y || !z || !vx || !vy || !vz || !m)
        return efail(e, NB_ERR_INVALID_ARG, "bad particle arrays");
    if (!(softening > 0.0) || !std::isfinite(softening) || !(dt > 0.0) || nsteps < 0)
        return efail(e, NB_ERR_INVALID_ARG, "softening and dt must be > 0, nsteps >= 0");
    if (n > e->p.max_particles)
        return efail(e, NB_ERR_ADMISSION, "%lld particles exceed the arena (%lld)", (long long)n,
                     (long long)e->p.max_particles);
    Request q;
    q.id = e->next_id++;
    q.n = n;
    q.in.resize((size_t)7 * n);
    const double* src[7] = {x, y, z, vx, vy, vz, m};
    for (int k = 0; k < 7; ++k) std::memcpy(q.in.data() + (size_t)k * n, src[k], sizeof(double) * n);
    q.soft = softening;
    q.dt = dt;
    q.nsteps = nsteps;
    *id = q.id;
    e->queue.push_back(q.id);
    e->reqs.emplace(q.id, std::move(q));
    return NB_OK;
}

int nb_engine_run(nb_engine* e, int64_t max_steps, int64_t* steps_done) {
    if (!e || max_steps < 0) return NB_ERR_INVALID_ARG;
    if (steps_done) *steps_done = 0;
    NE_CK(cudaSetDevice(e->dev));
    int rc = finish_inflight(e);
    if (rc) return rc;
    rc = prepare_chunk(e);
    if (rc) return rc;
    int64_t k = 0;
    rc = launch_chunk(e, max_steps, &k);
    if (rc) return rc;
    if (k > 0) {
        rc = complete_chunk(e, k);
        if (rc) return rc;
    } else {
        rc = retire(e);
        if (rc) return rc;
    }
    if (steps_done) *steps_done = k;
    return NB_OK;
}

int nb_engine_run_async(nb_engine* e, int64_t max_steps, int64_t* steps_launched) {
    if (!e || max_steps < 0) return NB_ERR_INVALID_ARG;
    if (steps_launched) *steps_launched = 0;
    NE_CK(cudaSetDevice(e->dev));
    int rc = finish_inflight(e);
    if (rc) return rc;
    rc = prepare_chunk(e);
    if (rc) return rc;
    int64_t k = 0;
    rc = launch_chunk(e, max_steps, &k);
    if (rc) return rc;
    if (k > 0) {
        e->inflight = true;
        e->inflight_k = k;
    }
    if (steps_launched) *steps_launched = k;
    return NB_OK;
}

int nb_engine_sync(nb_engine* e) {
    if (!e) return NB_ERR_INVALID_ARG;
    NE_CK(cudaSetDevice(e->dev));
    return finish_inflight(e);
}

int nb_batch_poll(nb_engine* e, int64_t id, int32_t* state, int64_t* steps_done) {
    if (!e) return NB_ERR_INVALID_ARG;
    auto it = e->reqs.find(id);
    if (it == e->reqs.end()) return efail(e, NB_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
    if (state) *state = it->second.state;
    if (steps_done) *steps_done = it->second.steps_done;
    return NB_OK;
}

int nb_batch_fetch(nb_engine* e, int64_t id, double* x, double* y, double* z, double* vx,
                   double* vy, double* vz) {
    if (!e) return NB_ERR_INVALID_ARG;
    auto it = e->reqs.find(id);
    if (it == e->reqs.end()) return efail(e, NB_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
    Request& q = it->second;
    if (q.state != NB_REQ_DONE) return efail(e, NB_ERR_STATE, "request %lld not finished", (long long)id);
    double* dst[6] = {x, y, z, vx, vy, vz};
    for (int k = 0; k < 6; ++k)
        if (dst[k]) std::memcpy(dst[k], q.out.data() + (size_t)k * q.n, sizeof(double) * q.n);
    e->reqs.erase(it);
    return NB_OK;
}

int nb_batch_cancel(nb_engine* e, int64_t id) {
    if (!e) return NB_ERR_INVALID_ARG;
    if (e->inflight) {
        NE_CK(cudaSetDevice(e->dev));
        int rc = finish_inflight(e);
        if (rc) return rc;
    }
    auto it = e->reqs.find(id);
    if (it == e->reqs.end()) return efail(e, NB_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
    Request& q = it->second;
    if (q.state == NB_REQ_QUEUED) {
        e->queue.erase(std::remove(e->queue.begin(), e->queue.end(), id), e->queue.end());
    } else if (q.state == NB_REQ_RUNNING) {
        NE_CK(cudaSetDevice(e->dev));
        NE_CK(nb::launch_fill_i32(e->sysid + q.aoff, q.n, -1, e->stream));
        NE_CK(cudaStreamSynchronize(e->stream));
        free_range(e, q.aoff, q.n);
        e->slot_req[q.slot] = -1;
        e->dirty = true;
    }
    q.state = NB_REQ_CANCELLED;
    return NB_OK;
}

int nb_batch_suspend(nb_engine* e, int64_t id) {
    if (!e) return NB_ERR_INVALID_ARG;
    if (e->inflight) {
        NE_CK(cudaSetDevice(e->dev));
        int rc = finish_inflight(e);
        if (rc) return rc;
    }
    auto it = e->reqs.find(id);
    if (it == e->reqs.end()) return efail(e, NB_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
    Request& q = it->second;
    if (q.state != NB_REQ_RUNNING)
        return efail(e, NB_ERR_STATE, "request %lld is not running", (long long)id);
    NE_CK(cudaSetDevice(e->dev));
    NE_CK(cudaStreamSynchronize(e->stream));
    q.in.resize((size_t)10 * q.n);
    q.order.resize((size_t)q.n);
    const size_t d = sizeof(double) * (size_t)q.n;
    const double* src[10] = {e->x, e->y, e->z, e->vx, e->vy, e->vz, e->m, e->ax, e->ay, e->az};
    for (int k = 0; k < 10; ++k)
        NE_CK(cudaMemcpyAsync(q.in.data() + (size_t)k * q.n, src[k] + q.aoff, d,
                              cudaMemcpyDeviceToHost, e->stream));
    NE_CK(cudaMemcpyAsync(q.order.data(), e->lperm + q.aoff, sizeof(int32_t) * (size_t)q.n,
                          cudaMemcpyDeviceToHost, e->stream));
    NE_CK(nb::launch_fill_i32(e->sysid + q.aoff, q.n, -1, e->stream));
    NE_CK(cudaStreamSynchronize(e->stream));
    free_range(e, q.aoff, q.n);
    e->slot_req[q.slot] = -1;
    q.slot = -1;
    q.aoff = -1;
    q.state = NB_REQ_SUSPENDED;
    e->dirty = true;
    return NB_OK;
}

int nb_batch_resume(nb_engine* e, int64_t id) {
    if (!e) return NB_ERR_INVALID_ARG;
    auto it = e->reqs.find(id);
    if (it == e->reqs.end()) return efail(e, NB_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
    Request& q = it->second;
    if (q.state != NB_REQ_SUSPENDED)
        return efail(e, NB_ERR_STATE, "request %lld is not suspended", (long long)id);
    q.state = NB_REQ_QUEUED;
    q.resumed = true;
    e->queue.push_back(id);
    return NB_OK;
}

int nb_engine_get_stats(nb_engine* e, nb_engine_stats* out) {
    if (!e || !out) return NB_ERR_INVALID_ARG;
    nb_engine_stats s = e->stats;
    s.queued = (int64_t)e->queue.size();
    s.running = 0;
    s.resident_particles = 0;
    for (int32_t k = 0; k < (int32_t)e->slot_req.size(); ++k) {
        if (e->slot_req[k] < 0) continue;
        const Request& q = e->reqs[e->slot_req[k]];
        if (q.state == NB_REQ_RUNNING) {
            s.running += 1;
            s.resident_particles += q.n;
        }
    }
    *out = s;
    return NB_OK;
}

int nb_engine_drain_done(nb_engine* e, int64_t* ids, int64_t cap, int64_t* count) {
    if (!e || !count || (cap > 0 && !ids)) return NB_ERR_INVALID_ARG;
    const int64_t k = std::min<int64_t>(cap, (int64_t)e->finished.size());
    for (int64_t i = 0; i < k; ++i) ids[i] = e->finished[i];
    e->finished.erase(e->finished.begin(), e->finished.begin() + k);
    *count = k;
    return NB_OK;
}

const char* nb_engine_last_error(nb_engine* e) {
    if (!e) return "null engine";
    return e->err.c_str();
}

}  // extern "C"
