// nb_force_worklist.cu -- persistent, evenly partitioned mixed-precision force
// over one or many independent systems.
//
// Work units are (system s, i-block b, j-tile t) in the order s, b, t; an
// i-block is kWBt = 256 targets of one system, a j-tile 256 of its sources.
// Every unit costs the same (256 x 256 pair evaluations), so the grid of G
// persistent CTAs splits the concatenated unit range [0, U) into G equal
// contiguous shares: CTA c takes [U c / G, U (c+1) / G).  Balance is exact to
// one unit whatever N, the number of systems or their sizes (the same idea as
// "stream-K" GEMM decompositions).
//
// A CTA walks its share in order.  Every warp keeps a cursor (s, b, t); when
// the cursor enters a new i-block the warp loads its targets, and when it
// leaves one it writes the result: the final acceleration/potential when the
// CTA covered the whole j-range of that block, otherwise a compensated
// (sum, carry) partial into slot 0 (the CTA's first block) or slot 1 (its last
// block).  k_force_fixup then adds the partials of every block cut by a CTA
// boundary, in CTA order, so results are deterministic for a given grid.
//
// The j-tiles of a share stream through the same bulk-copy ring as
// k_force_mixed (mbarrier per stage, last warp out refills it) -- the ring just
// runs across block and system boundaries.
#include "nb_pairs.cuh"

namespace nb {

constexpr int kWBlock = 128;
constexpr int kWIpt = 2;
constexpr int kWBt = kWBlock * kWIpt;
constexpr int kPartialQ = 8;  // (sum, carry) of ax, ay, az, pot

struct Cursor {
    int32_t s, b, t;
    int32_t ntiles, nblocks, tile_off, ntg;
    int64_t off;
};

__device__ __forceinline__ void cursor_load_sys(const WorkList& w, int32_t s, int32_t nb0,
                                                int32_t ntg0, Cursor& c) {
    const SysDesc& d = w.sys[s];
    c.s = s;
    c.ntiles = d.ntiles;
    c.tile_off = d.tile_off;
    c.off = d.off;
    const bool dyn = w.d_count != nullptr;
    c.nblocks = dyn ? nb0 : d.nblocks;
    c.ntg = dyn ? ntg0 : d.n;
}

__device__ __forceinline__ void cursor_advance(const WorkList& w, Cursor& c, int32_t nb0,
                                               int32_t ntg0, int32_t bstride = 1) {
    if (++c.t == c.ntiles) {
        c.t = 0;
        c.b += bstride;
        if (c.b >= c.nblocks) {
            c.b = 0;
            if (c.s + 1 < w.nsys)
                cursor_load_sys(w, c.s + 1, nb0, ntg0, c);
            else
                c.s = w.nsys;
        }
    }
}

__device__ __forceinline__ Cursor cursor_at(const WorkList& w, int64_t u, int32_t nb0,
                                            int32_t ntg0) {
    int32_t lo = 0, hi = w.nsys - 1;
    while (lo < hi) {  // last system with ubase <= u
        const int32_t mid = (lo + hi + 1) >> 1;
        if (w.sys[mid].ubase <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    Cursor c;
    cursor_load_sys(w, lo, nb0, ntg0, c);
    const int64_t r = u - w.sys[lo].ubase;
    c.b = (int32_t)(r / c.ntiles);
    c.t = (int32_t)(r % c.ntiles);
    return c;
}

// Problem size, possibly from the device-side active count (one system).
__device__ __forceinline__ int64_t total_units(const WorkList& w, int32_t& nb0, int32_t& ntg0) {
    nb0 = 0;
    ntg0 = 0;
    if (w.d_count) {
        ntg0 = *w.d_count;
        nb0 = (ntg0 + kWBt - 1) / kWBt;
        return (int64_t)nb0 * w.sys[0].ntiles;
    }
    return w.units;
}

__device__ __forceinline__ int32_t target_index(const WorkList& w, const Cursor& c, int32_t slot) {
    if (w.active) return w.active[slot];
    const int64_t q = c.off + slot;
    return w.perm ? w.perm[q] : (int32_t)q;
}

__device__ __forceinline__ void issue_tile(float4* buf, uint64_t* full, int st, const float4* pack,
                                           int64_t gtile) {
    mbar_arrive_expect_tx(&full[st], kTileJ * sizeof(float4));
    bulk_g2s(&buf[st * kTileJ], pack + gtile * kTileJ, kTileJ * sizeof(float4), &full[st]);
}

template <int LAW, bool ACC, bool POT>
__global__ void __launch_bounds__(kWBlock, (ACC && !POT) ? 8 : 1) k_force_worklist(WorkList w) {
    constexpr int IPT = kWIpt;
    constexpr int BLOCK = kWBlock;
    constexpr int NW = kWBlock / 32;
    __shared__ __align__(128) float4 buf[kStages * kTileJ];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ uint32_t done[kStages];
    __shared__ uint32_t issued;
    __shared__ float2 tpx[kWBt], tpy[kWBt], tpz[kWBt];

    int32_t nb0, ntg0;
    const int64_t U = total_units(w, nb0, ntg0);
    const int64_t G = gridDim.x, cta = blockIdx.x;
    int64_t len;
    int32_t bstride = 1;
    Cursor cur;
    if (w.block_cyclic) {
        // One system: this CTA takes the whole i-blocks cta, cta + G, ...
        cursor_load_sys(w, 0, nb0, ntg0, cur);
        if (cta >= cur.nblocks) return;  // CTA-uniform
        len = ((cur.nblocks - 1 - cta) / G + 1) * (int64_t)cur.ntiles;
        cur.b = (int32_t)cta;
        cur.t = 0;
        bstride = (int32_t)G;
    } else {
        const int64_t u0 = U * cta / G, u1 = U * (cta + 1) / G;
        if (u0 >= u1) return;  // CTA-uniform
        len = u1 - u0;
        cur = cursor_at(w, u0, nb0, ntg0);
    }
    const int tid = threadIdx.x, lane = tid & 31;

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            done[s] = 0;
        }
        issued = 0;
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        Cursor pc = cur;
        int v = 0;
        for (; v < kStages && v < len; ++v) {
            issue_tile(buf, full, v, w.pack, (int64_t)pc.tile_off + pc.t);
            cursor_advance(w, pc, nb0, ntg0, bstride);
        }
        issued = (uint32_t)v;
    }

    int32_t pidx[IPT];
    float hh[IPT], h2[IPT];
    float sx[IPT], sy[IPT], sz[IPT], sp[IPT];
    float cx[IPT], cy[IPT], cz[IPT], cp[IPT];
    int64_t seg_v0 = 0;
    int32_t seg_t0 = 0;
    bool timed_out = false;

    for (int64_t v = 0; v < len; ++v) {
        if (v == 0 || cur.t == 0) {
            // Entering i-block (s, b): load this thread's targets.
            seg_v0 = v;
            seg_t0 = cur.t;
            const SysDesc& d = w.sys[cur.s];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int32_t slot = cur.b * kWBt + k * BLOCK + tid;
                pidx[k] = -1;
                double x = 0.0, y = 0.0, z = 0.0, h = d.soft[0];
                if (slot < cur.ntg) {
                    const int32_t p = target_index(w, cur, slot);
                    pidx[k] = p;
                    x = w.x[p];
                    y = w.y[p];
                    z = w.z[p];
                    if (w.type) h = d.soft[w.type[p] - 1];
                }
                tpx[k * BLOCK + tid] = split_df(x);
                tpy[k * BLOCK + tid] = split_df(y);
                tpz[k * BLOCK + tid] = split_df(z);
                hh[k] = (float)h;
                h2[k] = hh[k] * hh[k];
                sx[k] = sy[k] = sz[k] = sp[k] = 0.0f;
                cx[k] = cy[k] = cz[k] = cp[k] = 0.0f;
            }
        }
        const int st = (int)(v % kStages);
        const uint32_t par = (uint32_t)(v / kStages) & 1u;
        const float4 oh = w.origin[cur.tile_off + cur.t].hi, ol = w.origin[cur.tile_off + cur.t].lo;
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
            if (lane == 0) atomicOr(w.err, DEVERR_TIMEOUT);
            break;
        }
        const float4* b = &buf[st * kTileJ];
        bool near = false;
        if (LAW == NB_LAW_SPLINE_G2)
            near = warp_near<IPT>(w.ext[cur.tile_off + cur.t], xr, yr, zr, hh, pidx);
        if (near)
            pair_loop_checked<LAW, ACC, POT, IPT>(b, xr, yr, zr, hh, h2, ax, ay, az, ap, w.ext[cur.tile_off + cur.t].w);
        else
            pair_loop_far<LAW, ACC, POT, IPT>(b, xr, yr, zr, h2, ax, ay, az, ap, w.ext[cur.tile_off + cur.t].w);

        // Release stage st; the last warp out refills it with unit v + kStages.
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t prev = atomicAdd(&done[st], 1u);
            if (prev == NW - 1) {
                __threadfence_block();
                done[st] = 0;
                if (v + kStages < len) {
                    Cursor pc = cur;
#pragma unroll
                    for (int k = 0; k < kStages; ++k) cursor_advance(w, pc, nb0, ntg0, bstride);
                    issue_tile(buf, full, st, w.pack, (int64_t)pc.tile_off + pc.t);
                    atomicAdd(&issued, 1u);
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

        if (cur.t == cur.ntiles - 1 || v == len - 1) {
            // Leaving i-block (s, b).
            const bool complete = seg_t0 == 0 && cur.t == cur.ntiles - 1;
            if (complete) {
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const int32_t p = pidx[k];
                    if (p < 0) continue;
                    if (ACC) {
                        w.ax[p] = ((double)sx[k] + (double)cx[k]) * w.G;
                        w.ay[p] = ((double)sy[k] + (double)cy[k]) * w.G;
                        w.az[p] = ((double)sz[k] + (double)cz[k]) * w.G;
                    }
                    if (POT) {
                        double phi = -((double)sp[k] + (double)cp[k]);
                        if (LAW == NB_LAW_PLUMMER)
                            phi += (double)((float)w.m[p] * rsqrt_approx(h2[k]));
                        w.pot[p] = phi * w.G;
                    }
                }
            } else {
                const int slot = seg_v0 == 0 ? 0 : 1;
                float* part = w.partial + (size_t)(cta * 2 + slot) * kPartialQ * kWBt;
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const int q = k * BLOCK + tid;
                    part[0 * kWBt + q] = sx[k];
                    part[1 * kWBt + q] = cx[k];
                    part[2 * kWBt + q] = sy[k];
                    part[3 * kWBt + q] = cy[k];
                    part[4 * kWBt + q] = sz[k];
                    part[5 * kWBt + q] = cz[k];
                    part[6 * kWBt + q] = sp[k];
                    part[7 * kWBt + q] = cp[k];
                }
            }
        }
        cursor_advance(w, cur, nb0, ntg0, bstride);
    }

    if (__syncthreads_or(timed_out)) {
        if (tid == 0) {
            // Drain the copies that may still be in flight (the last kStages issued).
            const uint32_t n_issued = issued;
            for (uint32_t u = n_issued > kStages ? n_issued - kStages : 0; u < n_issued; ++u)
                (void)mbar_wait_bounded(&full[u % kStages], (u / kStages) & 1u, kWaitTimeoutNs / 8);
        }
    }
}

// Adds the partials of every i-block cut by a CTA boundary.  Thread block c
// handles the block that contains the first unit of CTA c + 1, if that block
// starts inside CTA c's share (so each cut block is handled exactly once).
template <int LAW, bool ACC, bool POT>
__global__ void __launch_bounds__(kWBlock) k_force_fixup(WorkList w) {
    int32_t nb0, ntg0;
    const int64_t U = total_units(w, nb0, ntg0);
    const int64_t G = w.grid, c = blockIdx.x;
    if (c + 1 >= G) return;
    const int64_t uc = U * c / G;
    const int64_t un = U * (c + 1) / G;
    if (un >= U || un == uc) return;
    const Cursor cb = cursor_at(w, un, nb0, ntg0);
    if (cb.t == 0) return;  // CTA boundary coincides with a block boundary
    const int64_t ublk = un - cb.t;
    if (ublk < uc) return;  // block started in an earlier CTA
    const int64_t ulast = ublk + cb.ntiles - 1;
    int64_t cl = ulast * G / U;
    while (cl + 1 < G && U * (cl + 1) / G <= ulast) ++cl;
    while (cl > c && U * cl / G > ulast) --cl;
    const SysDesc& d = w.sys[cb.s];
    for (int q = threadIdx.x; q < kWBt; q += blockDim.x) {
        const int32_t slot = cb.b * kWBt + q;
        if (slot >= cb.ntg) continue;
        const int32_t p = target_index(w, cb, slot);
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int64_t cc = c; cc <= cl; ++cc) {
            const int64_t s0 = U * cc / G, s1 = U * (cc + 1) / G;
            if (s0 == s1) continue;  // empty share
            const int ps = (cc == c && ublk != uc) ? 1 : 0;
            const float* part = w.partial + (size_t)(cc * 2 + ps) * kPartialQ * kWBt;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                acc[j] += (double)part[(2 * j) * kWBt + q] + (double)part[(2 * j + 1) * kWBt + q];
        }
        if (ACC) {
            w.ax[p] = acc[0] * w.G;
            w.ay[p] = acc[1] * w.G;
            w.az[p] = acc[2] * w.G;
        }
        if (POT) {
            double phi = -acc[3];
            if (LAW == NB_LAW_PLUMMER) {
                const float h = (float)(w.type ? d.soft[w.type[p] - 1] : d.soft[0]);
                phi += (double)((float)w.m[p] * rsqrt_approx(h * h));
            }
            w.pot[p] = phi * w.G;
        }
    }
}

template <int LAW, bool ACC, bool POT>
static int occupancy_of() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_worklist<LAW, ACC, POT>, kWBlock,
                                                      0) != cudaSuccess)
        return 0;
    return nb;
}

int worklist_ctas_per_sm(int law, bool acc, bool pot) {
    if (law == NB_LAW_PLUMMER) {
        if (!acc) return occupancy_of<NB_LAW_PLUMMER, false, true>();
        return pot ? occupancy_of<NB_LAW_PLUMMER, true, true>()
                   : occupancy_of<NB_LAW_PLUMMER, true, false>();
    }
    if (!acc) return occupancy_of<NB_LAW_SPLINE_G2, false, true>();
    return pot ? occupancy_of<NB_LAW_SPLINE_G2, true, true>()
               : occupancy_of<NB_LAW_SPLINE_G2, true, false>();
}

size_t worklist_partial_bytes(int64_t grid) {
    return (size_t)grid * 2 * kPartialQ * kWBt * sizeof(float);
}

int worklist_block_targets() { return kWBt; }

template <int LAW, bool ACC, bool POT>
static cudaError_t launch_wl(const WorkList& w, cudaStream_t s) {
    k_force_worklist<LAW, ACC, POT><<<(unsigned)w.grid, kWBlock, 0, s>>>(w);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (w.grid > 1 && !w.block_cyclic)
        k_force_fixup<LAW, ACC, POT><<<(unsigned)(w.grid - 1), kWBlock, 0, s>>>(w);
    return cudaGetLastError();
}

cudaError_t launch_force_worklist(int law, const WorkList& w, cudaStream_t s) {
    const bool acc = w.ax != nullptr, pot = w.pot != nullptr;
    if (w.grid <= 0 || (!acc && !pot)) return cudaSuccess;
    if (law == NB_LAW_PLUMMER) {
        if (!acc) return launch_wl<NB_LAW_PLUMMER, false, true>(w, s);
        return pot ? launch_wl<NB_LAW_PLUMMER, true, true>(w, s)
                   : launch_wl<NB_LAW_PLUMMER, true, false>(w, s);
    }
    if (!acc) return launch_wl<NB_LAW_SPLINE_G2, false, true>(w, s);
    return pot ? launch_wl<NB_LAW_SPLINE_G2, true, true>(w, s)
               : launch_wl<NB_LAW_SPLINE_G2, true, false>(w, s);
}

}  // namespace nb
