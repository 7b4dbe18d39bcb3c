"""CPU check of the tile box the packs record (nb_force_mixed.cuh k_pack,
nb_batch.cu k_batch_pack): each particle is split into a double-float pair,
the box is reduced in FP32 from the pairs relative to the tile's first
particle c, the origin is c + the box centre (FP64, split again), and the
half extents are enlarged by 1e-5 relative plus 4e-7 of the largest offset.
The near-tile test relies on every source's FP32 coordinate relative to the
origin lying inside those half extents, and the expansion test on the
radius covering them.  This test emulates the FP32 steps in numpy on random
tiles, including compact tiles far from the coordinate origin."""
import numpy as np


def f32(v):
    return np.asarray(v, dtype=np.float64).astype(np.float32)


def split_df(v):
    h = f32(v)
    return h, f32(np.asarray(v, dtype=np.float64) - h.astype(np.float64))


def rel_df(h, l, oh, ol):
    # (t.x - oh) + (t.y - ol), each operation rounded to FP32
    return f32(f32(h - oh).astype(np.float64) + f32(l - ol).astype(np.float64))


def test_sources_lie_inside_the_recorded_box_and_radius():
    rng = np.random.default_rng(11)
    for trial in range(300):
        centre = rng.uniform(-1, 1, 3) * 10.0 ** rng.uniform(-3, 4)
        size = 10.0 ** rng.uniform(-6, 1)
        p = centre + rng.normal(size=(256, 3)) * size * rng.uniform(0.1, 1.0, 3)
        hs, ls = split_df(p)
        ch, cl = hs[0], ls[0]
        f = rel_df(hs, ls, ch, cl)                      # offsets from the first particle
        lo, hi = f.min(0), f.max(0)
        ex = f32(hi - lo)
        amax = np.max(np.abs(np.concatenate([lo, hi])))
        slack = f32(np.float32(4.0e-7) * amax)
        half = f32(f32(f32(np.float32(0.5) * ex) * np.float32(1.0 + 1e-5)) + slack)
        rr = np.float32(0.5) * np.sqrt(np.float32((ex.astype(np.float64) ** 2).sum()))
        radius = f32(float(rr) * (1.0 + 1e-5) + 4.0e-7 * float(amax))
        centre_off = f32(np.float32(0.5) * f32(lo + hi))
        origin = p[0] + centre_off.astype(np.float64)
        oh, ol = split_df(origin)
        q = rel_df(hs, ls, oh, ol)
        assert np.all(np.abs(q) <= half), (trial, np.max(np.abs(q) - half))
        assert np.all(np.sqrt((q.astype(np.float64) ** 2).sum(1)) <= radius), trial
