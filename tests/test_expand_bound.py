"""CPU check of the admission bound of the expanded far-tile loop
(nb_pairs.cuh, warp_expandable / pair_loop_expand): for a target x and a tile
of radius R whose box is at distance d from x, the loop is used when
R^2 + |x|^2 <= 5 d^2, and evaluates

    r^2 = (|q|^2 + |x|^2) - 2 q.x          (|q|^2 rounded once by the pack)

in FP32 (one add, three FMAs).  The bound caps the rounding error of r^2 at
about 3 x 5 ulp of r^2.  This test emulates those FP32 steps in numpy (an FMA
as an exact FP64 product-sum rounded once to FP32) on random tiles and
targets that pass the test, and checks the error against the exact r^2."""
import numpy as np

BOUND = 5.0
ULP = 2.0 ** -24


def f32(v):
    return np.asarray(v, dtype=np.float64).astype(np.float32).astype(np.float64)


def fma32(a, b, c):
    return f32(a * b + c)


def test_expanded_r2_error_stays_within_the_bound():
    rng = np.random.default_rng(3)
    worst = 0.0
    worst_rejected = 0.0
    count = 0
    for _ in range(400):
        half = rng.uniform(0.05, 1.0, 3)             # tile box half extents
        q = f32(rng.uniform(-1, 1, (256, 3)) * half)  # sources relative to the tile origin
        R = float(np.sqrt((half ** 2).sum()))
        # targets at random directions and distances, kept when the test admits them
        dirs = rng.normal(size=(64, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        x = f32(dirs * rng.uniform(0.5, 8.0, (64, 1)) * R)
        d = np.sqrt((np.maximum(np.abs(x) - half, 0.0) ** 2).sum(1))
        ok = (R * R + (x ** 2).sum(1)) <= BOUND * d * d
        for xt, admitted in zip(x, ok):
            qq = fma32(q[:, 0], q[:, 0], fma32(q[:, 1], q[:, 1], f32(q[:, 2] * q[:, 2])))
            cc = fma32(xt[0], xt[0], fma32(xt[1], xt[1], f32(xt[2] * xt[2])))
            r2 = f32(qq + cc)
            r2 = fma32(q[:, 2], f32(-2.0 * xt[2]), r2)
            r2 = fma32(q[:, 1], f32(-2.0 * xt[1]), r2)
            r2 = fma32(q[:, 0], f32(-2.0 * xt[0]), r2)
            exact = ((q - xt) ** 2).sum(1)
            err = float(np.max(np.abs(r2 - exact) / exact))
            if admitted:
                worst = max(worst, err)
                count += 1
            else:
                worst_rejected = max(worst_rejected, err)
    assert count > 1000
    assert worst <= 3 * BOUND * ULP * 2, worst   # about 3 x 5 ulp, with a factor 2 to spare
    # the targets the test turns away (closer to the tile) would fare worse
    assert worst_rejected > 4 * worst
