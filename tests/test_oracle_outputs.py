"""CPU tests of the oracle's snapshot loop: find_next_sync_point_and_drift
(src/base/Timestep.jl:197-245) with the schedule of src/base/Config.jl:436-439,
749-750, against a plain-Python restatement of the same loop.  Massless
particles keep a = 0, so the kicks leave the velocities alone and every
position is the exact chain of drifts the loop performs."""
import math

import numpy as np


def _free_particles(n=7, seed=3):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), np.zeros(n)


def _drift(pos, vel, dt):
    return pos + vel * dt  # elementwise IEEE products and sums, as drift_particles_kernel


def test_const_step_snapshots_follow_the_loop(oracle):
    pos, vel, m = _free_particles()
    dt, between, nsteps = 1e-3, 2.7e-3, 40
    o = oracle.OracleSim(pos, vel, m, soft=[0.01] * 6, dt=dt, time_end=1.0,
                         between_snapshots=between, max_snapshots=64)
    o.run_begin()
    o.step(nsteps)
    # restatement: src/base/Timestep.jl:197-215, src/directsum/timestep.jl:22-38
    t, next_out, x = 0.0, 0.0 + between, pos.copy()
    snaps = []
    for _ in range(nsteps):
        next_system = t + dt
        while next_out <= next_system:
            x = _drift(x, vel, next_out - t)
            t = next_out
            snaps.append((t, x.copy()))
            next_out += between
        x = _drift(x, vel, next_system - t)
        t = next_system
    got = o.snapshots
    assert len(got) == len(snaps) == 14
    for (ts, xs), g in zip(snaps, got):
        assert g["t_float"] == ts
        np.testing.assert_array_equal(g["pos"], xs)
        np.testing.assert_array_equal(g["vel"], vel)
    np.testing.assert_array_equal(o.pos, x)
    assert o.t_float == t
    assert o.next_output[1] == next_out


def test_adaptive_snapshots_on_the_integer_line(oracle):
    pos, vel, m = _free_particles(seed=4)
    T, between, max_step = 0.05, 3.7e-3, 1e-2
    o = oracle.OracleSim(pos, vel, m, soft=[0.01] * 6, time_end=T, max_step=max_step,
                         between_snapshots=between, max_snapshots=64)
    o.run_begin()
    ti = T / (1 << 30)
    between_int = math.floor(between / ti)
    # a = 0: dt = MaxStep, the largest power of two below MaxStep / TimeInterval
    step = 1 << 30
    while step > max_step / ti:
        step >>= 1
    t_int, next_out, x = 0, between_int, pos.copy()
    snaps = []
    for _ in range(6):
        end = t_int + step  # every particle shares the bin: min_endstep
        while next_out <= end:
            x = _drift(x, vel, (next_out - t_int) * ti)
            t_int = next_out
            snaps.append((t_int, 0.0 + t_int * ti, x.copy()))
            next_out += between_int
        x = _drift(x, vel, (end - t_int) * ti)
        t_int = end
        o.step(1)
        assert o.t_int == t_int
    got = o.snapshots
    assert len(got) == len(snaps) > 0
    for (ts, tf, xs), g in zip(snaps, got):
        assert g["t_int"] == ts and g["t_float"] == tf
        np.testing.assert_array_equal(g["pos"], xs)
    np.testing.assert_array_equal(o.pos, x)
    assert o.next_output[0] == next_out


def test_no_schedule_means_one_drift_per_step(oracle):
    pos, vel, m = _free_particles(seed=5)
    o = oracle.OracleSim(pos, vel, m, soft=[0.01] * 6, dt=1e-3, time_end=1.0)
    o.run_begin()
    o.step(5)
    x, t = pos.copy(), 0.0
    for _ in range(5):
        x = _drift(x, vel, (t + 1e-3) - t)
        t = t + 1e-3
    np.testing.assert_array_equal(o.pos, x)
    assert o.snapshots == []
