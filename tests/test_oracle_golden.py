"""CPU tests: the oracle (C restatement of the reference's CPU Float64 path)
against the known answers of the reference's own tests (tests/golden/)."""
import numpy as np
import pytest


def test_binary_static(oracle, golden):
    """test/StaticTest.jl:161-207 (unitless variant): force, energy, timestep, momentum."""
    g = golden("binary_static.json")
    pos = np.array(g["pos"])
    vel = np.array(g["vel"])
    m = np.full(2, g["mass"])
    s = oracle.OracleSim(pos, vel, m, soft=[g["softening"]] * 6, G=g["G"], eta=g["eta"],
                         time_end=0.1)
    s.compute_force()
    a = s.acc
    rtol = g["rtol"]
    assert abs(a[0, 0] + a[1, 0]) <= rtol * abs(a[0, 0])
    np.testing.assert_allclose(abs(a[0, 0]), g["acc_abs"], rtol=rtol)
    np.testing.assert_allclose(abs(a[1, 0]), g["acc_abs"], rtol=rtol)
    s.compute_potential()
    d = s.diagnostics()
    np.testing.assert_allclose(d["W"], g["potential"], rtol=rtol)
    np.testing.assert_allclose(d["K"], g["kinetic"], rtol=rtol)
    np.testing.assert_allclose(d["K"] + d["W"], g["energy"], rtol=rtol)
    s.init_timesteps()
    dt_sim = (s.ti_end[0] - s.ti_beg[0]) * s._s.time_interval
    assert dt_sim < g["dt_bound"]
    assert np.all(np.abs(d["P"]) <= rtol * g["mass"] * abs(g["vel"][0][1]))
    np.testing.assert_allclose(d["L"], g["angular_momentum"], rtol=rtol, atol=1e-30)


def test_box_probe(oracle, golden):
    """test/StaticTest.jl:299-350: force/potential of the box at the origin."""
    g = golden("box_probe.json")
    pos = np.array(g["pos"])
    m = np.full(len(pos), g["mass"])
    acc, pot = oracle.force(pos, m, np.array([g["probe"]]), g["softening"], G=g["G"])
    np.testing.assert_allclose(acc[0], g["acc"], rtol=1e-14)
    np.testing.assert_allclose(pot[0], g["pot"], rtol=1e-14)


def test_circular_binary_const_leapfrog(oracle, golden):
    """test/Local-Timestep.jl:402-421: run(sim) with constant-step leapfrog equals
    the hand-written leapfrog at the final x, y."""
    g = golden("circular_binary_const_leapfrog.json")
    s = oracle.OracleSim(np.array(g["pos0"]), np.array(g["vel0"]), np.full(2, g["mass"]),
                         soft=[g["softening"]] * 6, G=g["G"], dt=g["dt"], time_end=g["time_end"])
    s.run_begin()
    # the float time line t += dt reaches time_end after exactly N-1 steps
    t, k = 0.0, 0
    while True:
        t = t + g["dt"]
        k += 1
        if t >= g["time_end"]:
            break
    assert k == g["N"] - 1
    s.step(k)
    s.run_end()
    np.testing.assert_allclose(s.x[0], g["x_end"], rtol=g["rtol"])
    np.testing.assert_allclose(s.y[0], g["y_end"], rtol=g["rtol"])


def test_circular_binary_adaptive(oracle, golden):
    """Adaptive power-of-two time line (src/base/Timestep.jl:1-82, src/run.jl)
    against an independent pure-Python restatement."""
    g = golden("circular_binary_adaptive.json")
    s = oracle.OracleSim(np.array(g["pos0"]), np.array(g["vel0"]), np.full(2, g["mass"]),
                         soft=[g["softening"]] * 6, G=g["G"], eta=g["eta"],
                         time_base=g["time_base"], time_begin=g["time_begin"], time_end=g["time_end"])
    s.run_begin()
    steps = 0
    while True:
        s.step(1)
        steps += 1
        if g["time_begin"] + s.t_int * s._s.time_interval >= g["time_end"]:
            break
    s.run_end()
    assert steps == g["steps"]
    np.testing.assert_array_equal(s.ti_beg, g["ti_begstep"])
    np.testing.assert_array_equal(s.ti_end, g["ti_endstep"])
    np.testing.assert_allclose(s.pos, g["pos"], rtol=g["rtol"], atol=1e-15)
    np.testing.assert_allclose(s.vel, g["vel"], rtol=g["rtol"], atol=1e-15)


def test_julia_pairwise_sum(oracle):
    """or_jl_sum follows Base's blocked pairwise reduction: exact on integers,
    equal to a sequential sum below the block size, close to fsum above."""
    import math

    rng = np.random.default_rng(3)
    for n in (0, 1, 2, 15, 16, 17, 1023, 1024, 1025, 5000):
        a = rng.normal(size=n)
        if n == 0:
            assert oracle.jl_sum(a) == 0.0
            continue
        s = oracle.jl_sum(a)
        if n <= 1024:
            seq = 0.0 if n < 2 else a[0] + a[1]
            if n >= 2:
                for v in a[2:]:
                    seq = seq + v
            else:
                seq = a[0]
            assert s == seq
        assert abs(s - math.fsum(a)) <= 1e-12 * np.abs(a).sum()
    ints = np.arange(1, 100001, dtype=float)
    assert oracle.jl_sum(ints) == 100000 * 100001 / 2


def test_spline_continuity_and_gradient(oracle):
    """The spline branch r < h is pinned by no reference test: check continuity
    of force and potential at u = 0.5 and u = 1, the Newtonian limit r >= h, and
    a = -grad(phi) by central differences."""
    h = 0.1
    src = np.array([[0.0, 0.0, 0.0]])
    m = np.array([2.0])
    for u in (0.5, 1.0):
        r = u * h
        lo = np.array([[r * (1 - 1e-9), 0, 0]])
        hi = np.array([[r * (1 + 1e-9), 0, 0]])
        a_lo, p_lo = oracle.force(src, m, lo, h)
        a_hi, p_hi = oracle.force(src, m, hi, h)
        assert abs(a_lo[0, 0] - a_hi[0, 0]) <= 1e-6 * abs(a_hi[0, 0])
        assert abs(p_lo[0] - p_hi[0]) <= 1e-6 * abs(p_hi[0])
    r = 1.5 * h
    a, p = oracle.force(src, m, np.array([[r, 0, 0]]), h)
    np.testing.assert_allclose(a[0, 0], -2.0 / r ** 2, rtol=1e-14)
    np.testing.assert_allclose(p[0], -2.0 / r, rtol=1e-14)
    for r in (0.13 * h, 0.37 * h, 0.61 * h, 0.88 * h, 1.7 * h):
        eps = 1e-6 * h
        _, pp = oracle.force(src, m, np.array([[r + eps, 0, 0]]), h)
        _, pm = oracle.force(src, m, np.array([[r - eps, 0, 0]]), h)
        a, _ = oracle.force(src, m, np.array([[r, 0, 0]]), h)
        np.testing.assert_allclose(a[0, 0], -(pp[0] - pm[0]) / (2 * eps), rtol=2e-5)


def test_self_pair_and_coincident(oracle):
    """Self pair contributes zero force and zero potential (r == 0 branch)."""
    pos = np.array([[0.3, -0.2, 0.1]])
    a, p = oracle.force(pos, np.array([5.0]), pos, 0.01)
    assert np.all(a == 0.0) and p[0] == 0.0


def test_plummer_law_closed_form(oracle):
    """PLUMMER law: a = G m d / (r^2 + h^2)^(3/2), phi = -G m / sqrt(r^2 + h^2)."""
    h = 0.05
    src = np.array([[0.0, 0.0, 0.0]])
    tgt = np.array([[0.03, 0.04, 0.0]])
    a, p = oracle.force(src, np.array([3.0]), tgt, h, G=2.0, law=oracle.LAW_PLUMMER)
    r2 = 0.05 ** 2
    np.testing.assert_allclose(a[0], -2.0 * 3.0 * tgt[0] / (r2 + h * h) ** 1.5, rtol=1e-14)
    np.testing.assert_allclose(p[0], -2.0 * 3.0 / np.sqrt(r2 + h * h), rtol=1e-14)


def test_min_step_error(oracle):
    """src/base/Timestep.jl:9-11: dt < MinStep is an error."""
    pos = np.array([[0.0, 0, 0], [1e-6, 0, 0]])
    s = oracle.OracleSim(pos, np.zeros((2, 3)), np.full(2, 1e12), soft=[1e-9] * 6, min_step=1e-2)
    s.compute_force()
    with pytest.raises(RuntimeError):
        s.init_timesteps()
