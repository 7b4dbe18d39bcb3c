"""GPU integrator parity: kick/drift/bins through the C ABI against the oracle.
Given the same accelerations, velocities, positions and integer bins are
bit-identical (the integrator kernels round like the reference's expressions)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def load_pair(nb, oracle, data, acc, **kw):
    sim = nb.Simulation(data, **kw)
    sim.upload_acc(acc)
    okw = dict(soft=kw.get("ForceSofteningTable", [1e-4] * 6), G=kw.get("G", 1.0),
               dt=kw.get("TimeStep", None) or None, eta=kw.get("ErrTolTimestep", 0.025),
               time_end=kw.get("TimeEnd", 0.1), time_begin=kw.get("TimeBegin", 0.0),
               min_step=kw.get("MinStep", 1e-8), max_step=kw.get("MaxStep", float("inf")))
    o = oracle.OracleSim(data["pos"], data["vel"], data["mass"], **okw)
    o.ax[:], o.ay[:], o.az[:] = acc[:, 0], acc[:, 1], acc[:, 2]
    return sim, o


def test_const_kicks_and_drift_bitwise(nb, oracle):
    d = nb.plummer(3000, seed=4)
    acc = np.random.default_rng(1).normal(size=(3000, 3))
    sim, o = load_pair(nb, oracle, d, acc, ForceSofteningTable=[0.01] * 6, TimeStep=1e-3)
    nb.leapfrog_half_kick(sim, +1)
    o.half_kick(+1)
    nb.advance_and_find_timestep(sim)
    o.kick()
    nb.drift_particles_const_timestep(sim, 1e-3)
    o.drift_to_float(1e-3)
    nb.leapfrog_half_kick(sim, -1)
    o.half_kick(-1)
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["vel"], o.vel)
    np.testing.assert_array_equal(g["pos"], o.pos)


def test_adaptive_bins_kick_bitwise(nb, oracle):
    d = nb.plummer(3000, seed=6)
    rng = np.random.default_rng(2)
    acc = rng.normal(size=(3000, 3)) * 10.0 ** rng.uniform(-2, 3, size=(3000, 1))
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeEnd=1.0)
    sim, o = load_pair(nb, oracle, d, acc, **kw)
    nb.init_timesteps(sim)
    o.init_timesteps()
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
    nb.leapfrog_half_kick(sim, +1)
    o.half_kick(+1)
    mn = nb.find_min_endstep(sim)
    assert mn == o.find_min_endstep()
    nb.drift_particles_adaptive_timestep(sim, mn)
    o.drift_to_int(mn)
    nb.advance_and_find_timestep(sim)
    o.kick()
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["ti_begstep"], o.ti_beg)
    np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
    np.testing.assert_array_equal(g["vel"], o.vel)
    np.testing.assert_array_equal(g["pos"], o.pos)


def test_eta_sqrt_eps_criterion(nb, oracle):
    d = nb.plummer(500, seed=8)
    acc = np.random.default_rng(3).normal(size=(500, 3))
    sim = nb.Simulation(d, ForceSofteningTable=[5e-3] * 6, TimeEnd=1.0, criterion="eta_sqrt_eps")
    sim.upload_acc(acc)
    nb.init_timesteps(sim)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[5e-3] * 6, time_end=1.0,
                         criterion=oracle.CRIT_ETA_SQRT_EPS)
    o.ax[:], o.ay[:], o.az[:] = acc[:, 0], acc[:, 1], acc[:, 2]
    o.init_timesteps()
    np.testing.assert_array_equal(nb.get_all_data(sim)["ti_endstep"], o.ti_end)


def test_min_step_violation_raises(nb):
    """dt < MinStep: the reference's CPU path errors (src/base/Timestep.jl:9-11);
    here the call returns NB_ERR_NUMERIC."""
    pos = np.array([[0.0, 0, 0], [1e-6, 0, 0]])
    d = {"pos": pos, "vel": np.zeros((2, 3)), "mass": np.full(2, 1e12)}
    sim = nb.Simulation(d, ForceSofteningTable=[1e-9] * 6, MinStep=1e-2)
    nb.compute_force(sim)
    with pytest.raises(nb.NbodyError) as ei:
        nb.init_timesteps(sim)
    assert ei.value.code == -4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_circular_binary_const_leapfrog(nb, golden, precision):
    """test/Local-Timestep.jl:402-421 through run(sim) on the GPU."""
    g = golden("circular_binary_const_leapfrog.json")
    d = {"pos": np.array(g["pos0"]), "vel": np.array(g["vel0"]), "mass": np.full(2, g["mass"])}
    sim = nb.Simulation(d, G=g["G"], ForceSofteningTable=[g["softening"]] * 6, TimeStep=g["dt"],
                        TimeEnd=g["time_end"], precision=precision)
    nb.run(sim)
    p = nb.get_all_data(sim)["pos"]
    # mixed: FP32 pair forces (~1e-7 relative) accumulate into the orbital phase
    # over 2899 steps (one full orbit)
    rtol = g["rtol"] if precision == "fp64" else 1e-4
    np.testing.assert_allclose(p[0, 0], g["x_end"], rtol=rtol)
    np.testing.assert_allclose(p[0, 1], g["y_end"], rtol=rtol)


def test_circular_binary_adaptive(nb, golden):
    g = golden("circular_binary_adaptive.json")
    d = {"pos": np.array(g["pos0"]), "vel": np.array(g["vel0"]), "mass": np.full(2, g["mass"])}
    sim = nb.Simulation(d, G=g["G"], ForceSofteningTable=[g["softening"]] * 6,
                        ErrTolTimestep=g["eta"], TimeBase=g["time_base"],
                        TimeBegin=g["time_begin"], TimeEnd=g["time_end"], precision="fp64")
    nb.run(sim)
    r = nb.get_all_data(sim)
    np.testing.assert_array_equal(r["ti_begstep"], g["ti_begstep"])
    np.testing.assert_array_equal(r["ti_endstep"], g["ti_endstep"])
    np.testing.assert_allclose(r["pos"], g["pos"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(r["vel"], g["vel"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("law", ["spline", "plummer"])
def test_plummer4096_100_kdk_steps(nb, oracle, law):
    """Config: Plummer N=4096, eps=0.01, 100 KDK steps at dt=1e-3.  FP64 GPU vs
    oracle trajectories and energies; mixed form energy drift reported."""
    d = nb.plummer(4096, seed=1)
    h, dt = 0.01, 1e-3
    olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, dt=dt, time_end=0.1, law=olaw)
    o.compute_potential()
    e0 = o.diagnostics()
    o.run_begin()
    o.step(100)
    o.run_end()
    o.compute_potential()
    e1 = o.diagnostics()
    for precision in ("fp64", "mixed"):
        sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, TimeStep=dt, TimeEnd=0.1,
                            precision=precision, law=law)
        E0 = nb.diagnostics(sim)
        nb.run(sim, nsteps=100)
        E1 = nb.diagnostics(sim)
        g = nb.get_all_data(sim)
        if precision == "fp64":
            np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-9)
            np.testing.assert_allclose(E0["K"] + E0["W"], e0["K"] + e0["W"], rtol=1e-12)
            np.testing.assert_allclose(E1["K"] + E1["W"], e1["K"] + e1["W"], rtol=1e-10)
            np.testing.assert_allclose(E1["P"], e1["P"], atol=1e-14)
            np.testing.assert_allclose(E1["L"], e1["L"], atol=1e-13)
        else:
            drift = abs((E1["K"] + E1["W"]) / (E0["K"] + E0["W"]) - 1)
            odrift = abs((e1["K"] + e1["W"]) / (e0["K"] + e0["W"]) - 1)
            assert drift <= max(10 * odrift, 1e-6)
            np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-5)


def test_adaptive_many_body_matches_oracle(nb, oracle):
    """Adaptive bins on a 2000-body Plummer sphere: the FP64 GPU run keeps the
    oracle's integer time line (same bins, same number of substeps)."""
    d = nb.plummer(2000, seed=12)
    h = 0.01
    T1 = 0.05
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, time_end=T1, max_step=1e-2)
    o.run_begin()
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, TimeEnd=T1, MaxStep=1e-2, precision="fp64")
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    for _ in range(60):
        o.step(1)
        nb.step(sim, 1)
        ti, _ = sim.time()
        assert ti == o.t_int
        if ti >= 1 << 30:
            break
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
    np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-11)
    np.testing.assert_allclose(g["vel"], o.vel, rtol=0, atol=1e-9)


def test_step_graph_matches_single_calls(nb):
    """nb_step's graph replay equals the same operations issued one by one
    (with the sources re-ordered every step, as every nb_compute_force does)."""
    d = nb.plummer(5000, seed=3)
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, precision="mixed", resort_every=1)
    a = nb.Simulation(d, **kw)
    b = nb.Simulation(d, **kw)
    for s in (a, b):
        nb.compute_force(s)
        nb.leapfrog_half_kick(s, +1)
    nb.step(a, 5)
    t = 0.0
    for _ in range(5):
        t = t + 1e-3
        nb.drift_particles_const_timestep(b, t)
        nb.compute_force(b)
        nb.advance_and_find_timestep(b)
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    np.testing.assert_array_equal(ga["pos"], gb["pos"])
    np.testing.assert_array_equal(ga["vel"], gb["vel"])


@pytest.mark.parametrize("resort", [0, 7])
def test_step_graph_sort_interval(nb, resort):
    """Steps between two Morton re-orders pack the sources in the last order:
    the run matches the one that re-orders every step to FP32 round-off
    (after 40 steps of dt 1e-3 on a Plummer sphere: position difference
    <= 1e-9 of the system's extent, velocity difference <= 1e-6 of the
    largest speed).  A second nb_step call and an upload in between keep the
    order valid."""
    d = nb.plummer(6000, seed=31)
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, precision="mixed")
    a = nb.Simulation(d, resort_every=resort, **kw)
    b = nb.Simulation(d, resort_every=1, **kw)
    for s in (a, b):
        nb.compute_force(s)
        nb.leapfrog_half_kick(s, +1)
        nb.step(s, 25)
    # re-upload each run's own state (the clock restarts in both): the order of
    # the next steps is rebuilt before the first replay
    for s in (a, b):
        g = nb.get_all_data(s)
        s.upload({"pos": g["pos"], "vel": g["vel"], "mass": d["mass"]})
        nb.step(s, 15)
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    ext = np.ptp(gb["pos"], axis=0).max()
    assert np.abs(ga["pos"] - gb["pos"]).max() <= 1e-9 * ext
    vmax = np.linalg.norm(gb["vel"], axis=1).max()
    assert np.abs(ga["vel"] - gb["vel"]).max() <= 1e-6 * vmax


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_upload_of_same_size_reuses_step_graphs(nb, precision):
    """An upload of as many particles keeps the captured step graphs (they
    hold pointers and counts, not data): stepping the new state gives the
    same result, bit for bit, as a fresh handle holding it.  A smaller upload
    re-captures them."""
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, precision=precision, resort_every=1)
    a = nb.Simulation(nb.plummer(3000, seed=71), **kw)
    nb.step(a, 4)
    for n, seed in ((3000, 72), (1500, 73)):
        d = nb.plummer(n, seed=seed)
        a.upload(d)
        nb.step(a, 6)
        b = nb.Simulation(d, **kw)
        nb.step(b, 6)
        ga, gb = nb.get_all_data(a), nb.get_all_data(b)
        np.testing.assert_array_equal(ga["pos"], gb["pos"])
        np.testing.assert_array_equal(ga["vel"], gb["vel"])
        b.close()


def test_resort_every_validation(nb):
    d = nb.plummer(64, seed=1)
    for bad in (-1, (1 << 20) + 1):
        with pytest.raises(Exception, match="resort_every"):
            nb.Simulation(d, ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, resort_every=bad)


def test_collision_adaptive_mixed_vs_fp64(nb):
    """Two Hernquist spheres on a parabolic approach, power-of-two bins from
    dt_i = eta sqrt(eps/|a_i|) (eta 0.025, dt_max 1e-2), eps 5e-3: the mixed
    form's energy and momentum drift stay at the FP64 run's level, and both
    runs keep the same integer time line."""
    data = nb.collision(1024, seed=5, separation=20.0)
    T = 20 * 1e-2
    res = {}
    for prec in ("fp64", "mixed"):
        sim = nb.Simulation(data, ForceSofteningTable=[5e-3] * 6, TimeEnd=T, MaxStep=1e-2,
                            criterion="eta_sqrt_eps", precision=prec)
        d0 = nb.diagnostics(sim)
        nb.run(sim)
        d1 = nb.diagnostics(sim)
        steps, pairs = nb.counters(sim)
        assert steps > 20 and pairs >= steps * 1.0 and pairs <= steps * 2048.0 * 2048.0
        res[prec] = (d0, d1, steps, nb.get_all_data(sim))
    for prec, (d0, d1, steps, g) in res.items():
        e0, e1 = d0["K"] + d0["W"], d1["K"] + d1["W"]
        assert abs(e1 - e0) / abs(e0) < 1e-3, (prec, (e1 - e0) / e0)
        assert np.linalg.norm(d1["P"] - d0["P"]) < 1e-6
    (f0, f1, fs, fg), (m0, m1, ms, mg) = res["fp64"], res["mixed"]
    ef = (f1["K"] + f1["W"]) / (f0["K"] + f0["W"]) - 1
    em = (m1["K"] + m1["W"]) / (m0["K"] + m0["W"]) - 1
    assert abs(em - ef) < 1e-5, (em, ef)
    np.testing.assert_allclose(mg["pos"], fg["pos"], rtol=0, atol=1e-4)


def test_check_sync_point_follows_the_time_line(nb, oracle):
    """check_sync_point is true exactly after the steps at which every particle
    was active (all Ti_endstep past the step's min_endstep); FP64 run against
    the oracle's time line."""
    d = nb.plummer(600, seed=13)
    h, T1 = 0.01, 0.05
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, time_end=T1, max_step=1e-2)
    o.run_begin()
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, TimeEnd=T1, MaxStep=1e-2, precision="fp64")
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    seen = {True: 0, False: 0}
    for _ in range(40):
        m = o.find_min_endstep()
        o.step(1)
        nb.step(sim, 1)
        flag = nb.check_sync_point(sim)
        assert flag == bool(np.all(o.ti_end > m))
        assert flag == bool(np.all(nb.get_all_data(sim)["ti_endstep"] > m))
        seen[flag] += 1
        if o.t_int >= 1 << 30:
            break
    assert seen[True] > 0 and seen[False] > 0


@pytest.mark.parametrize("adaptive", [False, True])
def test_euler_time_integration_matches_oracle(nb, oracle, adaptive):
    """TimeIntegrationAlgorithm = Euler: the step loop without the half kicks
    (src/run.jl:85-87, 171-173), FP64 against the oracle driven the same way;
    the circular-orbit setting of test/Local-Timestep.jl:760-790 (two massless
    particles around a point-mass background field)."""
    GM, R = 1.0, 1.0
    v = np.sqrt(GM / R)
    d = {"pos": np.array([[R, 0, 0], [-R, 0, 0]], float),
         "vel": np.array([[0, v, 0], [0, -v, 0]], float), "mass": np.zeros(2)}
    T = 0.5
    kw = dict(ForceSofteningTable=[1e-4] * 6, TimeEnd=T, precision="fp64",
              bgforce=nb.PointMassField(GM), TimeIntegrationAlgorithm=nb.Euler)
    okw = dict(soft=[1e-4] * 6, time_end=T, bg_kind=1, bg_gm=GM)
    if adaptive:
        kw.update(MaxStep=1e-2)
        okw.update(max_step=1e-2)
    else:
        kw.update(TimeStep=1e-3)
        okw.update(dt=1e-3)
    sim = nb.Simulation(d, **kw)
    nb.run(sim, nsteps=200)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], **okw)
    o.compute_force()
    o.init_timesteps()
    o.step(200)
    g = nb.get_all_data(sim)
    np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-12)
    np.testing.assert_allclose(g["vel"], o.vel, rtol=0, atol=1e-12)


def test_unknown_time_integration_algorithm(nb):
    with pytest.raises(ValueError):
        nb.Simulation(nb.plummer(16, seed=1), ForceSofteningTable=[0.01] * 6,
                      TimeIntegrationAlgorithm="RK4")
