"""Snapshots inside steps on the GPU: find_next_sync_point_and_drift
(src/base/Timestep.jl:197-215 constant, :224-245 adaptive) against the oracle.

The device step graph stops its drift at every output time that falls inside a
step (a conditional graph node skips force and kick), the host writes the
snapshot, and the next replay finishes the step.  x + v dt1 + v dt2 rounds
differently from x + v dt, so these runs have their own trajectories; the
tests pin them:
* two bodies in FP64: every pair force is the same double on both sides and
  the sum of two terms is exact, so snapshots and final states are
  bit-identical to the oracle;
* many bodies in lock step: after each GPU step the oracle drifts with the
  same output splits, takes the GPU's accelerations and kicks; positions,
  velocities, bins and snapshots stay bit-identical;
* mixed precision against the free-running oracle at the stated tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Recorder:
    """sim.config.output.func stand-in: keeps (t_int, t_float, pos, vel)."""

    def __init__(self, nb):
        self.nb = nb
        self.snaps = []

    def __call__(self, sim):
        ti, tf = sim.time()
        g = self.nb.get_all_data(sim)
        self.snaps.append({"t_int": ti, "t_float": tf, "pos": g["pos"], "vel": g["vel"]})


def _binary():
    # circular binary (test/Local-Timestep.jl:402-421 setting), D >> h
    r, m = 0.5, 1.0
    v = np.sqrt(m / (4 * r))
    return {"pos": np.array([[r, 0.0, 0.0], [-r, 0.0, 0.0]]),
            "vel": np.array([[0.0, v, 0.0], [0.0, -v, 0.0]]), "mass": np.full(2, m)}


@pytest.mark.parametrize("adaptive", [False, True])
def test_binary_snapshots_bitwise(nb, oracle, adaptive):
    d = _binary()
    h = 0.01
    between = 2.7e-3
    kw = dict(ForceSofteningTable=[h] * 6, TimeEnd=1.0, precision="fp64",
              TimeBetweenSnapshots=between)
    okw = dict(soft=[h] * 6, time_end=1.0, between_snapshots=between, max_snapshots=256)
    if adaptive:
        kw.update(MaxStep=1e-2)
        okw.update(max_step=1e-2)
    else:
        kw.update(TimeStep=1e-3)
        okw.update(dt=1e-3)
    rec = Recorder(nb)
    sim = nb.Simulation(d, OutputFunc=rec, **kw)
    nsteps = 60 if adaptive else 100
    nb.run(sim, nsteps=nsteps)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], **okw)
    o.run_begin()
    o.step(nsteps)
    o.run_end()
    osn = o.snapshots
    # run() writes the initial conditions first (src/run.jl:90)
    assert len(rec.snaps) == len(osn) + 1 and len(osn) >= 10
    for g, r in zip(rec.snaps[1:], osn):
        assert g["t_float"] == r["t_float"]
        if adaptive:
            assert g["t_int"] == r["t_int"]
        np.testing.assert_array_equal(g["pos"], r["pos"])
        np.testing.assert_array_equal(g["vel"], r["vel"])
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["pos"], o.pos)
    np.testing.assert_array_equal(g["vel"], o.vel)
    _, _, at, k = sim.output_state()
    assert not at and k == len(osn)


@pytest.mark.parametrize("adaptive", [False, True])
def test_many_body_snapshots_lockstep_bitwise(nb, oracle, adaptive):
    d = nb.plummer(600, seed=13)
    h, T1, between = 0.01, 0.05, 3.7e-3
    kw = dict(ForceSofteningTable=[h] * 6, TimeEnd=T1, precision="fp64",
              TimeBetweenSnapshots=between)
    okw = dict(soft=[h] * 6, time_end=T1, between_snapshots=between, max_snapshots=512)
    if adaptive:
        kw.update(MaxStep=1e-2)
        okw.update(max_step=1e-2)
    else:
        kw.update(TimeStep=1e-3)
        okw.update(dt=1e-3)
    sim = nb.Simulation(d, **kw)
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    g0 = nb.get_all_data(sim)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], **okw)
    o.ax[:], o.ay[:], o.az[:] = g0["acc"][:, 0], g0["acc"][:, 1], g0["acc"][:, 2]
    o.init_timesteps()
    o.half_kick(+1)
    np.testing.assert_array_equal(g0["vel"], o.vel)
    nsteps = 60 if adaptive else 40
    seen = 0
    for _ in range(nsteps):
        snaps = []
        while True:
            k, at = nb.step_until_output(sim, 1)
            if not at:
                assert k == 1
                break
            assert k == 0
            ti, tf = sim.time()
            gs = nb.get_all_data(sim)
            snaps.append((ti, tf, gs["pos"], gs["vel"]))
        g = nb.get_all_data(sim)
        before = len(o.snapshots)
        o.sync_and_drift()
        o.ax[:], o.ay[:], o.az[:] = g["acc"][:, 0], g["acc"][:, 1], g["acc"][:, 2]
        o.kick()
        if not adaptive:
            o._s.last_t_float = o._s.t_float  # src/run.jl:164
        osn = o.snapshots[before:]
        assert len(osn) == len(snaps)
        for (ti, tf, p, v), r in zip(snaps, osn):
            assert tf == r["t_float"]
            if adaptive:
                assert ti == r["t_int"]
            np.testing.assert_array_equal(p, r["pos"])
            np.testing.assert_array_equal(v, r["vel"])
        seen += len(snaps)
        np.testing.assert_array_equal(g["pos"], o.pos)
        np.testing.assert_array_equal(g["vel"], o.vel)
        if adaptive:
            np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
            np.testing.assert_array_equal(g["ti_begstep"], o.ti_beg)
            ti, _ = sim.time()
            assert ti == o.t_int
            if ti >= 1 << 30:
                break
    assert seen >= 5


@pytest.mark.parametrize("adaptive", [False, True])
def test_mixed_snapshots_within_tolerance(nb, oracle, adaptive):
    d = nb.plummer(2048, seed=21)
    h, T1, between = 0.01, 0.05, 2.9e-3
    kw = dict(ForceSofteningTable=[h] * 6, TimeEnd=T1, precision="mixed",
              TimeBetweenSnapshots=between)
    okw = dict(soft=[h] * 6, time_end=T1, between_snapshots=between, max_snapshots=64)
    if adaptive:
        # MaxStep below every particle's criterion step: one shared bin, so
        # FP32 force errors cannot move a particle to another bin
        kw.update(MaxStep=1e-3)
        okw.update(max_step=1e-3)
    else:
        kw.update(TimeStep=1e-3)
        okw.update(dt=1e-3)
    rec = Recorder(nb)
    sim = nb.Simulation(d, OutputFunc=rec, **kw)
    nsteps = 30
    nb.run(sim, nsteps=nsteps)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], **okw)
    o.run_begin()
    o.step(nsteps)
    o.run_end()
    osn = o.snapshots
    assert len(rec.snaps) == len(osn) + 1 and len(osn) >= 5
    for g, r in zip(rec.snaps[1:], osn):
        assert g["t_float"] == r["t_float"]
        # FP32 pair forces (median relative error ~1e-7) over at most 30 steps
        np.testing.assert_allclose(g["pos"], r["pos"], rtol=0, atol=1e-7)
        np.testing.assert_allclose(g["vel"], r["vel"], rtol=0, atol=1e-5)


def test_step_passes_through_outputs(nb):
    """nb_step with a schedule splits the drift at output times without
    stopping: the result equals stopping at every output and resuming."""
    d = nb.plummer(1024, seed=5)
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, TimeEnd=1.0, precision="mixed",
              TimeBetweenSnapshots=2.5e-3)
    a = nb.Simulation(d, **kw)
    b = nb.Simulation(d, **kw)
    for s in (a, b):
        s._ck(s._lib.nb_run_begin(s.handle))
    nb.step(a, 20)  # no output function: passes through the output times
    done, stops = 0, 0
    while done < 20:
        k, at = nb.step_until_output(b, 20 - done)
        done += k
        stops += int(at)
    # the same float time line on the host: t += dt, output times += 2.5e-3
    t, out, expect = 0.0, 2.5e-3, 0
    for _ in range(20):
        nxt = t + 1e-3
        while out <= nxt:
            expect += 1
            out += 2.5e-3
        t = nxt
    assert stops == expect >= 7
    assert a.output_state()[3] == b.output_state()[3] == expect
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    np.testing.assert_array_equal(ga["pos"], gb["pos"])
    np.testing.assert_array_equal(ga["vel"], gb["vel"])
    # without a schedule the trajectory differs (one drift per step)
    c = nb.Simulation(d, **{**kw, "TimeBetweenSnapshots": None})
    c._ck(c._lib.nb_run_begin(c.handle))
    nb.step(c, 20)
    assert not np.array_equal(nb.get_all_data(c)["pos"], ga["pos"])


def test_checkpoint_at_an_output_resumes_bitwise(nb, tmp_path):
    """A restart file written while the time line is stopped at an output time
    inside a step continues the step bit-identically (the clock image holds the
    split step and the schedule)."""
    d = nb.plummer(700, seed=8)
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeEnd=0.05, MaxStep=1e-2, precision="fp64",
              TimeBetweenSnapshots=3.1e-3)
    a = nb.Simulation(d, **kw)
    a._ck(a._lib.nb_run_begin(a.handle))
    at = False
    while not at:
        _, at = nb.step_until_output(a, 50)
    path = tmp_path / "at_output.bin"
    nb.saverestart(a, str(path))
    b = nb.loadrestart(str(path))
    assert b.TimeBetweenSnapshots == 3.1e-3
    assert b.output_state() == a.output_state()
    for s in (a, b):
        for _ in range(3):
            nb.step_until_output(s, 10)
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    np.testing.assert_array_equal(ga["pos"], gb["pos"])
    np.testing.assert_array_equal(ga["vel"], gb["vel"])
    np.testing.assert_array_equal(ga["ti_endstep"], gb["ti_endstep"])
    assert a.time() == b.time()


def test_euler_restart_keeps_the_algorithm(nb, tmp_path):
    """An Euler run restarted from its restart file stays Euler: no half kick
    at the end (the image carries the algorithm, as the reference's restart
    file carries config.time.algorithm, src/restart.jl:129-139)."""
    GM, R = 1.0, 1.0
    v = np.sqrt(GM / R)
    d = {"pos": np.array([[R, 0, 0], [-R, 0, 0]], float),
         "vel": np.array([[0, v, 0], [0, -v, 0]], float), "mass": np.zeros(2)}
    kw = dict(ForceSofteningTable=[1e-4] * 6, TimeStep=1e-3, TimeEnd=0.5, precision="fp64",
              bgforce=nb.PointMassField(GM), TimeIntegrationAlgorithm=nb.Euler)
    ref = nb.Simulation(d, **kw)
    nb.run(ref, nsteps=100)
    a = nb.Simulation(d, **kw)
    a._ck(a._lib.nb_run_begin(a.handle))
    nb.step(a, 40)
    path = tmp_path / "euler.bin"
    nb.saverestart(a, str(path))
    b = nb.loadrestart(str(path))
    assert b.euler
    nb.step(b, 60)
    b._ck(b._lib.nb_run_end(b.handle))
    np.testing.assert_array_equal(nb.get_all_data(b)["vel"], nb.get_all_data(ref)["vel"])
    np.testing.assert_array_equal(nb.get_all_data(b)["pos"], nb.get_all_data(ref)["pos"])


def test_snapshot_interval_validation(nb):
    d = nb.plummer(64, seed=1)
    sim = nb.Simulation(d, ForceSofteningTable=[0.01] * 6, TimeEnd=1.0)
    with pytest.raises(nb.NbodyError):
        sim.set_snapshot_interval(-1.0)
    with pytest.raises(nb.NbodyError):
        # below TimeInterval: BetweenSnapshotsInt would be 0 and the reference's
        # output loop would never end
        sim.set_snapshot_interval(1.0 / (1 << 31))
    sim.set_snapshot_interval(0.01)
    ni, nf, at, k = sim.output_state()
    assert ni == int(np.floor(0.01 / (1.0 / (1 << 30)))) and nf == 0.01 and not at and k == 0
