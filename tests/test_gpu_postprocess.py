"""Force post-processing on the GPU (postprocessing_force of
src/directsumgpu/gravity.jl:64-79): analytic background field and Milgrom
MOND, against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


@pytest.mark.parametrize("field", ["point_mass", "pseudo_newtonian"])
@pytest.mark.parametrize("mond", [False, True])
def test_force_postprocessing_matches_oracle(nb, oracle, field, mond):
    d = nb.plummer(2000, seed=71)
    h, GM, rg, c = 0.01, 0.5, 0.01, (0.3, -0.2, 0.1)
    f = nb.PointMassField(GM, c) if field == "point_mass" else nb.PseudoNewtonianField(GM, rg, c)
    kw = dict(GravityModel=nb.MOND1983Milgrom, ACC0=0.2, MOND_nuIndex=2.0) if mond else {}
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="fp64", bgforce=f, **kw)
    nb.compute_force(sim)
    g = nb.get_all_data(sim)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6,
                         bg_kind=1 if field == "point_mass" else 2, bg_gm=GM, bg_center=c,
                         bg_rg=rg if field != "point_mass" else 0.0, mond=1 if mond else 0,
                         mond_acc0=0.2, mond_nu_index=2.0)
    o.compute_force()
    assert rel_err(g["acc"], o.acc).max() <= 1e-12


def test_circular_orbits_in_attractor_field(nb, oracle):
    """Two massless particles on a circular orbit around a point-mass
    background field, constant-step leapfrog for one period (the setting of
    test/Local-Timestep.jl:726-760): the FP64 GPU run follows the oracle and
    keeps the radius."""
    GM, R = 1.0, 1.0
    v = np.sqrt(GM / R)
    T = 2 * np.pi * np.sqrt(R ** 3 / GM)
    d = {"pos": np.array([[R, 0, 0], [-R, 0, 0]], float),
         "vel": np.array([[0, v, 0], [0, -v, 0]], float), "mass": np.zeros(2)}
    dt = T / 2000
    sim = nb.Simulation(d, ForceSofteningTable=[1e-4] * 6, TimeStep=dt, TimeEnd=T, precision="fp64",
                        bgforce=nb.PointMassField(GM))
    nb.run(sim, nsteps=2000)
    g = nb.get_all_data(sim)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[1e-4] * 6, dt=dt, time_end=T,
                         bg_kind=1, bg_gm=GM)
    o.run_begin()
    o.step(2000)
    o.run_end()
    np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-12)
    r = np.linalg.norm(g["pos"], axis=1)
    assert np.abs(r - R).max() < 1e-5
    np.testing.assert_allclose(g["pos"], d["pos"], rtol=0, atol=1e-4)


def test_adaptive_mond_time_line_matches_oracle(nb, oracle):
    """Adaptive bins with MOND: the timestep criterion sees the post-processed
    accelerations, and the FP64 GPU time line equals the oracle's."""
    d = nb.plummer(1500, seed=72)
    h, T1 = 0.01, 0.05
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, TimeEnd=T1, MaxStep=1e-2, precision="fp64",
                        GravityModel=nb.MOND1983Milgrom, ACC0=0.3)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, time_end=T1, max_step=1e-2,
                         mond=1, mond_acc0=0.3, mond_nu_index=2.0)
    o.run_begin()
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    for _ in range(40):
        o.step(1)
        nb.step(sim, 1)
        assert sim.time()[0] == o.t_int
        if o.t_int >= 1 << 30:
            break
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
    np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-11)


def test_postprocessing_parameter_errors(nb):
    d = nb.plummer(64, seed=73)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, GravityModel=nb.MOND1983Milgrom, ACC0=0.0)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, bgforce=nb.PointMassField(float("nan")))
