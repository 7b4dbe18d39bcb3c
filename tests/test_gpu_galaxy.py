"""Real-data parity: a subsample of the reference's Gadget-2 collision fixture
(halo + disk galaxy, kpc / km/s / 1e10 Msun, G in those units, softening
0.4 kpc as in examples/04-collisions/04-collisions.jl:73)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "galaxy_subsample.npz")
H = 0.4


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


@pytest.fixture(scope="module")
def galaxy():
    z = np.load(GOLDEN)
    return {k: z[k] for k in ("pos", "vel", "mass", "collection")}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_galaxy_force_and_potential_vs_oracle(nb, oracle, galaxy, precision):
    G = nb.internal_G()
    sim = nb.Simulation(galaxy, G=G, ForceSofteningTable=[H] * 6, precision=precision)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    a_ref, p_ref = oracle.force(galaxy["pos"], galaxy["mass"], galaxy["pos"], H, G=G)
    e = rel_err(g["acc"], a_ref)
    ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
    if precision == "fp64":
        assert e.max() <= 1e-12 and ep.max() <= 1e-12
    else:
        assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-4
        assert np.median(ep) <= 1e-6


def test_galaxy_adaptive_time_line_matches_oracle(nb, oracle, galaxy):
    """FP64 adaptive run of the galaxy (power-of-two bins, eta = 0.025,
    MaxStep 1e-3 time units): same integer time line and bins as the oracle."""
    G = nb.internal_G()
    T1 = 0.004
    o = oracle.OracleSim(galaxy["pos"], galaxy["vel"], galaxy["mass"], ptype=galaxy["collection"],
                         soft=[H] * 6, G=G, time_end=T1, max_step=1e-3, min_step=1e-9)
    o.run_begin()
    sim = nb.Simulation(galaxy, G=G, ForceSofteningTable=[H] * 6, TimeEnd=T1, MaxStep=1e-3,
                        MinStep=1e-9, precision="fp64")
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    for _ in range(40):
        o.step(1)
        nb.step(sim, 1)
        ti, _ = sim.time()
        assert ti == o.t_int
        if ti >= 1 << 30:
            break
    g = nb.get_all_data(sim)
    np.testing.assert_array_equal(g["ti_endstep"], o.ti_end)
    np.testing.assert_allclose(g["pos"], o.pos, rtol=0, atol=1e-9)


def test_write_snapshot_round_trip(nb, galaxy, tmp_path):
    sim = nb.Simulation(galaxy, G=nb.internal_G(), ForceSofteningTable=[H] * 6, TimeStep=1e-4,
                        TimeEnd=1e-3)
    nb.run(sim, nsteps=3)
    p = tmp_path / "snap_000.gadget2"
    nb.write_snapshot(sim, str(p))
    h, r = nb.read_gadget2(str(p))
    g = nb.get_all_data(sim)
    assert h["Npart"] == [0, int((galaxy["collection"] == 2).sum()),
                          int((galaxy["collection"] == 3).sum()), 0, 0, 0]
    assert abs(h["Time"] - sim.time()[1]) == 0.0
    np.testing.assert_array_equal(r["pos"], g["pos"].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(r["vel"], g["vel"].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(r["mass"], galaxy["mass"])
