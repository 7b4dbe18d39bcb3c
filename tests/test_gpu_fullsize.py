"""Size-independent properties of the force at the bench size (Plummer
N = 2^20, eps = 1e-3, mixed precision), where the oracle is too slow to
compare every particle: exact scaling with the masses, momentum balance
(Newton's third law), symmetry under a right-angle rotation, and agreement
with the oracle on a seeded subsample."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 20
EPS = 1e-3


@pytest.fixture(scope="module")
def big(nb):
    d = nb.plummer(N, seed=2)
    sim = nb.Simulation(d, ForceSofteningTable=[EPS] * 6, TimeStep=1e-4, precision="mixed")
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    sim.close()
    return d, g


def test_doubling_every_mass_doubles_every_force_exactly(nb, big):
    d, g = big
    d2 = dict(d, mass=2.0 * d["mass"])
    sim = nb.Simulation(d2, ForceSofteningTable=[EPS] * 6, TimeStep=1e-4, precision="mixed")
    nb.compute_force(sim, want_potential=True)
    g2 = nb.get_all_data(sim)
    np.testing.assert_array_equal(g2["acc"], 2.0 * g["acc"])
    np.testing.assert_array_equal(g2["pot"], 2.0 * g["pot"])


def test_momentum_balance(big):
    d, g = big
    m = d["mass"][:, None]
    net = np.abs((m * g["acc"]).sum(0))
    scale = (m * np.abs(g["acc"])).sum(0)
    assert (net / scale).max() <= 1e-6


def test_right_angle_rotation(nb, big):
    """(x, y, z) -> (-y, x, z) maps the force the same way, to FP32 round-off
    (the rotated system is Morton-sorted into other tiles)."""
    d, g = big
    p = d["pos"]
    rot = np.stack([-p[:, 1], p[:, 0], p[:, 2]], 1)
    sim = nb.Simulation(dict(d, pos=rot), ForceSofteningTable=[EPS] * 6, TimeStep=1e-4,
                        precision="mixed")
    nb.compute_force(sim)
    a = nb.get_all_data(sim)["acc"]
    expect = np.stack([-g["acc"][:, 1], g["acc"][:, 0], g["acc"][:, 2]], 1)
    e = np.linalg.norm(a - expect, axis=1) / np.linalg.norm(expect, axis=1)
    assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5


def test_subsample_against_oracle(oracle, big):
    d, g = big
    sub = np.random.default_rng(77).choice(N, size=512, replace=False)
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"][sub], EPS)
    e = np.linalg.norm(g["acc"][sub] - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5
    assert np.median(np.abs(g["pot"][sub] - p_ref) / np.abs(p_ref)) <= 1e-6
