"""CPU tests of the seeded initial-condition generators (the input spec that the
GPU path and the oracle both consume)."""
import numpy as np


def test_plummer_profile_and_virial(nb, oracle):
    d = nb.plummer(200000, seed=1)
    r = np.linalg.norm(d["pos"], axis=1)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.3048 a
    assert abs(np.median(r) - 1.3048) < 0.02
    assert abs(d["mass"].sum() - 1.0) < 1e-12
    np.testing.assert_allclose((d["mass"][:, None] * d["vel"]).sum(0), 0.0, atol=1e-15)
    s = nb.plummer(3000, seed=2)
    o = oracle.OracleSim(s["pos"], s["vel"], s["mass"], soft=[1e-4] * 6)
    o.compute_potential()
    e = o.diagnostics()
    assert abs(-2 * e["K"] / e["W"] - 1.0) < 0.1  # virial equilibrium


def test_hernquist_profile_and_energy(nb):
    d = nb.hernquist(300000, seed=3)
    r = np.linalg.norm(d["pos"], axis=1)
    assert r.max() <= 100.0 * 1.01 + 1.0
    # truncated at 100 a: half-mass radius (0.99/2) solves r^2/(r+1)^2 = 0.98/2
    assert abs(np.median(r) - 2.33) < 0.05
    k = 0.5 * np.mean(np.sum(d["vel"] ** 2, axis=1))
    assert abs(k - 1.0 / 12.0) < 0.01  # kinetic energy per unit mass of the model


def test_generators_are_seeded(nb):
    for gen in (nb.plummer, nb.hernquist):
        a, b, c = gen(500, seed=9), gen(500, seed=9), gen(500, seed=10)
        np.testing.assert_array_equal(a["pos"], b["pos"])
        np.testing.assert_array_equal(a["vel"], b["vel"])
        assert not np.array_equal(a["pos"], c["pos"])


def test_collision_setup(nb):
    d = nb.collision(2000, seed=4, separation=20.0)
    assert d["pos"].shape == (4000, 3)
    c1 = d["pos"][:2000].mean(0)
    c2 = d["pos"][2000:].mean(0)
    np.testing.assert_allclose(np.linalg.norm(c2 - c1), 20.0, rtol=0.05)
    vrel = d["vel"][2000:].mean(0) - d["vel"][:2000].mean(0)
    np.testing.assert_allclose(np.linalg.norm(vrel), np.sqrt(2 * 2 / 20.0), rtol=0.05)


def test_request_stream(nb):
    s = nb.RequestStream(rate=200.0, seed=5, pool_size=1, n_max=4096)
    reqs = [s.next() for _ in range(2000)]
    gaps = np.diff([0.0] + [q["arrival"] for q in reqs])
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0
    ns = np.array([q["n"] for q in reqs])
    assert ns.min() >= 256 and ns.max() <= 4096
    sys0 = s.system(reqs[0])
    assert sys0["pos"].shape == (reqs[0]["n"], 3)
    np.testing.assert_allclose(sys0["mass"].sum(), 1.0)
