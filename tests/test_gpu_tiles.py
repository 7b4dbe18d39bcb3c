"""Every j-tile size and ring depth of the mixed force kernel against the oracle
(mixed-form bars: median relative force error <= 1e-6, p99 <= 1e-5, max <=
1e-4; potential median <= 1e-6), repeatable bit for bit, and agreeing with the
default tiles of 256 sources within the same bars."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILES = [(128, 3), (128, 4), (128, 6), (256, 3), (256, 4), (256, 6), (512, 3), (512, 4)]


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.linalg.norm(b, axis=-1)


@pytest.mark.parametrize("law", ["spline", "plummer"])
@pytest.mark.parametrize("shape", [(128, 1, 1), (128, 2, 4), (128, 2, 8)])
@pytest.mark.parametrize("tile", TILES)
def test_tile_and_stages_match_oracle(nb, oracle, law, shape, tile):
    n, h = 5000, 0.01
    d = nb.plummer(n, seed=61)
    block, ipt, js = shape
    tj, st = tile
    olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=block,
                        i_per_thread=ipt, j_split=js, tile_j=tj, stages=st)
    nb.compute_force(sim)
    g1 = nb.get_all_data(sim)["acc"]
    nb.compute_force(sim)
    np.testing.assert_array_equal(g1, nb.get_all_data(sim)["acc"])
    e = rel_err(g1, a_ref)
    assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-4
    # the potential variant (4-stage ring) on the same tiles
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
    assert np.median(ep) <= 1e-6 and np.quantile(ep, 0.99) <= 1e-5
    ref = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=block,
                        i_per_thread=ipt, j_split=js)
    nb.compute_force(ref)
    # two mixed forms differ by FP32 round-off of their own (largest where the
    # force cancels)
    er = rel_err(g1, nb.get_all_data(ref)["acc"])
    assert np.median(er) <= 1e-6 and er.max() <= 1e-4


@pytest.mark.parametrize("n", [1, 2, 127, 129, 511, 513, 1025])
def test_ragged_sizes_with_large_tiles(nb, oracle, n):
    """Partial tiles of 512 and of 128 sources (zero-mass padding far away)."""
    h = 0.01
    d = nb.plummer(n, seed=62) if n > 2 else {"pos": np.array([[0.1, 0.2, 0.3], [0.4, -0.1, 0.2]])[:n],
                                              "vel": np.zeros((n, 3)), "mass": np.full(n, 0.5)}
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h)
    for tj in (128, 512):
        sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", tile_j=tj,
                            block=128, i_per_thread=2, j_split=2)
        nb.compute_force(sim, want_potential=True)
        g = nb.get_all_data(sim)
        if n == 1:
            assert np.all(g["acc"] == 0.0) and g["pot"][0] == p_ref[0] == 0.0
            continue
        e = rel_err(g["acc"], a_ref)
        assert np.median(e) <= 1e-6 and e.max() <= 1e-4
        np.testing.assert_allclose(g["pot"], p_ref, rtol=1e-5)


def test_bad_tile_parameters_are_rejected(nb):
    d = nb.plummer(64, seed=63)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, tile_j=384)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, stages=5)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, j_split=9)
    with pytest.raises(nb.NbodyError):
        # the persistent work-list kernel reads tiles of 256 only
        nb.Simulation(d, ForceSofteningTable=[0.01] * 6, block=-1, tile_j=512)
