"""Device-state checkpoint / restart (nb_checkpoint_*; saverestart and
loadrestart of src/restart.jl for (DirectSum, GPU))."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(nb, sim):
    g = nb.get_all_data(sim)
    return g, sim.time(), nb.counters(sim)


def _assert_same(a, b):
    ga, ta, ca = a
    gb, tb, cb = b
    for k in ("pos", "vel", "acc", "pot", "ti_begstep", "ti_endstep"):
        np.testing.assert_array_equal(ga[k], gb[k], err_msg=k)
    assert ta == tb


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_adaptive_run_resumes_bit_identically(nb, tmp_path, precision):
    d = nb.plummer(3000, seed=51)
    d["collection"] = np.where(np.arange(3000) % 3 == 0, 2, 1).astype(np.int32)
    kw = dict(ForceSofteningTable=[0.01, 0.02, 0.01, 0.01, 0.01, 0.01], TimeEnd=0.2,
              MaxStep=1e-2, precision=precision)
    sim = nb.Simulation(d, **kw)
    nb.compute_force(sim)
    nb.init_timesteps(sim)
    nb.leapfrog_half_kick(sim, +1)
    nb.step(sim, 12)
    path = tmp_path / "restart.0.nbgb300"
    nb.saverestart(sim, str(path))
    nb.step(sim, 15)
    ref = _state(nb, sim)
    sim2 = nb.loadrestart(str(path))
    assert sim2.n == 3000 and sim2.adaptive and sim2.TimeEnd == 0.2
    np.testing.assert_array_equal(sim2.collection, d["collection"])
    nb.step(sim2, 15)
    _assert_same(ref, _state(nb, sim2))
    # energy diagnostics read the restored masses and softening
    assert nb.total_energy(sim2) == pytest.approx(nb.total_energy(sim), rel=0, abs=0)


def test_restore_into_handle_of_other_size_and_shape(nb):
    """An image loads into a handle that holds another system with another
    launch shape (j_split 2): parameters, shape and arena follow the image."""
    d = nb.plummer(2500, seed=52)
    a = nb.Simulation(d, ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, TimeEnd=1.0,
                      block=128, i_per_thread=1, j_split=2)
    nb.run(a, nsteps=5)
    img = a.checkpoint()
    nb.step(a, 7)
    ref = _state(nb, a)
    b = nb.Simulation(nb.plummer(6000, seed=53), ForceSofteningTable=[0.05] * 6, precision="fp64")
    nb.compute_force(b)
    b.restore(img)
    assert b.n == 2500 and not b.adaptive and b.TimeStep == 1e-3
    nb.step(b, 7)
    _assert_same(ref, _state(nb, b))


def test_bad_images_are_rejected(nb):
    d = nb.plummer(500, seed=54)
    a = nb.Simulation(d, ForceSofteningTable=[0.01] * 6)
    img = bytearray(a.checkpoint())
    b = nb.Simulation(d, ForceSofteningTable=[0.01] * 6)
    with pytest.raises(nb.NbodyError):
        b.restore(bytes(img[:-8]))
    bad = bytearray(img)
    bad[0:8] = b"XXXXXXXX"
    with pytest.raises(nb.NbodyError):
        b.restore(bytes(bad))
    # the handle still works after the rejected loads
    nb.compute_force(b)


def test_image_with_a_bad_source_order_loads_and_resorts(nb):
    """The image keeps the step graphs' Morton permutation so that a restored
    run continues bit-identically; a block that is not a permutation of
    0..n-1 is dropped at load (the next step sorts again) instead of being
    gathered through."""
    n = 500
    d = nb.plummer(n, seed=55)
    kw = dict(ForceSofteningTable=[0.01] * 6, TimeStep=1e-3, TimeEnd=1.0, precision="mixed")
    a = nb.Simulation(d, **kw)
    nb.run(a, nsteps=3)
    nb.step(a, 2)
    img = bytearray(a.checkpoint())
    perm = np.frombuffer(bytes(img[-4 * n:]), dtype=np.int32)
    assert sorted(perm.tolist()) == list(range(n))
    for bad_value in (n, -1, int(perm[1])):
        bad = bytearray(img)
        bad[-4 * n:-4 * n + 4] = np.int32(bad_value).tobytes()
        b = nb.Simulation(d, **kw)
        b.restore(bytes(bad))
        nb.step(b, 4)
        g = nb.get_all_data(b)
        assert np.all(np.isfinite(g["pos"])) and np.all(np.isfinite(g["acc"]))
