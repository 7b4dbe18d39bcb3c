"""Failure detection on the GPU without a fault: the bounded mbarrier wait of
the force kernels runs out on a barrier that nothing completes, the error
word reports it, and the device context stays usable."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(nb):
    lib = nb.load()
    waited = ctypes.c_double()
    rc = lib.nb_selftest_wait_timeout(0, 50_000_000, ctypes.byref(waited))
    assert rc == nb._lib.NB_ERR_TIMEOUT
    assert 50.0 <= waited.value < 2000.0
    d = nb.plummer(1000, seed=91)
    sim = nb.Simulation(d, ForceSofteningTable=[0.01] * 6)
    nb.compute_force(sim)
    assert np.isfinite(nb.get_all_data(sim)["acc"]).all()


def test_selftest_rejects_bad_timeout(nb):
    lib = nb.load()
    assert lib.nb_selftest_wait_timeout(0, 0, None) == nb._lib.NB_ERR_INVALID_ARG
    assert lib.nb_selftest_wait_timeout(0, 3_000_000_000, None) == nb._lib.NB_ERR_INVALID_ARG
