"""Force post-processing in the oracle (background field, Milgrom MOND)
against closed forms."""
import numpy as np
import pytest

from oracle import oracle


def _one(pos, **kw):
    pos = np.atleast_2d(np.asarray(pos, dtype=float))
    n = pos.shape[0]
    o = oracle.OracleSim(pos, np.zeros_like(pos), np.zeros(n), soft=[1e-3] * 6, **kw)
    o.compute_force()
    return o.acc


def test_point_mass_field_closed_form():
    GM, R = 3.0, 2.5
    a = _one([[R, 0.0, 0.0], [0.0, -R, 0.0]], bg_kind=1, bg_gm=GM)
    np.testing.assert_allclose(a[0], [-GM / R ** 2, 0.0, 0.0], rtol=1e-15, atol=0)
    np.testing.assert_allclose(a[1], [0.0, GM / R ** 2, 0.0], rtol=1e-15, atol=0)
    # off-centre attractor
    a = _one([[1.0, 2.0, 3.0]], bg_kind=1, bg_gm=GM, bg_center=(1.0, 2.0, 1.0))
    np.testing.assert_allclose(a[0], [0.0, 0.0, -GM / 4.0], rtol=1e-15, atol=0)


def test_pseudo_newtonian_field_closed_form():
    GM, rg, R = 1.0, 0.1, 1.0
    a = _one([[0.0, 0.0, R]], bg_kind=2, bg_gm=GM, bg_rg=rg)
    np.testing.assert_allclose(a[0], [0.0, 0.0, -GM / (R - rg) ** 2], rtol=1e-15, atol=0)


@pytest.mark.parametrize("nu_index", [1.0, 2.0, 3.5])
def test_milgrom_mond_scaling(nu_index):
    GM, acc0 = 1.0, 0.05
    radii = np.array([0.3, 1.0, 4.0, 30.0])
    pos = np.stack([radii, np.zeros(4), np.zeros(4)], 1)
    a = _one(pos, bg_kind=1, bg_gm=GM, mond=1, mond_acc0=acc0, mond_nu_index=nu_index)
    an = GM / radii ** 2
    y = an / acc0
    nu = (0.5 * (1.0 + np.sqrt(1.0 + 4.0 * y ** -nu_index))) ** (1.0 / nu_index)
    np.testing.assert_allclose(-a[:, 0], an * nu, rtol=1e-14)
    if nu_index == 2.0:
        # deep-MOND limit a -> sqrt(a_N ACC0), Newtonian limit a -> a_N
        assert abs(-a[3, 0] / np.sqrt(an[3] * acc0) - 1) < 1e-2
        assert abs(-a[0, 0] / an[0] - 1) < 1e-3


def test_mond_keeps_zero_acceleration():
    a = _one([[0.0, 0.0, 0.0]], mond=1, mond_acc0=1.0)
    assert np.all(a == 0.0)
