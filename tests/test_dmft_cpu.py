"""DMFT drivers on the CPU: the two-site scheme with Lange's analytic impurity solver
(cmpy/dmft/twosite.py:25-172) against the published two-site result z_qp = 1 - U^2/36
(M. Potthoff, two-site DMFT of the half-filled Bethe lattice, t = 1), the helpers of
cmpy/dmft/utils.py, and the analytic hybridisation fit."""

import numpy as np
import pytest

from cmpy_gb300 import dmft


def test_helpers():
    g0 = np.array([1.0 + 2j, -0.5 + 0.1j])
    g = np.array([0.3 - 1j, 2.0 + 0.5j])
    np.testing.assert_allclose(dmft.self_energy(g0, g), 1 / g0 - 1 / g)
    assert dmft.mix_values(1.0, 3.0) == 3.0
    assert dmft.mix_values(1.0, 3.0, mixing=0.25) == pytest.approx(1.5)
    w = np.linspace(-0.5, 0.5, 101)
    assert dmft.quasiparticle_weight(w, -2.0 * w + 0.3j) == pytest.approx(1 / 3)
    assert dmft.quasiparticle_weight(w, -1e6 * w) == 0
    a1, a2, e1, e2 = dmft.impurity_params_ref(3.0, 0.7)
    assert 2 * (a1 + a2) == pytest.approx(1.0)
    assert 0 < e1 < e2


def test_bethe_dos_normalised():
    t = 1.0
    w = np.linspace(-2.5, 2.5, 200001)
    g = dmft.bethe_gf_omega(w + 1e-9j, t)
    dos = -g.imag / np.pi
    integral = np.sum(0.5 * (dos[1:] + dos[:-1]) * np.diff(w))
    assert integral == pytest.approx(1.0, abs=2e-4)
    assert dos.min() >= -1e-12


@pytest.mark.parametrize("u", [0.5, 2.0, 3.0, 4.0, 5.0])
def test_twosite_reference_solver_matches_potthoff(u):
    z = np.linspace(-10, 10, 20001) + 1e-3j
    siam = dmft.twosite_dmft_half_filling(z, u, t=1.0, verbose=False, ref=True, max_iter=2000)
    assert siam.stats.success
    assert siam.v[0] ** 2 == pytest.approx(1 - u**2 / 36, abs=2e-5)


def test_twosite_insulator_beyond_uc():
    z = np.linspace(-10, 10, 20001) + 1e-3j
    siam = dmft.twosite_dmft_half_filling(z, 6.5, t=1.0, verbose=False, ref=True, max_iter=2000)
    assert siam.v[0] < 1e-2


def test_fit_hybridization_recovers_bath():
    beta = 40.0
    iwn = 1j * (2 * np.arange(200) + 1) * np.pi / beta
    eb_true = np.array([-1.1, 0.2, 0.9])
    v_true = np.array([0.4, 0.25, 0.5])
    target = np.sum(v_true**2 / (iwn[:, None] - eb_true[None, :]), axis=1)
    eb, v, loss = dmft.fit_hybridization(iwn, target, eb_true + np.array([0.2, -0.1, 0.15]), v_true * 1.2)
    assert loss < 1e-16
    order = np.argsort(eb)
    np.testing.assert_allclose(eb[order], eb_true, atol=1e-6)
    np.testing.assert_allclose(v[order], v_true, atol=1e-6)
