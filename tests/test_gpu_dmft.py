"""DMFT drivers with the GPU impurity solver.

* The ED impurity Green's function of the half-filled two-site SIAM at T = 0 equals E. Lange's
  analytic result used by the reference (cmpy/dmft/twosite.py:25-84) — a known answer;
* the two-site DMFT loop driven by the ED solver converges to the same hybridisation as the
  analytic loop;
* the adjoint bath fit reproduces the interacting Green's function of a SIAM;
* the multi-bath Matsubara loop reaches self-consistency with the correct high-frequency tail.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("u,v", [(1.0, 0.8), (3.0, 0.9), (5.0, 0.4)])
def test_two_site_ed_equals_lange(cuda, u, v):
    from cmpy_gb300 import dmft
    from cmpy_gb300.models import SingleImpurityAndersonModel

    z = np.linspace(-6, 6, 301) + 0.05j
    siam = SingleImpurityAndersonModel(u, v=[v], mu=u / 2, temp=0.0)
    g_ed = dmft.compute_impurity_gf(z, siam, ref=False)
    g_ref = dmft.impurity_gf_ref(z, u, v)
    assert np.max(np.abs(g_ed - g_ref)) < 1e-10


def test_two_site_loop_ed_matches_analytic(cuda):
    from cmpy_gb300 import dmft

    z = np.linspace(-10, 10, 4001) + 1e-3j
    a = dmft.twosite_dmft_half_filling(z, 3.0, t=1.0, verbose=False, ref=True, max_iter=500)
    b = dmft.twosite_dmft_half_filling(z, 3.0, t=1.0, verbose=False, ref=False, max_iter=500)
    assert b.stats.success
    assert abs(a.v[0] - b.v[0]) < 1e-6


def test_adjoint_bath_fit_matches_target_gf(cuda):
    from cmpy_gb300 import dmft
    from cmpy_gb300.adjoint import greens_function_ad

    beta = 20.0
    iwn = 1j * (2 * np.arange(48) + 1) * np.pi / beta
    u = 3.0
    eb_true = np.array([-1.0, 0.1, 1.2])
    v_true = np.array([0.5, 0.35, 0.45])
    theta, ns, bonds, width = dmft._bath_theta(torch.tensor(eb_true, device="cuda"),
                                               torch.tensor(v_true, device="cuda"), u, u / 2)
    with torch.no_grad():
        target = greens_function_ad(theta, ns, bonds, (2, 2), iwn, sign_width=width, gs_steps=200, gf_levels=120)
    eb, v, hist = dmft.fit_impurity_gf(iwn, target.cpu().numpy(), u, eb_true + np.array([0.15, -0.1, -0.1]),
                                       v_true * 1.15, steps=40)
    # the loss falls by orders of magnitude and the fitted bath reproduces the target G (the
    # bath itself is not identifiable from 48 Matsubara points: nearby baths give nearly the same G)
    assert hist[-1] < 1e-4 * hist[0]
    theta, ns, bonds, width = dmft._bath_theta(torch.tensor(eb, device="cuda"), torch.tensor(v, device="cuda"),
                                               u, u / 2)
    with torch.no_grad():
        g_fit = greens_function_ad(theta, ns, bonds, (2, 2), iwn, sign_width=width, gs_steps=200, gf_levels=120)
    assert torch.max(torch.abs(g_fit - target)).item() < 3e-3 * torch.max(torch.abs(target)).item()


def test_multibath_matsubara_loop(cuda):
    from cmpy_gb300 import dmft

    res = dmft.dmft_bethe_matsubara(2.0, t=1.0, num_bath=5, beta=40.0, n_mats=128, max_iter=12, tol=1e-5)
    errs = np.asarray(res.stats.history).reshape(-1)
    assert errs[-1] < errs[0]
    iwn = 1j * (2 * np.arange(128) + 1) * np.pi / 40.0
    # high-frequency tail of a normalised Green's function: i w_n G(i w_n) -> 1
    assert abs(iwn[-1] * res.g_loc[-1] - 1.0) < 2e-2
    assert abs(iwn[-1] * res.g_imp[-1] - 1.0) < 2e-2
    # a metal at U = 2: the quasiparticle weight from the lowest Matsubara frequency is in (0, 1)
    z0 = 1.0 / (1.0 - res.sigma[0].imag / iwn[0].imag)
    assert 0.3 < z0 < 1.0
