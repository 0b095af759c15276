"""GPU parity of the real-time Green's functions (cmpy/exactdiag.py:248-316).

gf_greater / gf_lesser against golden vectors of the unmodified reference (same ground state
fed in), gf_tevo end to end, and fourier_t2z against the oracle's piecewise-linear Laplace
transform (gftool's default rule; gftool itself is absent)."""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu


def _model(tag, golden):
    from cmpy_gb300.models import ChainLattice, HubbardModel, SingleImpurityAndersonModel

    if tag == "chain4_U2":
        return HubbardModel(ChainLattice(4, False), inter=2.0, mu=1.0, hop=1.0)
    if tag == "chain6_U4":
        return HubbardModel(ChainLattice(6, False), inter=4.0, mu=2.0, hop=1.0)
    g = golden["coo"]
    return SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=g["siam_eps_bath"][:3], v=g["siam_v"][:3],
                                       temp=0.1)


@pytest.mark.parametrize("tag", ["chain4_U2", "chain6_U4", "siam3"])
def test_greater_lesser_vs_reference(cuda, golden, tag):
    from cmpy_gb300.exactdiag import EigenState, gf_greater, gf_lesser

    t = golden["tevo"]
    m = _model(tag, golden)
    nu, nd = (int(x) for x in t[f"{tag}_sector"])
    gs = EigenState(float(t[f"{tag}_e0"]), t[f"{tag}_state"], nu, nd)
    times = t[f"{tag}_times"]
    tt, gg = gf_greater(m, gs, times[0], times[-1], len(times), n_lev=None)
    _, gl = gf_lesser(m, gs, times[0], times[-1], len(times), n_lev=None)
    np.testing.assert_allclose(tt, times, rtol=0, atol=1e-14)
    assert np.max(np.abs(gg - t[f"{tag}_greater"])) < 1e-9
    assert np.max(np.abs(gl - t[f"{tag}_lesser"])) < 1e-9


def test_krylov_truncation_converges(cuda, golden):
    """A Krylov space much smaller than the sector reproduces short-time dynamics."""
    from cmpy_gb300.exactdiag import EigenState, gf_greater

    t = golden["tevo"]
    m = _model("chain6_U4", golden)
    gs = EigenState(float(t["chain6_U4_e0"]), t["chain6_U4_state"], 3, 3)
    times = t["chain6_U4_times"]
    _, gg = gf_greater(m, gs, times[0], times[-1], len(times), n_lev=120)  # target sector: 300 states
    assert np.max(np.abs(gg - t["chain6_U4_greater"])) < 1e-9


def test_gf_tevo_end_to_end(cuda, golden):
    from cmpy_gb300.exactdiag import compute_groundstate, gf_tevo

    t = golden["tevo"]
    m = _model("chain4_U2", golden)
    gs = compute_groundstate(m)
    assert (gs.n_up, gs.n_dn) == tuple(int(x) for x in t["chain4_U2_sector"])
    times, g = gf_tevo(m, 0.0, 20.0, 201)
    ref = t["chain4_U2_greater"] - t["chain4_U2_lesser"]
    assert np.max(np.abs(g - ref)) < 1e-9


def test_fourier_t2z_vs_oracle(cuda, golden):
    from cmpy_gb300.exactdiag import fourier_t2z

    t = golden["tevo"]
    times = t["chain4_U2_times"]
    gt = t["chain4_U2_greater"] - t["chain4_U2_lesser"]
    w = np.linspace(-6, 6, 301)
    z, gw = fourier_t2z(times, gt, w, delta=1e-3)
    assert np.allclose(z.imag, -np.log(1e-3) / times[-1])
    ref = O.laplace_lin(times, gt, z)
    assert np.max(np.abs(gw - ref)) < 1e-11 * max(1.0, np.max(np.abs(ref)))
    # trapezoidal rule
    _, gtr = fourier_t2z(times, gt, w, delta=1e-3, method="trapz")
    integrand = np.exp(1j * z[:, None] * times[None, :]) * gt[None, :]
    ref_tr = 0.5 * np.sum((integrand[:, 1:] + integrand[:, :-1]) * np.diff(times)[None, :], axis=1)
    assert np.max(np.abs(gtr - ref_tr)) < 1e-11 * max(1.0, np.max(np.abs(ref_tr)))


def test_fourier_small_frequency_branch(cuda):
    """|u h| < 1/4 takes the Taylor branch of phi1/phi2: still exact for linear samples."""
    from cmpy_gb300 import engine as E

    t = np.linspace(0.0, 2.0, 41)
    a, b = 0.5 + 0.1j, -0.3 + 0.2j
    z = np.array([1e-4 + 1e-3j, 0.3 + 0.01j, 3.0 + 0.5j])
    u, T = 1j * z, t[-1]
    ref = O.laplace_lin(t, a + b * t, z)
    out = E.laplace_t2z(t, a + b * t, z).cpu().numpy()
    assert np.max(np.abs(out - ref)) < 1e-13
    exact = a * (np.exp(u * T) - 1) / u + b * (T * np.exp(u * T) / u - (np.exp(u * T) - 1) / u**2)
    assert np.max(np.abs(out[1:] - exact[1:])) < 1e-11
