"""Real-time Green's functions and their Laplace transform: the oracle against the reference.

gf_greater / gf_lesser (cmpy/exactdiag.py:248-301) golden vectors come from the unmodified
reference (scipy expm_multiply inside), with the ground state it used stored beside them.
fourier_t2z (exactdiag.py:311-316) calls gftool.fourier.tt2z, which is not installed: its
rule (exact integral of the piecewise-linear interpolant) is pinned by known answers here.
"""

import numpy as np
import pytest

from oracle import ed_oracle as O

CASES = {
    "chain4_U2": (4, lambda g: O.hubbard_descriptor(4, [[i, i + 1] for i in range(3)], inter=2.0, mu=1.0, hop=1.0)),
    "chain6_U4": (6, lambda g: O.hubbard_descriptor(6, [[i, i + 1] for i in range(5)], inter=4.0, mu=2.0, hop=1.0)),
    "siam3": (4, lambda g: O.siam_descriptor(4.0, 0.0, g["coo"]["siam_eps_bath"][:3], g["coo"]["siam_v"][:3])),
}


def dense(n_sites, desc, nu, nd):
    eps, u, bonds, width = desc
    up, dn = O.sector_states(n_sites, nu), O.sector_states(n_sites, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    return O.dense_from_coo(len(up) * len(dn), r, c, v), up, dn


@pytest.mark.parametrize("tag", list(CASES))
def test_gf_time_dense_matches_reference(golden, tag):
    t = golden["tevo"]
    n_sites, mk = CASES[tag]
    desc = mk(golden)
    nu, nd = (int(x) for x in t[f"{tag}_sector"])
    e0, psi, times = float(t[f"{tag}_e0"]), t[f"{tag}_state"], t[f"{tag}_times"]
    _, up, dn = dense(n_sites, desc, nu, nd)
    for greater, key, dnu in ((True, "greater", 1), (False, "lesser", -1)):
        Ht, upt, dnt = dense(n_sites, desc, nu + dnu, nd)
        phi = O.apply_fermion(up, dn, upt, dnt, 0, 1, greater, psi)
        g = O.gf_time_dense(Ht, phi, e0, times, greater)
        assert np.max(np.abs(g - t[f"{tag}_{key}"])) < 1e-10, (tag, key)


def test_laplace_lin_exact_for_linear_samples():
    rng = np.random.default_rng(3)
    t = np.sort(np.concatenate([[0.0, 4.0], rng.uniform(0, 4, 30)]))
    a, b = 0.3 - 0.2j, 1.1 + 0.4j
    z = np.array([0.7 + 0.3j, -1.2 + 0.05j, 0.2 + 0.01j, 25.0 + 0.1j, -3.0 + 2.0j])
    u, T = 1j * z, t[-1]
    exact = a * (np.exp(u * T) - 1) / u + b * (T * np.exp(u * T) / u - (np.exp(u * T) - 1) / u**2)
    np.testing.assert_allclose(O.laplace_lin(t, a + b * t, z), exact, rtol=1e-12, atol=1e-13)


def test_laplace_lin_converges_quadratically():
    """g(t) = -i e^{-i eps t}: the integral of the interpolant converges as h^2."""
    eps = 0.7
    z = np.array([0.5 + 0.2j, -1.0 + 0.3j])
    T = 10.0
    u = 1j * z
    exact = -1j * (np.exp((u - 1j * eps) * T) - 1) / (u - 1j * eps)
    errs = []
    for n in (201, 401, 801):
        t = np.linspace(0, T, n)
        errs.append(np.max(np.abs(O.laplace_lin(t, -1j * np.exp(-1j * eps * t), z) - exact)))
    assert errs[0] / errs[1] == pytest.approx(4.0, rel=0.05)
    assert errs[1] / errs[2] == pytest.approx(4.0, rel=0.05)
