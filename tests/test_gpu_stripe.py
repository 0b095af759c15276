"""GPU parity of the two-pass stripe fixed-point matvec (variant 6).

* on every benchmark-like sector its integer H·x equals the single-pass kernel's (variant 3)
  bit for bit, and the oracle's integer matrix on small sectors, with exact and rounded
  (arbitrary on-site energy) diagonals and open and periodic chains;
* a Lanczos run in its renumbered basis (states sorted by hop count) gives the same
  coefficients and ground state as the single-pass run, and the 12-site ring's ground-state
  energy measured on the reference; its Ritz vector is an eigenvector in the sector's order;
* the 14-site ring's ground-state energy equals the oracle's eigsh value;
* the particle-sector continued-fraction coefficients (lanczos_coeffs from c^dag psi) equal the
  single-pass ones.
"""

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import ed_oracle as O
from test_gpu_sweep import CASES, _hub, _rand_mantissas

pytestmark = pytest.mark.gpu


def _with_variant(p, v):
    p.set_matvec_variant(v)
    assert p.matvec_variant == v


@pytest.mark.parametrize("name,mk,sec", CASES, ids=[c[0] for c in CASES])
def test_stripe_bitexact_vs_single_pass(cuda, name, mk, sec):
    p = mk().plan(*sec)
    xm = _rand_mantissas(p, 9)
    try:
        _with_variant(p, 3)
        w3, e3 = p.matvec_fixed(xm, -10)
        _with_variant(p, 6)
        w6, e6 = p.matvec_fixed(xm, -10)
    finally:
        p.set_matvec_variant(0)
    assert e6 == e3
    assert torch.equal(w6, w3), (name, int((w6 != w3).sum()))


@pytest.mark.parametrize("nu,nd,periodic", [(3, 3, True), (2, 4, True), (4, 1, True), (3, 5, False), (1, 1, False)])
def test_stripe_vs_oracle_integer_matrix(cuda, nu, nd, periodic):
    """Dyadic sector (t = 1/2, U = 3): the integer matvec equals the oracle's H * 2^F, on
    periodic and open chains (8 choose 4 = 70 states: a ragged last stripe)."""
    m = _hub(8, periodic, inter=3.0, mu=1.5, hop=0.5)
    p = m.plan(nu, nd)
    _with_variant(p, 6)
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(8, nu), O.sector_states(8, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    F = 1
    D = len(up) * len(dn)
    A = sp.csr_matrix((np.ldexp(v, F).astype(np.int64), (c, r)), shape=(D, D))
    x = np.random.default_rng(nu * 10 + nd).integers(-(1 << 40), 1 << 40, size=D)
    wm, ew = p.matvec_fixed(torch.as_tensor(x).cuda(), 0)
    p.set_matvec_variant(0)
    assert ew == -F
    assert np.array_equal(wm.cpu().numpy(), A @ x)


def test_stripe_odd_dimensions_vs_single_pass(cuda):
    """Sectors whose num_up and num_dn are odd and not multiples of 4 (9 sites: 9 choose 4 =
    126, 9 choose 3 = 84, 9 choose 2 = 36; 7 sites: 35, 21): the 8-byte copy path and the
    ragged last stripes of both passes."""
    for n_sites, sec in ((9, (4, 3)), (9, (2, 4)), (7, (3, 2)), (7, (4, 4))):
        p = _hub(n_sites, True, inter=4.0, mu=2.0).plan(*sec)
        xm = _rand_mantissas(p, 3)
        try:
            p.set_matvec_variant(3)
            w_ref, e_ref = p.matvec_fixed(xm, 0)
            _with_variant(p, 6)
            w6, e6 = p.matvec_fixed(xm, 0)
        finally:
            p.set_matvec_variant(0)
        assert e6 == e_ref
        assert torch.equal(w6, w_ref), (n_sites, sec)


def test_stripe_lanczos_matches_single_pass(cuda):
    from cmpy_gb300 import engine as E

    p = _hub(12, True, inter=4.0, mu=2.0).plan(6, 6)
    g = torch.Generator(device="cuda").manual_seed(12)
    v0 = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    kw = dict(max_steps=200, want_vector=True, v0=v0, tol=1e-12, check_every=10)
    r3 = E.lanczos(p, **kw)
    try:
        _with_variant(p, 6)
        r6 = E.lanczos(p, **kw)
        hv = p.matvec(r6.vector)
    finally:
        p.set_matvec_variant(0)
    assert r6.steps == r3.steps
    # before the ground state converges the runs agree to rounding of the dot products
    np.testing.assert_allclose(r6.alpha[:60].cpu().numpy(), r3.alpha[:60].cpu().numpy(), rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(r6.beta[:61].cpu().numpy(), r3.beta[:61].cpu().numpy(), rtol=1e-11, atol=1e-11)
    assert abs(r6.energy - r3.energy) <= 1e-12 * abs(r3.energy)
    assert abs(r6.energy - (-30.920353562419)) <= 1e-10 * 30.92
    torch.testing.assert_close(r6.vector, r3.vector, rtol=0, atol=1e-9)
    assert torch.linalg.norm(hv - r6.energy * r6.vector).item() < 1e-7


def test_stripe_ring14_energy_vs_oracle(cuda, golden):
    from cmpy_gb300 import engine as E

    p = _hub(14, True, inter=4.0, mu=2.0).plan(7, 7)
    try:
        _with_variant(p, 6)
        r = E.lanczos(p, max_steps=250, want_vector=False)
    finally:
        p.set_matvec_variant(0)
    e_ref = float(golden["bench_e0"]["ring14_77_U4_e0"])
    assert abs(r.energy - e_ref) <= 1e-10 * abs(e_ref)


def test_stripe_gf_coefficients_match_single_pass(cuda):
    """Continued-fraction coefficients of the particle sector (8,7) of the 14-site ring from a
    seeded start vector: the renumbered run gives the single-pass coefficients."""
    from cmpy_gb300 import engine as E

    p = _hub(14, True, inter=4.0, mu=2.0).plan(8, 7)
    g = torch.Generator(device="cuda").manual_seed(4)
    s = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    a3, b3, _ = E.lanczos_coeffs(p, s, max_steps=40)
    try:
        _with_variant(p, 6)
        a6, b6, _ = E.lanczos_coeffs(p, s, max_steps=40)
    finally:
        p.set_matvec_variant(0)
    # the dot products are exact; only the FP64 sum of the per-CTA partials is grouped
    # differently, and 40 steps from a random start amplify that little
    np.testing.assert_allclose(a6.cpu().numpy(), a3.cpu().numpy(), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(b6.cpu().numpy(), b3.cpu().numpy(), rtol=1e-10, atol=1e-10)


def test_coefficient_runs_interleaved_equal_separate(cuda):
    """ed_lanczos_coeffs_multi: the particle and hole runs of the 14-site ground-state Green's
    function (sectors (8,7) and (6,7)) with interleaved steps give exactly the coefficients of
    separate runs; so do an FP64 plan (non-dyadic t) mixed in and a zero start vector."""
    from cmpy_gb300 import engine as E

    m = _hub(14, True, inter=4.0, mu=2.0)
    pp, pm = m.plan(8, 7), m.plan(6, 7)
    g = torch.Generator(device="cuda").manual_seed(8)
    s1 = torch.rand(pp.dim, dtype=torch.float64, device="cuda", generator=g)
    s2 = torch.rand(pm.dim, dtype=torch.float64, device="cuda", generator=g)
    sep = [E.lanczos_coeffs(pp, s1, max_steps=60), E.lanczos_coeffs(pm, s2, max_steps=60)]
    mult = E.lanczos_coeffs_multi([(pp, s1), (pm, s2)], max_steps=60)
    for (a, b, n), (a2, b2, n2) in zip(sep, mult):
        assert torch.equal(a, a2) and torch.equal(b, b2) and n == n2
    small = _hub(8, True, inter=4.0, mu=2.0, hop=0.7).plan(4, 4)  # no integer matvec
    z = torch.zeros(small.dim, dtype=torch.float64, device="cuda")
    s3 = torch.rand(small.dim, dtype=torch.float64, device="cuda", generator=g)
    out = E.lanczos_coeffs_multi([(small, s3), (small, z)], max_steps=40)
    ref = E.lanczos_coeffs(small, s3, max_steps=40)
    assert torch.equal(out[0][0], ref[0]) and torch.equal(out[0][1], ref[1])
    assert out[1][0].numel() == 0 and out[1][2] == 0.0
