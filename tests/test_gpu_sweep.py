"""GPU parity of the banded two-pass fixed-point matvec (variant 5, the "sweep").

* it is available on the benchmark sectors (the plans choose a faster single-pass variant by
  default) and its integer H·x equals variant 3's bit for bit, and the oracle's integer matrix on small sectors, for exact and
  rounded (arbitrary on-site energy) diagonals;
* a Lanczos run in its renumbered basis gives the same coefficients and ground state as the
  single-pass run, and the 12-site ring's ground-state energy measured on the reference;
* a first wait that gives up (wait limit -1: no polling) reports ED_ERR_TIMEOUT, and the next
  call on the plan succeeds.
"""

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu


def _hub(N, periodic, **kw):
    from cmpy_gb300.models import ChainLattice, HubbardModel

    return HubbardModel(ChainLattice(N, periodic), **kw)


def _rand_mantissas(p, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    lim = 1 << (p.fixed_point - 1)
    return torch.randint(-lim, lim, (p.dim,), dtype=torch.int64, device="cuda", generator=g)


CASES = [
    ("ring14_77", lambda: _hub(14, True, inter=4.0, mu=2.0), (7, 7)),
    ("ring14_87", lambda: _hub(14, True, inter=4.0, mu=2.0), (8, 7)),
    ("ring12_66", lambda: _hub(12, True, inter=4.0, mu=2.0), (6, 6)),
    ("ring10_55_U6", lambda: _hub(10, True, inter=6.0, mu=3.0), (5, 5)),
    ("chain8_dis_44", lambda: _hub(8, False, inter=4.0, eps=np.random.default_rng(3).uniform(-1, 1, 8), mu=2.0), (4, 4)),
    ("chain8_dis_25", lambda: _hub(8, False, inter=4.0, eps=np.random.default_rng(4).uniform(-1, 1, 8), mu=2.0), (2, 5)),
    ("ring10_t05_46", lambda: _hub(10, True, inter=3.0, mu=1.5, hop=0.5), (4, 6)),
]


@pytest.mark.parametrize("name,mk,sec", CASES, ids=[c[0] for c in CASES])
def test_sweep_bitexact_vs_single_pass(cuda, name, mk, sec):
    p = mk().plan(*sec)
    xm = _rand_mantissas(p, 7)
    try:
        p.set_matvec_variant(3)
        assert p.matvec_variant == 3, name
        w3, e3 = p.matvec_fixed(xm, -10)
        p.set_matvec_variant(5)
        assert p.matvec_variant == 5
        w5, e5 = p.matvec_fixed(xm, -10)
    finally:
        p.set_matvec_variant(0)
    assert e5 == e3
    assert torch.equal(w5, w3), (name, int((w5 != w3).sum()))


@pytest.mark.parametrize("nu,nd", [(3, 3), (2, 4), (4, 1)])
def test_sweep_vs_oracle_integer_matrix(cuda, nu, nd):
    """Dyadic sector (t = 1/2, U = 3): the integer matvec equals the oracle's H * 2^F."""
    m = _hub(8, True, inter=3.0, mu=1.5, hop=0.5)
    p = m.plan(nu, nd)
    p.set_matvec_variant(5)
    assert p.matvec_variant == 5
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(8, nu), O.sector_states(8, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    F = 1
    vi = np.ldexp(v, F)
    D = len(up) * len(dn)
    A = sp.csr_matrix((vi.astype(np.int64), (c, r)), shape=(D, D))
    x = np.random.default_rng(nu * 10 + nd).integers(-(1 << 40), 1 << 40, size=D)
    wm, ew = p.matvec_fixed(torch.as_tensor(x).cuda(), 0)
    assert ew == -F
    assert np.array_equal(wm.cpu().numpy(), A @ x)


def test_sweep_lanczos_matches_single_pass(cuda):
    """12-site ring (6,6), U=4, mu=2: the renumbered run reproduces the single-pass run and
    the ground-state energy measured with the reference (eigsh on its operator)."""
    from cmpy_gb300 import engine as E

    p = _hub(12, True, inter=4.0, mu=2.0).plan(6, 6)
    g = torch.Generator(device="cuda").manual_seed(12)
    v0 = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    # once the ground state has converged (~100 steps here), a Lanczos run without
    # reorthogonalisation turns rounding differences (here the reduction order of the dot
    # products) into different ghost copies: compare the coefficients before that
    kw = dict(max_steps=200, want_vector=True, v0=v0, tol=1e-12, check_every=10)
    try:
        p.set_matvec_variant(3)
        assert p.matvec_variant == 3
        r3 = E.lanczos(p, **kw)
        p.set_matvec_variant(5)
        assert p.matvec_variant == 5
        r5 = E.lanczos(p, **kw)
    finally:
        p.set_matvec_variant(0)
    assert r5.steps == r3.steps
    np.testing.assert_allclose(r5.alpha[:60].cpu().numpy(), r3.alpha[:60].cpu().numpy(), rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(r5.beta[:61].cpu().numpy(), r3.beta[:61].cpu().numpy(), rtol=1e-11, atol=1e-11)
    assert abs(r5.energy - r3.energy) <= 1e-12 * abs(r3.energy)
    assert abs(r5.energy - (-30.920353562419)) <= 1e-10 * 30.92
    torch.testing.assert_close(r5.vector, r3.vector, rtol=0, atol=1e-9)
    # the Ritz vector is back in the sector's own order: it is an eigenvector of H there
    hv = p.matvec(r5.vector)
    assert torch.linalg.norm(hv - r5.energy * r5.vector).item() < 1e-7


@pytest.mark.parametrize("variant", [5, 3])
def test_first_wait_gives_up_then_recovers(cuda, variant):
    """Wait limit -1: the matvec's first wait for its copies gives up without polling, the
    kernel lets its copies land and returns, the solve reports ED_ERR_TIMEOUT; with the
    default limit the next solve on the same plan succeeds."""
    from cmpy_gb300 import _native as N
    from cmpy_gb300 import engine as E

    p = _hub(12, True, inter=4.0, mu=2.0).plan(6, 6)
    p.set_matvec_variant(variant)
    try:
        assert p.matvec_variant == variant
        p.set_wait_limit(-1)
        with pytest.raises(N.EDError) as ei:
            E.lanczos(p, max_steps=40, want_vector=False)
        assert ei.value.status == N.ED_ERR_TIMEOUT
        p.set_wait_limit(0)
        r = E.lanczos(p, max_steps=200, want_vector=False, tol=1e-12, check_every=10)
        assert abs(r.energy - (-30.920353562419)) <= 1e-10 * 30.92
    finally:
        p.set_wait_limit(0)
        p.set_matvec_variant(0)
