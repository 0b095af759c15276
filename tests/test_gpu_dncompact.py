"""GPU parity of variant 7 of the fixed-point matvec: the single-pass kernel with the dn states
renumbered by their numbers of + and - hops, so that each 64-column chunk runs over its own
list lengths instead of every bond slot.

* its integer H·x equals variant 3's bit for bit on the benchmark-like sectors, and the oracle's
  integer matrix on small dyadic sectors;
* a Lanczos run in its renumbered basis gives variant 3's coefficients and ground state, and
  the Ritz vector comes back in the sector's own order;
* the 14-site ring's ground-state energy equals the oracle's eigsh pin.
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
def test_compact_bitexact_vs_single_pass(cuda, name, mk, sec):
    p = mk().plan(*sec)
    xm = _rand_mantissas(p, 11)
    try:
        _with_variant(p, 3)
        w3, e3 = p.matvec_fixed(xm, -10)
        _with_variant(p, 7)
        w7, e7 = p.matvec_fixed(xm, -10)
    finally:
        p.set_matvec_variant(0)
    assert e7 == e3
    assert torch.equal(w7, w3), (name, int((w7 != w3).sum()))


@pytest.mark.parametrize("nu,nd,periodic", [(3, 3, True), (2, 4, True), (4, 4, False), (4, 2, False)])
def test_compact_vs_oracle_integer_matrix(cuda, nu, nd, periodic):
    """Dyadic sector (t = 1/2, U = 3): the integer matvec equals the oracle's H * 2^F."""
    m = _hub(8, periodic, inter=3.0, mu=1.5, hop=0.5)
    p = m.plan(nu, nd)
    _with_variant(p, 7)
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


def test_compact_lanczos_matches_single_pass(cuda):
    from cmpy_gb300 import engine as E

    p = _hub(12, True, inter=4.0, mu=2.0).plan(6, 6)
    g = torch.Generator(device="cuda").manual_seed(12)
    v0 = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    kw = dict(max_steps=200, want_vector=True, v0=v0, tol=1e-12, check_every=10)
    r3 = E.lanczos(p, **kw)
    try:
        _with_variant(p, 7)
        r7 = E.lanczos(p, **kw)
        hv = p.matvec(r7.vector)
    finally:
        p.set_matvec_variant(0)
    assert r7.steps == r3.steps
    np.testing.assert_allclose(r7.alpha[:60].cpu().numpy(), r3.alpha[:60].cpu().numpy(), rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(r7.beta[:61].cpu().numpy(), r3.beta[:61].cpu().numpy(), rtol=1e-11, atol=1e-11)
    assert abs(r7.energy - r3.energy) <= 1e-12 * abs(r3.energy)
    torch.testing.assert_close(r7.vector, r3.vector, rtol=0, atol=1e-9)
    assert torch.linalg.norm(hv - r7.energy * r7.vector).item() < 1e-7


def test_default_variant(cuda):
    """The benchmark sectors run variant 7 by default; a forced variant 3 is honoured."""
    for name, mk, sec in CASES:
        p = mk().plan(*sec)
        assert p.matvec_variant == 7, name
        p.set_matvec_variant(3)
        assert p.matvec_variant == 3, name
        p.set_matvec_variant(0)
        assert p.matvec_variant == 7, name


def test_compact_ring14_energy_vs_oracle(cuda, golden):
    from cmpy_gb300 import engine as E

    p = _hub(14, True, inter=4.0, mu=2.0).plan(7, 7)
    try:
        _with_variant(p, 7)
        r = E.lanczos(p, max_steps=250, want_vector=False)
    finally:
        p.set_matvec_variant(0)
    e_ref = float(golden["bench_e0"]["ring14_77_U4_e0"])
    assert abs(r.energy - e_ref) <= 1e-10 * abs(e_ref)
