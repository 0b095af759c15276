"""GPU parity of the block-fixed-point (int64 mantissa) path.

* the integer matvec is bit-exact against the oracle's integer matrix (H * 2^F) applied with
  exact int64 arithmetic;
* the fixed-point Lanczos reproduces dense-eigh ground-state energies to 1e-10 relative and
  the FP64-vector Lanczos;
* Green's functions built on it match the dense Lehmann oracle to 1e-8.
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


def _int_matrix(model, nu, nd, F):
    eps, u, bonds, width = model.fermion_descriptor()
    up, dn = O.sector_states(model.num_sites, nu), O.sector_states(model.num_sites, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    vi = np.ldexp(v, F)
    assert np.all(vi == np.round(vi))
    D = len(up) * len(dn)
    # y[col] += val * x[row]  (the reference's product) with exact int64 arithmetic
    return sp.csr_matrix((vi.astype(np.int64), (c, r)), shape=(D, D))


def test_eligibility(cuda):
    from cmpy_gb300.models import SingleImpurityAndersonModel

    assert _hub(14, True, inter=4.0, mu=2.0).plan(7, 7).fixed_point >= 48
    assert _hub(6, False, inter=4.0, mu=2.0).plan(3, 3).fixed_point >= 48
    assert _hub(8, True, inter=3.0, mu=1.5, hop=0.5).plan(4, 4).fixed_point >= 48
    rng = np.random.default_rng(1)
    siam = SingleImpurityAndersonModel(u=4.0, eps_bath=rng.uniform(-2, 2, 5), v=rng.uniform(0.1, 0.6, 5))
    assert siam.plan(3, 3).fixed_point == 0  # several hopping magnitudes
    # arbitrary on-site energies: fixed-point with a rounded (int64) diagonal
    dis = _hub(6, False, inter=4.0, eps=rng.uniform(-1, 1, 6), mu=2.0)
    assert dis.plan(3, 3).fixed_point >= 48
    assert _hub(6, False, inter=4.0, mu=2.0, hop=0.3).plan(3, 3).fixed_point == 0  # t not dyadic


@pytest.mark.parametrize("nu,nd", [(4, 4), (3, 5), (2, 2)])
def test_fixed_random_eps(cuda, nu, nd):
    """Disordered on-site energies (the batched disorder workload): rounded diagonal, exact hops."""
    from cmpy_gb300 import engine as E

    rng = np.random.default_rng(11 + nu)
    m = _hub(8, False, inter=4.0, eps=rng.uniform(-1, 1, 8), mu=2.0)
    p = m.plan(nu, nd)
    x = torch.as_tensor(rng.standard_normal(p.dim)).cuda()
    xm, ex = E.fixed_from_f64(x, p.fixed_point)
    wm, ew = p.matvec_fixed(xm, ex)
    y = p.matvec(E.fixed_to_f64(xm, ex))
    yq = E.fixed_to_f64(wm, ew)
    assert torch.max(torch.abs(yq - y)).item() <= 4e-15 * torch.max(torch.abs(y)).item()
    ref = np.linalg.eigvalsh(O.dense_from_coo(*_coo(m, nu, nd)))[0]
    r = E.lanczos(p, max_steps=300, want_vector=True, tol=1e-12, check_every=10, arithmetic="fixed")
    assert abs(r.energy - ref) <= 1e-10 * abs(ref)


@pytest.mark.parametrize("case", [("chain6", 6, False, 3, 3, 4.0, 2.0, 1.0), ("ring8", 8, True, 4, 3, 6.0, 3.0, 1.0),
                                  ("ring8h", 8, True, 4, 4, 3.0, 1.5, 0.5), ("ring9odd", 9, True, 4, 5, 4.0, 2.0, 1.0),
                                  ("ring10", 10, True, 5, 5, 6.0, 3.0, -1.0),
                                  # odd number of up rows (165): the last row group holds one row
                                  ("ring11odd", 11, True, 3, 4, 4.0, 2.0, 1.0)])
def test_matvec_fixed_bit_exact(cuda, case):
    from cmpy_gb300 import engine as E

    _, N, per, nu, nd, U, mu, t = case
    m = _hub(N, per, inter=U, mu=mu, hop=t)
    p = m.plan(nu, nd)
    m_in = p.fixed_point
    assert m_in > 0
    rng = np.random.default_rng(7)
    x = rng.standard_normal(p.dim)
    xm, ex = E.fixed_from_f64(torch.as_tensor(x).cuda(), m_in)
    xm_h = xm.cpu().numpy()
    assert np.abs(xm_h).max() < 2**m_in
    wm, ew = p.matvec_fixed(xm, ex)
    F = ex - ew
    A = _int_matrix(m, nu, nd, F)
    ref = A @ xm_h  # int64, exact (|values| < 2^62)
    assert np.array_equal(wm.cpu().numpy(), ref)
    # and it is H x up to the input quantisation
    y = p.matvec(torch.as_tensor(x).cuda()).cpu().numpy()
    yq = E.fixed_to_f64(wm, ew).cpu().numpy()
    assert np.max(np.abs(yq - y)) <= 1e-14 * np.max(np.abs(y))


def test_matvec_fixed_14_site(cuda):
    """14-site (7,7), full size: the integer matvec agrees with the FP64 matvec and is exactly
    linear (H(a+b) == Ha + Hb in int64)."""
    from cmpy_gb300 import engine as E

    p = _hub(14, True, inter=4.0, mu=2.0).plan(7, 7)
    gen = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(p.dim, dtype=torch.float64, device="cuda", generator=gen)
    y = torch.randn(p.dim, dtype=torch.float64, device="cuda", generator=gen)
    xm, ex = E.fixed_from_f64(x, p.fixed_point)
    ym, ey = E.fixed_from_f64(y, p.fixed_point)
    assert ex == ey
    hx, ew = p.matvec_fixed(xm, ex)
    ref = p.matvec(x)
    hxf = E.fixed_to_f64(hx, ew)
    torch.testing.assert_close(hxf, ref, rtol=0, atol=1e-14 * ref.abs().max().item())
    a, b = xm >> 1, ym >> 1
    hab, _ = p.matvec_fixed(a + b, ex)
    ha, _ = p.matvec_fixed(a, ex)
    hb, _ = p.matvec_fixed(b, ex)
    assert torch.equal(hab, ha + hb)


@pytest.mark.parametrize("case", ["chain8_44", "ring10_55", "ring10_64", "ring8_half_hop"])
def test_fixed_lanczos_vs_dense(cuda, case):
    from cmpy_gb300 import engine as E

    if case == "chain8_44":
        m, (nu, nd) = _hub(8, False, inter=4.0, mu=2.0), (4, 4)
        ref = np.linalg.eigvalsh(O.dense_from_coo(*_coo(m, 4, 4)))[0]
    elif case == "ring10_55":
        m, (nu, nd) = _hub(10, True, inter=6.0, mu=3.0), (5, 5)
        ref = -34.254559411302544  # reference compute_groundstate value, 10-site ring U=6
    elif case == "ring10_64":
        m, (nu, nd) = _hub(10, True, inter=4.0, mu=2.0), (6, 4)
        ref = None
    else:
        m, (nu, nd) = _hub(8, True, inter=3.0, mu=1.5, hop=0.5), (4, 3)
        ref = np.linalg.eigvalsh(O.dense_from_coo(*_coo(m, 4, 3)))[0]
    p = m.plan(nu, nd)
    rf = E.lanczos(p, max_steps=300, want_vector=True, tol=1e-12, check_every=10, arithmetic="fixed")
    r64 = E.lanczos(p, max_steps=300, want_vector=True, tol=1e-12, check_every=10, arithmetic="f64")
    if ref is None:
        ref = r64.energy
    assert abs(rf.energy - ref) <= 1e-10 * abs(ref), (rf.energy, ref)
    assert abs(r64.energy - ref) <= 1e-10 * abs(ref)
    v = rf.vector
    res = torch.linalg.norm(p.matvec(v) - rf.energy * v).item()
    assert res < 1e-9 * abs(rf.energy)
    assert abs(torch.linalg.norm(v).item() - 1.0) < 1e-12
    # the first Lanczos coefficients of both arithmetics agree (same start vector)
    k = min(20, rf.steps, r64.steps)
    np.testing.assert_allclose(rf.alpha[:k].cpu().numpy(), r64.alpha[:k].cpu().numpy(), rtol=1e-12, atol=1e-12)


def _coo(m, nu, nd):
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(m.num_sites, nu), O.sector_states(m.num_sites, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    return len(up) * len(dn), r, c, v


def test_fixed_arithmetic_errors(cuda):
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import SingleImpurityAndersonModel

    siam = SingleImpurityAndersonModel(u=4.0, eps_bath=[-1.3, 0.7, 0.2], v=[0.31, 0.2, 0.45])
    p = siam.plan(2, 2)
    with pytest.raises(ValueError):
        E.lanczos(p, max_steps=20, arithmetic="fixed")
    with pytest.raises(ValueError):
        p.matvec_fixed(torch.zeros(p.dim, dtype=torch.int64, device="cuda"), 0)
    q = _hub(6, False, inter=4.0, mu=2.0).plan(3, 3)
    with pytest.raises(ValueError):
        E.lanczos(q, max_steps=20, reorth=True, arithmetic="fixed")


def test_fixed_gf_vs_dense(cuda):
    """The CF Green's function on fixed-point Lanczos coefficients matches the dense oracle."""
    from cmpy_gb300.exactdiag import gf_continued_fraction, groundstate_sector

    m = _hub(8, True, inter=4.0, mu=2.0)
    nu, nd = 4, 4
    e0, psi = groundstate_sector(m, nu, nd, max_steps=400, tol=1e-13)
    z = np.concatenate([np.linspace(-8, 8, 256) + 0.05j, 1j * (2 * np.arange(128) + 1) * np.pi / 50.0])
    # 1000 levels resolve the real axis at eta = 0.05 for this sector (1285 weighted poles)
    g = gf_continued_fraction(m, z, nu, nd, e0, psi, pos=0, n_lev=1000)
    psi_h = psi.cpu().numpy()
    up, dn = O.sector_states(8, nu), O.sector_states(8, nd)
    upp, upm = O.sector_states(8, nu + 1), O.sector_states(8, nu - 1)
    cd = O.apply_fermion(up, dn, upp, dn, 0, O.UP, True, psi_h)
    cm = O.apply_fermion(up, dn, upm, dn, 0, O.UP, False, psi_h)
    Hp = O.dense_from_coo(*_coo(m, nu + 1, nd))
    Hm = O.dense_from_coo(*_coo(m, nu - 1, nd))
    ref = O.gf_zero_temperature_dense(None, Hp, Hm, cd, cm, e0, z)
    assert np.max(np.abs(g - ref)) < 1e-8
