"""GPU parity: the matrix-free matvec, the generic triplet operator and c^dag / c."""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu

SECTORS = {
    "chain6_U4": [(3, 3), (3, 2), (4, 3), (2, 3), (0, 1), (6, 6)],
    "ring5_dis": [(2, 3), (3, 2), (1, 1), (0, 2), (5, 4)],
    "siam": [(2, 2), (3, 2), (2, 1), (5, 5)],
}


def _model(name, golden):
    from cmpy_gb300.models import ChainLattice, HubbardModel, SingleImpurityAndersonModel

    g = golden["coo"]
    if name == "chain6_U4":
        return HubbardModel(ChainLattice(6), inter=4.0, mu=2.0, hop=1.0)
    if name == "ring5_dis":
        return HubbardModel(ChainLattice(5, True), inter=3.0, eps=g["ring5_eps"], mu=1.5, hop=0.7)
    return SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=g["siam_eps_bath"], v=g["siam_v"])


@pytest.mark.parametrize("name", list(SECTORS))
def test_matvec_vs_reference(cuda, golden, name):
    g = golden["coo"]
    m = _model(name, golden)
    for nu, nd in SECTORS[name]:
        tag = f"{name}_{nu}{nd}"
        op = m.hamilton_operator(nu, nd)
        y = op.matvec(g[f"{tag}_x"])
        ref = g[f"{tag}_y"]
        np.testing.assert_allclose(y, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
        # generic triplet operator (reference constructor) is bit-exact
        from cmpy_gb300.operators import HamiltonOperator

        gen = HamiltonOperator(op.shape[0], g[f"{tag}_vals"], np.stack([g[f"{tag}_rows"], g[f"{tag}_cols"]]))
        yg = gen.matvec(g[f"{tag}_x"])
        assert np.array_equal(yg.view(np.int64), ref.view(np.int64)), tag
        # matmat, trace, adjoint, torch in/out
        X = np.stack([g[f"{tag}_x"], 2 * g[f"{tag}_x"]], 1)
        Y = op.matmat(X)
        np.testing.assert_allclose(Y[:, 1], 2 * y, rtol=1e-14, atol=1e-14)
        if f"{tag}_dense" in g:
            assert abs(op.trace() - np.trace(g[f"{tag}_dense"])) < 1e-10
        assert op.adjoint() is op or op.H is not None
        yt = op.matvec(torch.as_tensor(g[f"{tag}_x"]).cuda())
        assert isinstance(yt, torch.Tensor) and yt.is_cuda


def _ring14_slice(up_rows: int):
    """Oracle CSR of the reference triplets whose origin lies in the first `up_rows` up-rows
    of the 14-site ring (7,7) (U=4, mu=2, t=1)."""
    import scipy.sparse as sp

    up = O.sector_states(14, 7)
    ring = [(i, (i + 1) % 14) if i < (i + 1) % 14 else ((i + 1) % 14, i) for i in range(14)]
    eps, uu, bonds, width = O.hubbard_descriptor(14, ring, inter=4.0, hop=1.0, mu=2.0)
    r, c, v = O.coo_fermion_rows(up, up, eps, uu, bonds, width, up_rows)
    nd = len(up)
    return sp.csr_matrix((v, (r, c)), shape=(up_rows * nd, len(up) * nd))


def test_matvec_14site_properties(cuda):
    """Full-size 14-site (7,7) sector: agreement with the oracle's CSR of the reference
    triplets on the first 96 of 3432 up-rows (FP64 matvec to 1e-13; the fixed-point matvec
    bit-exact on an integer vector, where every partial sum is an exact FP64 integer), plus
    symmetry <x,Hy> = <Hx,y> and linearity on the whole sector."""
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(14, True), inter=4.0, mu=2.0, hop=1.0)
    p = m.plan(7, 7)
    assert p.dim == 3432 * 3432
    rows = 96
    csr = _ring14_slice(rows)
    n = csr.shape[0]
    rng = np.random.default_rng(14)
    xh = rng.standard_normal(p.dim)
    ref = csr @ xh
    y = p.matvec(torch.as_tensor(xh).cuda())[:n].cpu().numpy()
    np.testing.assert_allclose(y, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    xi = rng.integers(-(1 << 20), 1 << 20, size=p.dim).astype(np.int64)
    wm, ew = p.matvec_fixed(torch.as_tensor(xi).cuda(), 0)
    assert ew == 0
    ref_i = csr @ xi.astype(np.float64)
    assert np.array_equal(wm[:n].cpu().numpy(), ref_i.astype(np.int64))
    # the same through FP64 -> fixed point -> FP64 (the Lanczos store's encoding)
    xm, ex = E.fixed_from_f64(torch.as_tensor(xh).cuda(), p.fixed_point)
    wm2, ew2 = p.matvec_fixed(xm, ex)
    yf = E.fixed_to_f64(wm2, ew2)[:n].cpu().numpy()
    np.testing.assert_allclose(yf, ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(p.dim, dtype=torch.float64, device="cuda", generator=gen)
    yv = torch.randn(p.dim, dtype=torch.float64, device="cuda", generator=gen)
    Hx, Hy = p.matvec(x), p.matvec(yv)
    a, b = torch.dot(x, Hy).item(), torch.dot(Hx, yv).item()
    assert abs(a - b) <= 1e-12 * (abs(a) + abs(b))
    Hxy = p.matvec(2.0 * x - 3.0 * yv)
    torch.testing.assert_close(Hxy, 2.0 * Hx - 3.0 * Hy, rtol=1e-12, atol=1e-11)


def test_matvec_heisenberg20(cuda):
    from cmpy_gb300.models import ChainLattice, HeisenbergModel

    rng = np.random.default_rng(0)
    J = np.zeros((20, 20))
    for i in range(20):
        k = (i + 1) % 20
        J[i, k] = J[k, i] = 1 + 0.1 * rng.standard_normal()
    m = HeisenbergModel(ChainLattice(20, True), j=J)
    p = m.plan(0.0)
    assert p.dim == 184756
    x = torch.randn(p.dim, dtype=torch.float64, device="cuda")
    y = torch.randn(p.dim, dtype=torch.float64, device="cuda")
    a, b = torch.dot(x, p.matvec(y)).item(), torch.dot(p.matvec(x), y).item()
    assert abs(a - b) <= 1e-12 * (abs(a) + abs(b))
    # against the oracle CSR on the full sector
    states = O.sector_states(20, 10)
    pairs = O.heisenberg_pairs([[(i - 1) % 20, (i + 1) % 20] for i in range(20)], J)
    pairs = [(p1, p2, jj, jz) for p1, p2, jj, jz in pairs]
    r, c, v = O.coo_heisenberg(states, sorted(pairs, key=lambda t: (t[0], t[1])))
    xs = x.cpu().numpy()
    ref = O.csr_from_coo(len(states), c, r, v) @ xs
    np.testing.assert_allclose(p.matvec(x).cpu().numpy(), ref, rtol=1e-12, atol=1e-12)


def test_fermion_ops_up_golden(cuda, golden):
    from cmpy_gb300.basis import UP, Basis
    from cmpy_gb300.operators import AnnihilationOperator, CreationOperator

    g = golden["fermion_ops"]
    b4 = Basis(4)
    for nu, nd in [(2, 1), (1, 2), (0, 0)]:
        sec, sp1 = b4.get_sector(nu, nd), b4.upper_sector(nu, nd, UP)
        for pos in range(4):
            y = CreationOperator(sec, sp1, pos, UP).matvec(g[f"cdag_x_{nu}{nd}"])
            assert np.array_equal(np.real(y), g[f"cdag_{nu}{nd}_p{pos}"])
            y2 = AnnihilationOperator(sp1, sec, pos, UP).matvec(g[f"c_x_{nu}{nd}_p{pos}"])
            assert np.array_equal(np.real(y2), g[f"c_{nu}{nd}_p{pos}"])


@pytest.mark.parametrize("jw", [False, True])
def test_fermion_ops_dn_and_jw_vs_oracle(cuda, jw):
    from cmpy_gb300.basis import DN, UP, Basis
    from cmpy_gb300.operators import AnnihilationOperator, CreationOperator

    N = 5
    b = Basis(N)
    rng = np.random.default_rng(5)
    for sigma in (UP, DN):
        for nu, nd in [(2, 1), (1, 3), (3, 3), (0, 0)]:
            sec = b.get_sector(nu, nd)
            tgt = b.upper_sector(nu, nd, sigma)
            up, dn = O.sector_states(N, nu), O.sector_states(N, nd)
            up_t, dn_t = np.asarray(tgt.up_states), np.asarray(tgt.dn_states)
            X = rng.standard_normal((sec.size, 3))
            for pos in range(N):
                cd = CreationOperator(sec, tgt, pos, sigma, jw_sign=jw)
                ref = O.apply_fermion(up, dn, up_t, dn_t, pos, sigma, True, X, jw)
                assert np.array_equal(np.real(cd.matmat(X)), ref)
                an = AnnihilationOperator(tgt, sec, pos, sigma, jw_sign=jw)
                # adjointness: c = (c^dag)^T
                A = np.real(an.toarray())
                Cd = np.real(cd.toarray())
                assert np.array_equal(A, Cd.T)
