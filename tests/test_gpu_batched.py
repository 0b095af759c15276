"""GPU parity of the batched form: all sectors / many disorder realisations in one launch.

Energies agree with the per-sector solver and the dense oracle to 1e-10 relative, ground-state
vectors satisfy H psi = E psi, batched Green's functions match the per-problem continued
fraction and the dense Lehmann oracle to 1e-8, graph replay is bitwise reproducible."""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu


def _hub(N, periodic, **kw):
    from cmpy_gb300.models import ChainLattice, HubbardModel

    return HubbardModel(ChainLattice(N, periodic), **kw)


def _dense(m, nu, nd):
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(m.num_sites, nu), O.sector_states(m.num_sites, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    return O.dense_from_coo(len(up) * len(dn), r, c, v)


def test_all_sectors_chain6(cuda, golden):
    from cmpy_gb300.batched import groundstate_all_sectors

    m = _hub(6, False, inter=4.0, mu=2.0)
    fillings, res, b = groundstate_all_sectors(m, max_steps=300)
    e = res.energy.cpu().numpy()
    for (nu, nd), ei in zip(fillings, e):
        ref = np.linalg.eigvalsh(_dense(m, nu, nd))[0]
        assert abs(ei - ref) <= 1e-10 * max(1.0, abs(ref)), (nu, nd, ei, ref)
    g = golden["exactdiag"]
    i = int(np.argmin(e))
    assert tuple(fillings[i]) == tuple(g["chain6_U4_sector"])
    assert abs(e[i] - g["chain6_U4_E0"]) <= 1e-10 * abs(g["chain6_U4_E0"])
    assert b.threads in (128, 256, 512, 1024)


def test_all_sectors_ring10(cuda):
    """The 121-sector sweep of the 10-site ring (U=6) against per-sector plain solves."""
    from cmpy_gb300 import engine as E
    from cmpy_gb300.batched import groundstate_all_sectors

    m = _hub(10, True, inter=6.0, mu=3.0)
    fillings, res, _ = groundstate_all_sectors(m, max_steps=300)
    e = res.energy.cpu().numpy()
    assert len(fillings) == 121
    i = int(np.argmin(e))
    assert tuple(fillings[i]) == (5, 5)
    assert abs(e[i] - (-34.254559411302544)) <= 1e-10 * 34.25
    for k in (0, 7, 33, 60, 88, 120):
        nu, nd = fillings[k]
        p = m.plan(nu, nd)
        ref = E.lanczos(p, max_steps=min(300, p.dim), want_vector=False, tol=1e-12, check_every=10).energy
        assert abs(e[k] - ref) <= 1e-10 * max(1.0, abs(ref)), (nu, nd)


def test_batched_vectors_and_configs(cuda):
    from cmpy_gb300.batched import Batch

    rng = np.random.default_rng(2)
    models = [_hub(8, False, inter=4.0, eps=rng.uniform(-1, 1, 8), mu=2.0) for _ in range(12)]
    sectors = [tuple(rng.integers(2, 6, 2)) for _ in models]
    plans = [m.plan(int(a), int(b)) for m, (a, b) in zip(models, sectors)]
    b = Batch(plans)
    r1 = b.lanczos(max_steps=300, want_vector=True)
    for m, (nu, nd), p, ei, v in zip(models, sectors, plans, r1.energy.cpu().numpy(), r1.vectors):
        ref = np.linalg.eigvalsh(_dense(m, int(nu), int(nd)))[0]
        assert abs(ei - ref) <= 1e-10 * abs(ref)
        assert abs(torch.linalg.norm(v).item() - 1) < 1e-12
        assert torch.linalg.norm(p.matvec(v) - ei * v).item() < 1e-8 * abs(ei)
    # every launch configuration gives the same energies, thread-block clusters included
    # (a cluster of CTAs shares each problem: the partial sums are combined in another order)
    for th, ps, cs in ((128, 4, 1), (256, 2, 1), (1024, 1, 1), (512, 2, 2), (1024, 1, 4), (512, 2, 8)):
        b.threads, b.ctas_per_sm, b.cluster_size = th, ps, cs
        r2 = b.lanczos(max_steps=300, want_vector=cs == 4)
        np.testing.assert_allclose(r2.energy.cpu().numpy(), r1.energy.cpu().numpy(), rtol=1e-12)
        if cs == 4:
            for p, ei, v in zip(plans, r2.energy.cpu().numpy(), r2.vectors):
                assert abs(torch.linalg.norm(v).item() - 1) < 1e-12
                assert torch.linalg.norm(p.matvec(v) - ei * v).item() < 1e-8 * abs(ei)


def test_batched_gf_vs_dense(cuda):
    """Realisations of the 8-site Anderson-Hubbard chain (eps ~ U[-1,1], U=4, t=1, mu=2),
    sectors up to (4,4) (target sectors of dimension 3,920): with 2000 Lanczos levels the
    batched continued fractions equal the dense-eigh Lehmann sum to 1e-8 on the real axis
    (eta = 0.05) and on the Matsubara axis, and equal the per-realisation runs to 1e-8."""
    from cmpy_gb300.batched import greens_functions_batched
    from cmpy_gb300.exactdiag import gf_continued_fraction, groundstate_sector

    rng = np.random.default_rng(4)
    n = 8
    sectors = [(4, 4), (3, 4), (5, 3), (2, 2), (4, 5), (3, 3)]
    models = [_hub(n, False, inter=4.0, eps=rng.uniform(-1, 1, n), mu=2.0) for _ in sectors]
    nw = 256
    z = np.concatenate([np.linspace(-8, 8, nw) + 0.05j, 1j * (2 * np.arange(64) + 1) * np.pi / 10.0])
    levels = 2000
    e, g = greens_functions_batched(models, sectors, z, gf_levels=levels)
    g = g.cpu().numpy()
    for i, (m, (nu, nd)) in enumerate(zip(models, sectors)):
        e0, psi = groundstate_sector(m, nu, nd, max_steps=400, tol=1e-13)
        assert abs(e[i].item() - e0) <= 1e-10 * abs(e0)
        ref = gf_continued_fraction(m, z, nu, nd, e0, psi, pos=0, n_lev=levels)
        assert np.max(np.abs(g[i] - ref)) < 1e-8
        # dense oracle: Lehmann sum over the eigenpairs of both neighbouring sectors
        psi_h = psi.cpu().numpy()
        up, dn = O.sector_states(n, nu), O.sector_states(n, nd)
        cd = O.apply_fermion(up, dn, O.sector_states(n, nu + 1), dn, 0, 1, True, psi_h)
        cm = O.apply_fermion(up, dn, O.sector_states(n, nu - 1), dn, 0, 1, False, psi_h)
        dref = O.gf_zero_temperature_dense(None, _dense(m, nu + 1, nd), _dense(m, nu - 1, nd), cd, cm, e0, z)
        assert np.max(np.abs(g[i][:nw] - dref[:nw])) < 1e-8, (i, np.max(np.abs(g[i][:nw] - dref[:nw])))
        assert np.max(np.abs(g[i][nw:] - dref[nw:])) < 1e-8


def test_batch_graph_replay(cuda):
    from cmpy_gb300.batched import Batch, BatchGraph

    m = _hub(8, True, inter=4.0, mu=2.0)
    plans = [m.plan(a, b) for a in range(2, 6) for b in range(2, 6)]
    b = Batch(plans)
    ref = b.lanczos(max_steps=200).energy.clone()
    g = BatchGraph(b, max_steps=200)
    out = g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out.energy, ref)
    out2 = g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out2.energy, ref)


def test_batch_rejects_non_fixed_point(cuda):
    from cmpy_gb300.batched import Batch
    from cmpy_gb300.models import SingleImpurityAndersonModel

    s = SingleImpurityAndersonModel(u=4.0, eps_bath=[-1.3, 0.7], v=[0.31, 0.2])
    with pytest.raises(ValueError):
        Batch([s.plan(1, 1)])


@pytest.mark.parametrize("sigma,create,jw", [(1, True, False), (1, False, True), (2, True, True), (2, False, False)])
def test_apply_fermion_batch_equals_single(cuda, sigma, create, jw):
    """ed_apply_fermion_batch: every problem bit-identical to its own ed_apply_fermion call."""
    from cmpy_gb300 import engine as E

    rng = np.random.default_rng(11)
    models = [_hub(7, True, inter=3.0, eps=rng.uniform(-1, 1, 7), mu=1.5) for _ in range(5)]
    sectors = [(3, 3), (2, 4), (4, 2), (1, 3), (3, 1)]
    d = 1 if create else -1
    src, dst = [], []
    for m, (nu, nd) in zip(models, sectors):
        src.append(m.plan(nu, nd))
        dst.append(m.plan(nu + d, nd) if sigma == 1 else m.plan(nu, nd + d))
    x_off = np.concatenate([[0], np.cumsum([p.dim for p in src])[:-1]]).astype(np.int64)
    x = torch.randn(int(sum(p.dim for p in src)) + 3, dtype=torch.float64, device="cuda")
    y, y_off = E.apply_fermion_batch(src, dst, 2, sigma, create, x, x_off, jw_sign=jw)
    for p, t, xo, yo in zip(src, dst, x_off, y_off):
        ref = p.apply_fermion(t, 2, sigma, create, x[xo:xo + p.dim], jw_sign=jw)
        assert torch.equal(y[yo:yo + t.dim], ref)


def test_apply_fermion_batch_rejects_before_launch(cuda):
    from cmpy_gb300 import engine as E

    m = _hub(6, False, inter=4.0, mu=2.0)
    src = [m.plan(3, 3), m.plan(2, 3)]
    dst = [m.plan(4, 3), m.plan(2, 4)]  # second target is not the up-neighbour sector
    x = torch.zeros(src[0].dim + src[1].dim, dtype=torch.float64, device="cuda")
    with pytest.raises(Exception):
        E.apply_fermion_batch(src, dst, 0, 1, True, x, [0, src[0].dim])
    with pytest.raises(ValueError):
        E.apply_fermion_batch(src, [m.plan(4, 3), m.plan(3, 3)], 0, 1, True, x, [0, src[0].dim + 1])
