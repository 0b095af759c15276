"""GPU parity of the adjoint (reverse-mode) Green's function.

Gradients of a least-squares loss on G_imp(i w_n) of single-impurity Anderson models with
respect to bath energies and hybridisations are checked against (1) central finite
differences of the same forward and (2) torch autograd through a dense FP64 reference
(torch.linalg.eigh for the ground state, a dense resolvent for the excitations), to 1e-6
relative."""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu


def _target(z):
    rng = np.random.default_rng(30)
    ek = rng.uniform(-2, 2, 30)
    delta = np.sum(0.3**2 / (z[:, None] - ek[None, :]), axis=1)
    return 1.0 / (z - delta)


def _loss(g, gt):
    return torch.sum(torch.abs(g - gt) ** 2)


def _siam_theta(u, eb, v):
    from cmpy_gb300.adjoint import siam_parameters

    return siam_parameters(torch.tensor(u, dtype=torch.float64, device="cuda"), torch.tensor(0.0, dtype=torch.float64, device="cuda"), eb, v)


def _dense_reference(theta, n_sites, bonds, sector, z, pos=0):
    """Exact T=0 G(z) as a torch function of theta (H is linear in theta)."""
    nu, nd = sector

    def mats(a, b):
        up, dn = O.sector_states(n_sites, a), O.sector_states(n_sites, b)
        D = len(up) * len(dn)
        occ_u = ((up[:, None] >> np.arange(n_sites)) & 1).astype(float)
        occ_d = ((dn[:, None] >> np.arange(n_sites)) & 1).astype(float)
        M = []
        for j in range(n_sites):
            M.append(np.diag((occ_u[:, j][:, None] + occ_d[:, j][None, :]).reshape(-1)))
        for j in range(n_sites):
            M.append(np.diag((occ_u[:, j][:, None] * occ_d[:, j][None, :]).reshape(-1)))
        for (i, j) in bonds:
            r, c, v = O.coo_hopping(up, dn, 0, i, j, 1.0)
            M.append(O.dense_from_coo(D, r, c, v))
        return torch.as_tensor(np.stack(M)).cuda(), up, dn

    M0, up, dn = mats(nu, nd)
    H0 = torch.einsum("p,pij->ij", theta, M0)
    w, V = torch.linalg.eigh(H0)
    e0, psi = w[0], V[:, 0]
    zt = torch.as_tensor(z).cuda()
    g = torch.zeros_like(zt)
    for delta, create, sign in ((1, True, 1), (-1, False, -1)):
        a = nu + delta
        if not 0 <= a <= n_sites:
            continue
        M1, up1, _ = mats(a, nd)
        H1 = torch.einsum("p,pij->ij", theta, M1)
        A = torch.as_tensor(O.apply_fermion(up, dn, up1, dn, pos, 1, create, np.eye(len(up) * len(dn)))).cuda()
        phi = A @ psi
        I = torch.eye(H1.shape[0], dtype=torch.complex128, device="cuda")
        for k in range(zt.numel()):
            Rz = (sign * zt[k] + e0) * I - H1.to(torch.complex128)
            g[k] = g[k] + sign * torch.dot(phi.to(torch.complex128), torch.linalg.solve(Rz, phi.to(torch.complex128)))
    return g


@pytest.mark.parametrize("nbath", [3, 4])
def test_adjoint_vs_dense_autograd_and_fd(cuda, nbath):
    from cmpy_gb300.adjoint import greens_function_ad

    rng = np.random.default_rng(nbath)
    eb = torch.tensor(rng.uniform(-2, 2, nbath), dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor(rng.uniform(0.1, 0.6, nbath), dtype=torch.float64, device="cuda", requires_grad=True)
    beta = 100.0
    z = 1j * (2 * np.arange(48) + 1) * np.pi / beta
    gt = torch.as_tensor(_target(z)).cuda()
    nh = (nbath + 1) // 2
    sector = (nh, nh)

    theta, n_sites, bonds, width = _siam_theta(4.0, eb, v)
    g = greens_function_ad(theta, n_sites, bonds, sector, z, sign_width=width, gs_steps=200, gf_levels=200, ckpt=4)
    L = _loss(g, gt)
    L.backward()
    grad = torch.cat([eb.grad, v.grad]).cpu().numpy()

    # dense autograd reference
    eb2 = eb.detach().clone().requires_grad_(True)
    v2 = v.detach().clone().requires_grad_(True)
    theta2, _, _, _ = _siam_theta(4.0, eb2, v2)
    gd = _dense_reference(theta2, n_sites, bonds, sector, z)
    assert torch.max(torch.abs(gd - g.detach())).item() < 1e-8
    Ld = _loss(gd, gt)
    Ld.backward()
    gref = torch.cat([eb2.grad, v2.grad]).cpu().numpy()
    np.testing.assert_allclose(grad, gref, rtol=1e-6, atol=1e-9 * np.abs(gref).max())

    # central finite differences of the same forward
    h = 1e-5
    fd = []
    base = torch.cat([eb.detach(), v.detach()])
    for i in range(base.numel()):
        vals = []
        for s in (1, -1):
            p = base.clone()
            p[i] += s * h
            th, _, _, _ = _siam_theta(4.0, p[:nbath], p[nbath:])
            with torch.no_grad():
                gg = greens_function_ad(th, n_sites, bonds, sector, z, sign_width=width, gs_steps=200,
                                        gf_levels=200, ckpt=4)
            vals.append(_loss(gg, gt).item())
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    np.testing.assert_allclose(grad, fd, rtol=1e-6, atol=1e-8 * np.abs(fd).max())


def test_adjoint_checkpoint_invariance(cuda):
    """The gradient does not depend on the checkpoint spacing (memory bound)."""
    from cmpy_gb300.adjoint import greens_function_ad

    rng = np.random.default_rng(9)
    eb0 = rng.uniform(-2, 2, 5)
    v0 = rng.uniform(0.1, 0.6, 5)
    z = 1j * (2 * np.arange(32) + 1) * np.pi / 100.0
    gt = torch.as_tensor(_target(z)).cuda()
    grads = []
    for c in (1, 7, 32):
        eb = torch.tensor(eb0, dtype=torch.float64, device="cuda", requires_grad=True)
        v = torch.tensor(v0, dtype=torch.float64, device="cuda", requires_grad=True)
        theta, n_sites, bonds, width = _siam_theta(4.0, eb, v)
        g = greens_function_ad(theta, n_sites, bonds, (3, 3), z, sign_width=width, gs_steps=150, gf_levels=120,
                               ckpt=c)
        _loss(g, gt).backward()
        grads.append(torch.cat([eb.grad, v.grad]).cpu().numpy())
    np.testing.assert_allclose(grads[1], grads[0], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(grads[2], grads[0], rtol=1e-9, atol=1e-12)


def test_adjoint_batch_equals_single(cuda):
    """greens_function_ad_batch (all problems in each launch) gives each problem the forward
    and the gradient of greens_function_ad (same arithmetic; the reductions are blocked
    differently, so to rounding)."""
    from cmpy_gb300.adjoint import greens_function_ad, greens_function_ad_batch

    rng = np.random.default_rng(41)
    B, nb = 5, 4
    z = 1j * (2 * np.arange(40) + 1) * np.pi / 100.0
    gt = torch.as_tensor(_target(z)).cuda()
    eb0 = rng.uniform(-2, 2, (B, nb))
    v0 = rng.uniform(0.1, 0.6, (B, nb))
    kw = dict(gs_steps=150, gf_levels=100, ckpt=8)

    eb = torch.tensor(eb0, dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor(v0, dtype=torch.float64, device="cuda", requires_grad=True)
    rows = []
    for i in range(B):
        th, n_sites, bonds, width = _siam_theta(4.0, eb[i], v[i])
        rows.append(th)
    thetas = torch.stack(rows)
    g = greens_function_ad_batch(thetas, n_sites, bonds, (2, 3), z, sign_width=width, **kw)
    _loss(g, gt.expand_as(g)).backward()

    for i in range(B):
        ebi = torch.tensor(eb0[i], dtype=torch.float64, device="cuda", requires_grad=True)
        vi = torch.tensor(v0[i], dtype=torch.float64, device="cuda", requires_grad=True)
        th, _, _, _ = _siam_theta(4.0, ebi, vi)
        gi = greens_function_ad(th, n_sites, bonds, (2, 3), z, sign_width=width, **kw)
        torch.testing.assert_close(gi.detach(), g[i].detach(), rtol=1e-10, atol=1e-12)
        _loss(gi, gt).backward()
        torch.testing.assert_close(ebi.grad, eb.grad[i], rtol=1e-8, atol=1e-10)
        torch.testing.assert_close(vi.grad, v.grad[i], rtol=1e-8, atol=1e-10)
