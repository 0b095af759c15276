"""Adjoint Green's function with respect to every model parameter: on-site energies, U and the
hopping of each bond (theta = [eps(N), U(N), t(n_bonds)], cmpy/models/hubbard.py:75-81 and
cmpy/models/anderson.py:147-158 define the models).

* Hubbard chain with site-dependent eps, U and bond-dependent t: the gradient of a Matsubara
  least-squares loss equals torch autograd through a dense FP64 reference and central finite
  differences, to 1e-6 relative, for all 14 parameters;
* SIAM: d/dU and d/d eps_imp through siam_parameters (U enters both the interaction and mu = U/2);
* at the size of the differentiated benchmark (1 impurity + 9 bath sites, sector (5,5),
  D = 63,504, 250 ground-state steps, 150 levels, 1024 Matsubara frequencies at beta = 100):
  the adjoint gradient of U, eps_imp, one bath energy and one hybridisation equals central
  finite differences of the same forward to 1e-6 relative.
"""

import numpy as np
import pytest
import torch

from test_gpu_adjoint import _dense_reference, _loss, _target

pytestmark = pytest.mark.gpu


def _fd(fun, x0, h):
    out = []
    for i in range(x0.numel()):
        vals = []
        for s in (1, -1):
            x = x0.clone()
            x[i] += s * h
            with torch.no_grad():
                vals.append(fun(x))
        out.append((vals[0] - vals[1]) / (2 * h))
    return np.array(out)


def test_hubbard_chain_all_parameters(cuda):
    from cmpy_gb300.adjoint import greens_function_ad

    n = 5
    rng = np.random.default_rng(17)
    bonds = [(i, i + 1) for i in range(n - 1)]
    eps = rng.uniform(-1, 1, n) - 1.5
    uu = rng.uniform(2.0, 4.0, n)
    tt = rng.uniform(0.6, 1.2, n - 1)
    theta = torch.tensor(np.concatenate([eps, uu, tt]), dtype=torch.float64, device="cuda", requires_grad=True)
    sector = (2, 2)
    z = 1j * (2 * np.arange(40) + 1) * np.pi / 20.0
    gt = torch.as_tensor(_target(z)).cuda()
    kw = dict(sign_width=n, gs_steps=100, gf_levels=100, ckpt=4)

    g = greens_function_ad(theta, n, bonds, sector, z, **kw)
    _loss(g, gt).backward()
    grad = theta.grad.cpu().numpy()

    th2 = theta.detach().clone().requires_grad_(True)
    gd = _dense_reference(th2, n, bonds, sector, z)
    assert torch.max(torch.abs(gd - g.detach())).item() < 1e-8
    _loss(gd, gt).backward()
    gref = th2.grad.cpu().numpy()
    np.testing.assert_allclose(grad, gref, rtol=1e-6, atol=1e-9 * np.abs(gref).max())
    # the t and U entries are not trivially zero
    assert np.min(np.abs(grad[n:])) > 1e-6 * np.abs(grad).max()

    fd = _fd(lambda th: _loss(greens_function_ad(th, n, bonds, sector, z, **kw), gt).item(), theta.detach(), 1e-5)
    np.testing.assert_allclose(grad, fd, rtol=1e-6, atol=1e-8 * np.abs(fd).max())


def test_siam_interaction_and_impurity_level(cuda):
    from cmpy_gb300.adjoint import greens_function_ad, siam_parameters

    rng = np.random.default_rng(23)
    nb = 3
    eb = torch.tensor(rng.uniform(-2, 2, nb), dtype=torch.float64, device="cuda")
    v = torch.tensor(rng.uniform(0.1, 0.6, nb), dtype=torch.float64, device="cuda")
    z = 1j * (2 * np.arange(48) + 1) * np.pi / 100.0
    gt = torch.as_tensor(_target(z)).cuda()
    kw = dict(gs_steps=150, gf_levels=150, ckpt=4)

    def loss_of(p, dense=False):
        th, ns, bonds, width = siam_parameters(p[0], p[1], eb, v)
        if dense:
            return _loss(_dense_reference(th, ns, bonds, (2, 2), z), gt)
        return _loss(greens_function_ad(th, ns, bonds, (2, 2), z, sign_width=width, **kw), gt)

    p = torch.tensor([4.0, 0.3], dtype=torch.float64, device="cuda", requires_grad=True)
    loss_of(p).backward()
    grad = p.grad.cpu().numpy()
    p2 = p.detach().clone().requires_grad_(True)
    loss_of(p2, dense=True).backward()
    np.testing.assert_allclose(grad, p2.grad.cpu().numpy(), rtol=1e-6)
    fd = _fd(lambda q: loss_of(q).item(), p.detach(), 1e-5)
    np.testing.assert_allclose(grad, fd, rtol=1e-6)


def test_config_size_siam_fd(cuda):
    """One SIAM of the differentiated benchmark at full size (D = 63,504)."""
    from cmpy_gb300.adjoint import greens_function_ad, siam_parameters

    rng = np.random.default_rng(5)
    ek = rng.uniform(-2, 2, 30)
    z = 1j * (2 * np.arange(1024) + 1) * np.pi / 100.0
    gt = torch.as_tensor(1.0 / (z - np.sum(0.3**2 / (z[:, None] - ek[None, :]), axis=1))).cuda()
    eb0 = torch.tensor(rng.uniform(-2, 2, 9), dtype=torch.float64, device="cuda")
    v0 = torch.tensor(rng.uniform(0.1, 0.6, 9), dtype=torch.float64, device="cuda")
    kw = dict(gs_steps=250, gf_levels=150, ckpt=16)

    # parameters under test: U, eps_imp, eps_bath[0], v[0]
    def loss_of(p):
        eb = torch.cat([p[2:3], eb0[1:]])
        v = torch.cat([p[3:4], v0[1:]])
        th, ns, bonds, width = siam_parameters(p[0], p[1], eb, v)
        return _loss(greens_function_ad(th, ns, bonds, (5, 5), z, sign_width=width, **kw), gt)

    p = torch.tensor([4.0, 0.0, float(eb0[0]), float(v0[0])], dtype=torch.float64, device="cuda",
                     requires_grad=True)
    loss_of(p).backward()
    grad = p.grad.cpu().numpy()
    fd = _fd(lambda q: loss_of(q).item(), p.detach(), 1e-5)
    np.testing.assert_allclose(grad, fd, rtol=1e-6, atol=1e-9 * np.abs(fd).max())
