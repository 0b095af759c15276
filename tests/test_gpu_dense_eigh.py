"""GPU parity of the library's dense symmetric eigensolver (ed_dense_eigh_batch: Householder
tridiagonalisation, Sturm multisection, inverse iteration re-orthogonalised within clusters,
back-transformation) and of the tridiagonal one (ed_tridiag_eigh), against numpy / scipy
(LAPACK) on the CPU.

Tolerances: eigenvalues 1e-12 relative to the spectral radius; residual ||A v - lambda v|| and
orthogonality ||V^T V - I|| (max abs) 1e-11. Degenerate spectra (identity, repeated blocks, a
Hubbard sector with its symmetries) must still give an orthonormal eigenbasis; in every case
the spectral projector sum_i lambda_i v_i v_i^T reproduces A.
"""

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu

TOL_W = 1e-12
TOL_V = 1e-11


def _check(A, w, V):
    w = w.cpu().numpy()
    V = V.cpu().numpy()
    n = A.shape[0]
    scale = max(1.0, np.max(np.abs(np.linalg.eigvalsh(A))))
    assert np.all(np.diff(w) >= -TOL_W * scale)
    np.testing.assert_allclose(w, np.linalg.eigvalsh(A), rtol=0, atol=TOL_W * scale)
    assert np.max(np.abs(A @ V - V * w)) <= TOL_V * scale
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= TOL_V
    assert np.max(np.abs((V * w) @ V.T - A)) <= TOL_V * scale


def _rand_sym(n, seed):
    a = np.random.default_rng(seed).standard_normal((n, n))
    return (a + a.T) / 2


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 64, 255, 400])
def test_random_symmetric(cuda, n):
    from cmpy_gb300 import engine as E

    A = _rand_sym(n, n)
    w, V = E.dense_eigh(torch.as_tensor(A).cuda())
    _check(A, w, V)


def test_degenerate_spectra(cuda):
    from cmpy_gb300 import engine as E

    blk = _rand_sym(7, 3)
    cases = [
        np.eye(9) * 2.5,
        np.kron(np.eye(4), blk),                      # every eigenvalue four-fold
        sla.block_diag(blk, blk, _rand_sym(5, 4), blk),
        np.diag([1.0, 1.0, 1.0, 2.0, 2.0, 3.0]),
        np.zeros((4, 4)),
    ]
    for A in cases:
        w, V = E.dense_eigh(torch.as_tensor(A).cuda())
        _check(A, w, V)


def test_batch_of_mixed_sizes(cuda):
    from cmpy_gb300 import engine as E

    mats = [_rand_sym(n, 10 + n) for n in (1, 4, 33, 100, 2, 71)]
    out = E.dense_eigh_batch([torch.as_tensor(a).cuda() for a in mats])
    for A, (w, V) in zip(mats, out):
        _check(A, w, V)


@pytest.mark.parametrize("nu,nd", [(3, 3), (2, 3), (4, 4)])
def test_hubbard_sectors_vs_oracle(cuda, nu, nd):
    """Sectors of the 6-site ring (many degeneracies: translations and reflections) and of the
    8-site open chain (4,4): eigenvalues vs numpy on the oracle's dense matrix."""
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import ChainLattice, HubbardModel

    n_sites = 8 if (nu, nd) == (4, 4) else 6
    m = HubbardModel(ChainLattice(n_sites, n_sites == 6), inter=4.0, mu=2.0, hop=1.0)
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(n_sites, nu), O.sector_states(n_sites, nd)
    H = O.dense_from_coo(len(up) * len(dn), *O.coo_fermion(up, dn, eps, u, bonds, width))
    w, V = E.dense_eigh(torch.as_tensor(H).cuda())
    _check(H, w, V)


def test_solve_sector_uses_library_solver(cuda):
    """exactdiag's dense path (solve_sector) gives the oracle's eigenvalues."""
    from cmpy_gb300.exactdiag import _dense_eigh
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(6), inter=4.0, mu=2.0, hop=1.0)
    w, V = _dense_eigh(m.plan(3, 2))
    eps, u, bonds, width = m.fermion_descriptor()
    up, dn = O.sector_states(6, 3), O.sector_states(6, 2)
    H = O.dense_from_coo(len(up) * len(dn), *O.coo_fermion(up, dn, eps, u, bonds, width))
    _check(H, w, V)


@pytest.mark.parametrize("m", [1, 2, 50, 600])
def test_tridiagonal(cuda, m):
    from cmpy_gb300 import engine as E

    rng = np.random.default_rng(m)
    a = rng.standard_normal(m)
    b = np.concatenate([[0.0], rng.standard_normal(m - 1)])
    if m > 10:
        b[m // 2] = 0.0  # a split: the two blocks may share eigenvalues
        a[m // 2:] = a[: m - m // 2]
        b[m // 2 + 1:] = b[1: m - m // 2]
    w, V = E.tridiag_eigh(torch.as_tensor(a).cuda(), torch.as_tensor(b).cuda())
    T = np.diag(a) + np.diag(b[1:], 1) + np.diag(b[1:], -1)
    _check(T, w, V)


def test_invalid_arguments(cuda):
    from cmpy_gb300 import _native as N
    from cmpy_gb300 import engine as E

    with pytest.raises(ValueError):
        E.dense_eigh_batch([torch.zeros((3, 4), dtype=torch.float64, device="cuda")])
    a = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    w = torch.empty(4, dtype=torch.float64, device="cuda")
    import ctypes as C

    hn = (C.c_int * 1)(5)  # order above n_max
    st = N.lib().ed_dense_eigh_batch(N.ptr(a), 4, 16, hn, 1, 4, N.ptr(w), N.ptr(a), 4, 16, None)
    assert st == N.ED_ERR_INVALID_ARG


def test_tridiagonal_beyond_shared_memory(cuda):
    """m = 6000: the inverse-iteration arrays (5 m doubles) no longer fit in one CTA's shared
    memory, so the eigenvectors take the kernel with global work arrays; eigenvalues and
    eigenpair residuals against LAPACK."""
    from cmpy_gb300 import engine as E

    m = 6000
    rng = np.random.default_rng(6000)
    a = rng.standard_normal(m)
    b = np.concatenate([[0.0], rng.standard_normal(m - 1)])
    w, V = E.tridiag_eigh(torch.as_tensor(a).cuda(), torch.as_tensor(b).cuda())
    w, V = w.cpu().numpy(), V.cpu().numpy()
    w_ref = sla.eigh_tridiagonal(a, b[1:], eigvals_only=True)
    scale = np.max(np.abs(w_ref))
    np.testing.assert_allclose(w, w_ref, rtol=0, atol=TOL_W * scale)
    TV = a[:, None] * V
    TV[:-1] += b[1:, None] * V[1:]
    TV[1:] += b[1:, None] * V[:-1]
    assert np.max(np.abs(TV - V * w)) <= TOL_V * scale
    # orthogonality of 200 random eigenvectors: pairs closer than the cluster tolerance are
    # re-orthogonalised; for close pairs above it inverse iteration's orthogonality error is
    # ~ eps ||T|| / gap (smallest gaps ~1e-7 among 6000 values), hence 1e-8
    cols = rng.choice(m, 200, replace=False)
    G = V[:, cols].T @ V[:, cols]
    assert np.max(np.abs(G - np.eye(len(cols)))) <= 1e-8


_FORMS = """
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np, torch
from cmpy_gb300 import engine as E
import test_gpu_dense_eigh as T
for n in (200, 300):
    A = T._rand_sym(n, n + 1)
    w, V = E.dense_eigh(torch.as_tensor(A).cuda())
    T._check(A, w, V)
mats = [T._rand_sym(n, 7 * n) for n in (150, 300, 260)]
for A, (w, V) in zip(mats, E.dense_eigh_batch([torch.as_tensor(a).cuda() for a in mats])):
    T._check(A, w, V)
print("forms ok")
"""


@pytest.mark.parametrize("form", ["16", "8", "0"])
def test_householder_forms(cuda, form):
    """Orders 150-300 through each Householder form, forced in a fresh process: a cluster of 16
    CTAs per matrix, of 8 (the portable size, used where 16 cannot be scheduled), and the
    per-step launches."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    code = _FORMS.format(root=str(root), tests=str(root / "tests"))
    env = dict(os.environ, CMPY_ED_HH_CLUSTER=form)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "forms ok" in r.stdout
