"""The native adjoint pieces (taped Lanczos, segment replay, reverse sweep, continued-fraction
adjoint) against their step-by-step torch restatement (tests/_adjoint_ref.py) on the same
inputs: same tape length, scalars and gradients to rounding (FP64, 1e-10 relative).

Without reorthogonalisation the two roundings drift apart exponentially once the Krylov basis
loses orthogonality (about 45 steps on these 400-dimensional sectors), so the step-by-step
comparisons stay at 30 steps or fewer; the long runs are compared through converged
quantities and through finite differences."""

import numpy as np
import pytest
import torch

import _adjoint_ref as R

pytestmark = pytest.mark.gpu


def _siam_plan(nbath, sector, seed):
    from cmpy_gb300.adjoint import plan_from_params, siam_parameters

    rng = np.random.default_rng(seed)
    eb = torch.tensor(rng.uniform(-2, 2, nbath), dtype=torch.float64, device="cuda")
    v = torch.tensor(rng.uniform(0.1, 0.6, nbath), dtype=torch.float64, device="cuda")
    u = torch.tensor(4.0, dtype=torch.float64, device="cuda")
    theta, n_sites, bonds, width = siam_parameters(u, torch.tensor(0.0, dtype=torch.float64, device="cuda"), eb, v)
    return plan_from_params(theta, n_sites, bonds, width, *sector), theta.numel()


def _start(dim, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.rand(dim, generator=g, dtype=torch.float64).cuda()


@pytest.mark.parametrize("c", [1, 5, 16])
def test_tape_forward_matches_torch(cuda, c):
    from cmpy_gb300.adjoint import tape_forward

    plan, _ = _siam_plan(5, (3, 3), 1)
    s = _start(plan.dim, 2)
    nat = tape_forward(plan, s, 30, c, tol=0.0)
    ref = R.lanczos_taped(plan, s, 30, c)
    assert nat.m == ref.m
    np.testing.assert_allclose(nat.alpha.cpu().numpy(), ref.alpha.cpu().numpy(), rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(nat.beta.cpu().numpy(), ref.beta.cpu().numpy(), rtol=1e-11, atol=1e-12)
    # checkpoints hold [q_{k-1}, q_k]
    for k in range(0, nat.m, c):
        qp, q = ref.ckpt[k]
        torch.testing.assert_close(nat.ckpt[k // c, 1], q, rtol=1e-7, atol=1e-9)
        if qp is None:
            assert torch.count_nonzero(nat.ckpt[k // c, 0]).item() == 0
        else:
            torch.testing.assert_close(nat.ckpt[k // c, 0], qp, rtol=1e-7, atol=1e-9)


def test_tape_forward_convergence_and_breakdown(cuda):
    from cmpy_gb300.adjoint import tape_forward

    plan, _ = _siam_plan(5, (3, 3), 3)
    s = _start(plan.dim, 4)
    nat = tape_forward(plan, s, 300, 8, tol=1e-12)
    ref = R.lanczos_taped(plan, s, 300, 8, tol=1e-12)
    assert nat.m == ref.m < 300
    # converged: the lowest Ritz values agree although the bases differ by rounding
    def lowest(t):
        a, b = t.alpha.cpu().numpy(), t.beta.cpu().numpy()
        T = np.diag(a) + np.diag(b[1:t.m], 1) + np.diag(b[1:t.m], -1)
        return np.linalg.eigvalsh(T)[0]

    assert abs(lowest(nat) - lowest(ref)) < 1e-11 * abs(lowest(ref))
    assert abs(lowest(nat) - torch.linalg.eigvalsh(plan.dense())[0].item()) < 1e-10
    # a start vector inside a 2-dimensional invariant subspace breaks down after 2 steps
    w, V = torch.linalg.eigh(plan.dense())
    s2 = V[:, 0] + 0.5 * V[:, 1]
    t2 = tape_forward(plan, s2, 50, 4)
    assert t2.m == 2
    # a zero start vector has no tape
    assert tape_forward(plan, torch.zeros(plan.dim, dtype=torch.float64, device="cuda"), 10, 4) is None


@pytest.mark.parametrize("c", [3, 16])
def test_tape_combine_matches_torch(cuda, c):
    from cmpy_gb300.adjoint import tape_combine, tape_forward

    plan, _ = _siam_plan(5, (3, 3), 5)
    s = _start(plan.dim, 6)
    nat = tape_forward(plan, s, 30, c)
    ref = R.lanczos_taped(plan, s, 30, c)
    coef = torch.linspace(-1.0, 1.0, nat.m, dtype=torch.float64, device="cuda")
    probe = _start(plan.dim, 7)
    y, dots = tape_combine(nat, coef=coef, probe=probe)
    yr = torch.zeros_like(y)
    dr = torch.zeros(nat.m, dtype=torch.float64, device="cuda")
    for s0 in sorted(ref.ckpt):
        qs = R._segment(plan, ref, s0, min(s0 + c, ref.m))
        for k in range(s0, min(s0 + c, ref.m)):
            yr += coef[k] * qs[k]
            dr[k] = torch.dot(qs[k], probe)
    torch.testing.assert_close(y, yr, rtol=1e-10, atol=1e-11)
    torch.testing.assert_close(dots, dr, rtol=1e-10, atol=1e-11)


@pytest.mark.parametrize("ext", [False, True])
def test_tape_reverse_matches_torch(cuda, ext):
    from cmpy_gb300.adjoint import tape_forward, tape_reverse

    plan, P = _siam_plan(5, (3, 3), 8)
    s = _start(plan.dim, 9)
    c = 6
    nat = tape_forward(plan, s, 25, c)
    ref = R.lanczos_taped(plan, s, 25, c)
    m = nat.m
    rng = np.random.default_rng(10)
    abar = torch.tensor(rng.standard_normal(m), dtype=torch.float64, device="cuda")
    bbar = torch.tensor(rng.standard_normal(m + 1), dtype=torch.float64, device="cuda")
    ec = torch.tensor(rng.standard_normal(m), dtype=torch.float64, device="cuda") if ext else None
    ev = _start(plan.dim, 11) if ext else None
    th = torch.zeros(P, dtype=torch.float64, device="cuda")
    sbar = tape_reverse(nat, abar, bbar, th, ext_coef=ec, ext_vec=ev)
    th_r = torch.zeros(P, dtype=torch.float64, device="cuda")
    qext = {k: ec[k] * ev for k in range(m)} if ext else None
    sbar_r = R.lanczos_reverse(plan, ref, abar, bbar, qext, th_r)
    scale = th_r.abs().max().item()
    torch.testing.assert_close(th, th_r, rtol=1e-8, atol=1e-9 * scale)
    torch.testing.assert_close(sbar, sbar_r, rtol=1e-8, atol=1e-9 * sbar_r.abs().max().item())


def test_tape_reverse_is_the_transpose_of_the_forward(cuda):
    """<start_bar, ds> equals the directional derivative of L = abar.alpha + bbar.beta along ds
    (central differences of the native forward)."""
    from cmpy_gb300.adjoint import tape_forward, tape_reverse

    plan, P = _siam_plan(4, (2, 3), 12)
    s = _start(plan.dim, 13)
    m = 12
    nat = tape_forward(plan, s, m, 4)
    rng = np.random.default_rng(14)
    abar = torch.tensor(rng.standard_normal(nat.m), dtype=torch.float64, device="cuda")
    bbar = torch.tensor(rng.standard_normal(nat.m + 1), dtype=torch.float64, device="cuda")
    bbar[-1] = 0.0  # the last residual norm feeds no Green's function; its adjoint is not propagated
    th = torch.zeros(P, dtype=torch.float64, device="cuda")
    sbar = tape_reverse(nat, abar, bbar, th)
    ds = _start(plan.dim, 15) - 0.5
    h = 1e-6

    def L(x):
        t = tape_forward(plan, x, m, 4)
        assert t.m == nat.m
        return (torch.dot(abar, t.alpha) + torch.dot(bbar, t.beta)).item()

    fd = (L(s + h * ds) - L(s - h * ds)) / (2 * h)
    assert abs(torch.dot(sbar, ds).item() - fd) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("sign", [1, -1])
def test_cf_adjoint_matches_torch(cuda, sign):
    from cmpy_gb300.adjoint import cf_adjoint

    rng = np.random.default_rng(20 + sign)
    m = 37
    alpha = torch.tensor(rng.uniform(-2, 2, m), dtype=torch.float64, device="cuda")
    beta = torch.tensor(rng.uniform(0.2, 1.5, m + 1), dtype=torch.float64, device="cuda")
    n2 = float(beta[0].item()) ** 2
    z = torch.as_tensor(1j * (2 * np.arange(300) + 1) * np.pi / 40.0 + 0.1).cuda()
    gbar = torch.as_tensor(rng.standard_normal(300) + 1j * rng.standard_normal(300)).cuda()
    e0 = -3.25
    abar, bbar, e0bar = cf_adjoint(alpha, beta, n2, z, e0, sign, gbar)
    _, abar_r, bbar_r, e0bar_r = R.cf_adjoint(alpha, beta, torch.tensor(n2, dtype=torch.float64, device="cuda"), z,
                                              torch.tensor(e0, dtype=torch.float64, device="cuda"), sign, gbar)
    torch.testing.assert_close(abar, abar_r, rtol=1e-11, atol=1e-13)
    torch.testing.assert_close(bbar, bbar_r, rtol=1e-11, atol=1e-13)
    assert abs(e0bar.item() - e0bar_r.item()) < 1e-11 * max(1.0, abs(e0bar_r.item()))


def _batch_thetas(B, nbath, seed):
    from cmpy_gb300.adjoint import siam_parameters

    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(B):
        eb = torch.tensor(rng.uniform(-2, 2, nbath), dtype=torch.float64, device="cuda")
        v = torch.tensor(rng.uniform(0.1, 0.6, nbath), dtype=torch.float64, device="cuda")
        th, n_sites, bonds, width = siam_parameters(torch.tensor(4.0, dtype=torch.float64, device="cuda"),
                                                    torch.tensor(0.0, dtype=torch.float64, device="cuda"), eb, v)
        rows.append(th)
    return torch.stack(rows).contiguous(), n_sites, bonds, width


def test_batch_matvec_bit_identical_to_single(cuda):
    """H(theta_b) x_b of the batched kernel equals each problem's own plan matvec bit for bit."""
    from cmpy_gb300.adjoint import batch_diag, batch_matvec, plan_from_params, structure_plan

    thetas, n_sites, bonds, width = _batch_thetas(4, 5, 31)
    sp = structure_plan(n_sites, bonds, width, 3, 3)
    diag = batch_diag(sp, thetas)
    X = torch.rand((4, sp.dim), dtype=torch.float64, device="cuda") - 0.5
    Y = batch_matvec(sp, thetas, diag, X)
    for b in range(4):
        p = plan_from_params(thetas[b], n_sites, bonds, width, 3, 3)
        assert torch.equal(Y[b], p.matvec(X[b]))


def test_batch_tape_matches_single(cuda):
    from cmpy_gb300.adjoint import (batch_diag, batch_tape_combine, batch_tape_forward, batch_tape_reverse,
                                    plan_from_params, structure_plan, tape_combine, tape_forward, tape_reverse)

    B, c = 3, 5
    thetas, n_sites, bonds, width = _batch_thetas(B, 5, 32)
    P = thetas.shape[1]
    sp = structure_plan(n_sites, bonds, width, 3, 3)
    diag = batch_diag(sp, thetas)
    starts = torch.stack([_start(sp.dim, 40 + b) for b in range(B)])
    bt = batch_tape_forward(sp, thetas, diag, starts, 25, c)
    rng = np.random.default_rng(33)
    coef = torch.tensor(rng.standard_normal((B, bt.K)), dtype=torch.float64, device="cuda")
    probe = torch.rand((B, sp.dim), dtype=torch.float64, device="cuda")
    Yb, Db = batch_tape_combine(bt, coef=coef, probe=probe)
    abar = torch.tensor(rng.standard_normal((B, bt.K)), dtype=torch.float64, device="cuda")
    bbar = torch.tensor(rng.standard_normal((B, bt.K + 1)), dtype=torch.float64, device="cuda")
    ec = torch.tensor(rng.standard_normal((B, bt.K)), dtype=torch.float64, device="cuda")
    ev = torch.rand((B, sp.dim), dtype=torch.float64, device="cuda")
    thb = torch.zeros((B, P), dtype=torch.float64, device="cuda")
    sb = batch_tape_reverse(bt, abar, bbar, thb, ext_coef=ec, ext_vec=ev)
    for b in range(B):
        p = plan_from_params(thetas[b], n_sites, bonds, width, 3, 3)
        t = tape_forward(p, starts[b], 25, c)
        assert bt.m[b] == t.m
        m = t.m
        torch.testing.assert_close(bt.alpha[b, :m], t.alpha, rtol=1e-12, atol=1e-13)
        torch.testing.assert_close(bt.beta[b, :m + 1], t.beta, rtol=1e-12, atol=1e-13)
        y, d = tape_combine(t, coef=coef[b, :m], probe=probe[b])
        torch.testing.assert_close(Yb[b], y, rtol=1e-10, atol=1e-11)
        torch.testing.assert_close(Db[b, :m], d, rtol=1e-10, atol=1e-11)
        th = torch.zeros(P, dtype=torch.float64, device="cuda")
        s1 = tape_reverse(t, abar[b, :m], bbar[b, :m + 1], th, ext_coef=ec[b, :m], ext_vec=ev[b])
        torch.testing.assert_close(thb[b], th, rtol=1e-8, atol=1e-9 * th.abs().max().item())
        torch.testing.assert_close(sb[b], s1, rtol=1e-8, atol=1e-9 * s1.abs().max().item())


def test_batch_tape_ragged_lengths(cuda):
    """Problems of one batch stop at different steps (convergence, an eigenvector start that
    breaks down after one step, a zero start vector); each keeps its own tape length."""
    from cmpy_gb300.adjoint import batch_diag, batch_tape_forward, plan_from_params, structure_plan, tape_forward

    B = 3
    thetas, n_sites, bonds, width = _batch_thetas(B, 5, 34)
    sp = structure_plan(n_sites, bonds, width, 3, 3)
    diag = batch_diag(sp, thetas)
    p1 = plan_from_params(thetas[1], n_sites, bonds, width, 3, 3)
    w, V = torch.linalg.eigh(p1.dense())
    starts = torch.stack([_start(sp.dim, 50), V[:, 0], torch.zeros(sp.dim, dtype=torch.float64, device="cuda")])
    bt = batch_tape_forward(sp, thetas, diag, starts, 300, 8, tol=1e-12)
    assert bt.m[1] == 1 and bt.m[2] == 0
    assert abs(bt.alpha[1, 0].item() - w[0].item()) < 1e-12 * abs(w[0].item())
    t0 = tape_forward(plan_from_params(thetas[0], n_sites, bonds, width, 3, 3), starts[0], 300, 8, tol=1e-12)
    assert bt.m[0] == t0.m < 300


def test_batch_continued_fraction_matches_single(cuda):
    from cmpy_gb300 import engine as E
    from cmpy_gb300.adjoint import (batch_cf, batch_cf_adjoint, batch_diag, batch_tape_forward, cf_adjoint,
                                    structure_plan)

    B = 3
    thetas, n_sites, bonds, width = _batch_thetas(B, 5, 35)
    sp = structure_plan(n_sites, bonds, width, 3, 3)
    starts = torch.stack([_start(sp.dim, 60 + b) for b in range(B)])
    bt = batch_tape_forward(sp, thetas, batch_diag(sp, thetas), starts, 40, 8)
    zt = torch.as_tensor(1j * (2 * np.arange(100) + 1) * np.pi / 30.0 + 0.05).cuda()
    n2 = bt.beta[:, 0].cpu().numpy() ** 2
    e0 = np.array([-3.0, -2.5, -4.0])
    g = torch.zeros((B, zt.numel()), dtype=torch.complex128, device="cuda")
    batch_cf(bt, n2, e0, -1, zt, g)
    gbar = torch.rand((B, zt.numel()), dtype=torch.complex128, device="cuda")
    Ab, Bb, eb = batch_cf_adjoint(bt, n2, e0, -1, zt, gbar)
    for b in range(B):
        m = bt.m[b]
        gs = E.continued_fraction(bt.alpha[b, :m], bt.beta[b, :m + 1], float(n2[b]), zt, float(e0[b]), -1)
        assert torch.equal(g[b], gs)
        ab, bb, e = cf_adjoint(bt.alpha[b, :m], bt.beta[b, :m + 1], float(n2[b]), zt, float(e0[b]), -1, gbar[b])
        assert torch.equal(Ab[b, :m], ab) and torch.equal(Bb[b, :m + 1], bb) and eb[b].item() == e.item()
