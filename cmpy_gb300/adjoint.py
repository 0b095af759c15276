"""Adjoint (reverse-mode) zero-temperature Green's function behind torch.autograd.

No reference counterpart: cmpy has no derivatives. Its use is fitting Anderson bath
parameters (cmpy/models/anderson.py:24-164) for the DMFT loop (cmpy/dmft/twosite.py:103-172).

Forward, for a sector (n_up, n_dn) of a fermionic model with parameters
theta = [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}] (the plan's order):
  1. ground-state Lanczos (m0 steps) -> T0 -> lowest eigenpair (E0, c) -> psi0 = Q c/||Q c||;
  2. phi = c^dag_{pos,sigma} psi0, chi = c_{pos,sigma} psi0;
  3. Lanczos of phi in the (n+1) sector and of chi in the (n-1) sector;
  4. G(z) = CF_particle(z) + CF_hole(z)  (continued fractions, z' = +-z + E0).
Every Lanczos run is a native tape (ed_lanczos_tape): it keeps its scalars and the Krylov
vectors q_k at k = 0 (mod c) (with q_{k-1}); the backward pass (ed_tape_reverse) recomputes
each segment of c vectors from its checkpoint with the stored (alpha, beta), bit-identical to
the forward, and sweeps the adjoint recurrence backwards through it. Memory: about 2m/c + 2c
vectors per run instead of m. The host only enqueues kernels and reads m.

Backward (exact reverse of the computed recurrences):
  * continued fraction: dG/dalpha_l, dG/dbeta_l, dG/dnorm^2, dG/dE0 by the chain through
    t_l = z' - alpha_l - beta_{l+1}^2 / t_{l+1};
  * Lanczos step k (w = H q_k, alpha = q.w, r = w - alpha q_k - beta_k q_{k-1},
    beta_{k+1} = ||r||, q_{k+1} = r / beta_{k+1}) reversed, with
    theta_bar += wbar_k^T (dH/dtheta) q_k (fused into the step's elementwise kernel) and
    qbar_k += H wbar_k;
  * Ritz vector and tridiagonal eigenpair: Tbar = Ebar c c^T + v c^T, v = -(T - E0)^+ cbar
    (the eigenpair and this m x m solve run on the device, ed_tridiag_lowest_batch and
    ed_tridiag_pinv_solve_batch).
Costs: forward = m0 + m_p + m_h matvecs; backward = one matvec per step for the segment
recompute plus one for H wbar, i.e. about 2x the forward.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import engine as E

__all__ = ["Tape", "tape_forward", "tape_combine", "tape_reverse", "cf_adjoint", "greens_function_ad",
           "greens_function_ad_batch", "GreensFunctionAD", "GreensFunctionADBatch", "siam_parameters", "sandwich",
           "BatchTape", "structure_plan", "batch_diag", "batch_matvec", "batch_tape_forward", "batch_tape_combine",
           "batch_tape_reverse"]


# ------------------------------------------------------------------------------------------
# plan construction from a flat parameter vector
# ------------------------------------------------------------------------------------------


def plan_from_params(theta: torch.Tensor, n_sites: int, bonds, sign_width: int, n_up: int, n_dn: int) -> E.Plan:
    th = theta.detach().double().cpu().numpy()
    eps = th[:n_sites]
    u = th[n_sites:2 * n_sites]
    t = th[2 * n_sites:]
    return E.Plan.fermion(n_sites, eps, u, [(i, j, float(tb)) for (i, j), tb in zip(bonds, t)], n_up, n_dn,
                          sign_width)


def sandwich(plan: E.Plan, a: torch.Tensor, b: torch.Tensor, out: torch.Tensor) -> None:
    """out += a^T (dH/dtheta) b for every parameter (device kernel)."""
    N.check(N.lib().ed_param_sandwich(plan.handle, N.ptr(a), N.ptr(b), N.ptr(out), 1, E._stream()))


# ------------------------------------------------------------------------------------------
# native tape: taped FP64 Lanczos, segment replay, reverse sweep (csrc/ed_adjoint.cu)
# ------------------------------------------------------------------------------------------


@dataclass
class Tape:
    """A taped Lanczos run of `plan`: alpha[m], beta[m+1] (beta[0] = ||start||), the
    checkpoint pairs [q_{k-1}, q_k] for k = 0 (mod c), and the shared workspace."""
    plan: E.Plan
    alpha: torch.Tensor
    beta: torch.Tensor
    ckpt: torch.Tensor
    m: int
    c: int
    work: torch.Tensor


def _workspace(plan: E.Plan, steps: int, c: int) -> torch.Tensor:
    nb = C.c_size_t()
    N.check(N.lib().ed_tape_workspace(plan.handle, int(steps), int(c), C.byref(nb)))
    return torch.empty(int(nb.value), dtype=torch.uint8, device=E.device())


def tape_forward(plan: E.Plan, start: torch.Tensor, max_steps: int, c: int = 16, tol: float = 0.0,
                 check_every: int = 10, breakdown: float = 1e-13) -> Tape | None:
    """Taped Lanczos from `start` (None for a zero start vector). Stops on breakdown and,
    with tol > 0, once the lowest Ritz pair has residual <= tol * max(1, |E|)."""
    with plan._dev():
        s = start.reshape(-1).to(dtype=torch.float64).contiguous()
        K = int(min(max_steps, plan.dim))
        work = _workspace(plan, K, c)
        alpha = torch.empty(K, dtype=torch.float64, device=E.device())
        beta = torch.empty(K + 1, dtype=torch.float64, device=E.device())
        ckpt = torch.empty(((K + c - 1) // c, 2, plan.dim), dtype=torch.float64, device=E.device())
        steps = C.c_int()
        N.check(N.lib().ed_lanczos_tape(plan.handle, N.ptr(s), K, int(c), float(tol), int(check_every),
                                        float(breakdown), N.ptr(work), work.numel(), N.ptr(alpha), N.ptr(beta),
                                        N.ptr(ckpt), C.byref(steps), E._stream()))
        m = int(steps.value)
        if m == 0:
            return None
        return Tape(plan, alpha[:m], beta[:m + 1], ckpt, m, int(c), work)


def tape_combine(tape: Tape, coef: torch.Tensor | None = None, probe: torch.Tensor | None = None):
    """Replays the tape: (sum_k coef_k q_k or None, [q_k . probe]_k or None)."""
    p = tape.plan
    with p._dev():
        out = torch.empty(p.dim, dtype=torch.float64, device=E.device()) if coef is not None else None
        dots = torch.empty(tape.m, dtype=torch.float64, device=E.device()) if probe is not None else None
        cf = coef.to(dtype=torch.float64).contiguous() if coef is not None else None
        pr = probe.reshape(-1).to(dtype=torch.float64).contiguous() if probe is not None else None
        N.check(N.lib().ed_tape_combine(p.handle, tape.m, tape.c, N.ptr(tape.alpha), N.ptr(tape.beta),
                                        N.ptr(tape.ckpt), N.ptr(cf), N.ptr(out), N.ptr(pr), N.ptr(dots),
                                        N.ptr(tape.work), tape.work.numel(), E._stream()))
        return out, dots


def tape_reverse(tape: Tape, abar: torch.Tensor, bbar: torch.Tensor, theta_bar: torch.Tensor,
                 ext_coef: torch.Tensor | None = None, ext_vec: torch.Tensor | None = None) -> torch.Tensor:
    """Reverse sweep: accumulates dL/dtheta into theta_bar, returns dL/dstart. abar[m] and
    bbar[m+1] are the adjoints of the tape's scalars (bbar[0]: of ||start||); the Krylov
    vectors get the external adjoints q_bar_k += ext_coef[k] * ext_vec."""
    p = tape.plan
    with p._dev():
        ab = abar.to(dtype=torch.float64).contiguous()
        bb = bbar.to(dtype=torch.float64).contiguous()
        ec = ext_coef.to(dtype=torch.float64).contiguous() if ext_coef is not None else None
        ev = ext_vec.reshape(-1).to(dtype=torch.float64).contiguous() if ext_vec is not None else None
        sbar = torch.empty(p.dim, dtype=torch.float64, device=E.device())
        N.check(N.lib().ed_tape_reverse(p.handle, tape.m, tape.c, N.ptr(tape.alpha), N.ptr(tape.beta),
                                        N.ptr(tape.ckpt), N.ptr(ab), N.ptr(bb), N.ptr(ec), N.ptr(ev),
                                        N.ptr(tape.work), tape.work.numel(), N.ptr(theta_bar), N.ptr(sbar),
                                        E._stream()))
        return sbar


def cf_adjoint(alpha: torch.Tensor, beta: torch.Tensor, n2: float, z: torch.Tensor, e0: float, sign: int,
               gbar: torch.Tensor):
    """Adjoints (abar[m], bbar[m+1] with bbar[0] for sqrt(n2), e0bar) of
    L = Re sum conj(gbar) G for G = sign n2 / (z' - alpha_0 - beta_1^2 / ...), z' = sign z + e0."""
    m = alpha.numel()
    abar = torch.empty(m, dtype=torch.float64, device=E.device())
    bbar = torch.empty(m + 1, dtype=torch.float64, device=E.device())
    scal = torch.empty(2, dtype=torch.float64, device=E.device())
    zt = E._as_dev_c128(z)
    gb = E._as_dev_c128(gbar)
    N.check(N.lib().ed_cf_adjoint(N.ptr(alpha), N.ptr(beta), m, float(n2), float(e0), int(sign),
                                  N.ptr(torch.view_as_real(zt)), zt.numel(), N.ptr(torch.view_as_real(gb)),
                                  N.ptr(abar), N.ptr(bbar), N.ptr(scal), E._stream()))
    return abar, bbar, scal[0]


# ------------------------------------------------------------------------------------------
# the autograd function
# ------------------------------------------------------------------------------------------


def _gf_forward(theta: torch.Tensor, spec, zt: torch.Tensor, g: torch.Tensor):
    """Forward of one problem on the current stream: adds G(z) into g, returns what the
    backward needs."""
    n_sites, bonds, width, (nu, nd), pos, sigma, m0, mgf, c, seed = spec
    plan = plan_from_params(theta, n_sites, bonds, width, nu, nd)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    v0 = torch.rand(plan.dim, generator=gen, dtype=torch.float64).to(E.device())
    tape0 = tape_forward(plan, v0, m0, c, tol=1e-12)
    m = tape0.m
    e0_d, vecs = E.tridiag_lowest_batch(tape0.alpha[None, :m], tape0.beta[None, :m + 1], [m])
    e0 = float(e0_d[0])
    cvec = vecs[0, :m].contiguous()
    y, _ = tape_combine(tape0, coef=cvec)
    ynorm = torch.linalg.norm(y)
    psi = y / ynorm
    parts = []
    for delta, create, sign in ((1, True, 1), (-1, False, -1)):
        tu, td = (nu + delta, nd) if sigma == 1 else (nu, nd + delta)
        if not (0 <= tu <= n_sites and 0 <= td <= n_sites):
            parts.append(None)
            continue
        tp = plan_from_params(theta, n_sites, bonds, width, tu, td)
        start = plan.apply_fermion(tp, pos, sigma, create, psi)
        tape = tape_forward(tp, start, mgf, c)
        if tape is None:
            parts.append(None)
            continue
        n2 = float(tape.beta[0].item()) ** 2
        E.continued_fraction(tape.alpha, tape.beta, n2, zt, e0, sign, out=g)
        parts.append((tp, tape, sign, create, n2))
    return (plan, tape0, e0_d, cvec, e0, ynorm, psi, zt, parts, spec)


def _gf_backward(saved, gbar: torch.Tensor) -> torch.Tensor:
    """Backward of one problem on the current stream: dL/dtheta for L = Re sum conj(gbar) G."""
    plan, tape0, e0_d, cvec, e0, ynorm, psi, zt, parts, spec = saved
    n_sites, bonds, width, (nu, nd), pos, sigma, m0, mgf, c, seed = spec
    P = 2 * n_sites + len(bonds)
    theta_bar = torch.zeros(P, dtype=torch.float64, device=E.device())
    e0bar = 0.0
    psibar = torch.zeros_like(psi)
    gb = gbar.to(E.device()).contiguous()
    for part in parts:
        if part is None:
            continue
        tp, tape, sign, create, n2 = part
        abar, bbar, eb = cf_adjoint(tape.alpha, tape.beta, n2, zt, e0, sign, gb)
        e0bar += float(eb.item())
        sbar = tape_reverse(tape, abar, bbar, theta_bar)
        # start = c^dag psi (or c psi): its adjoint maps back with the opposite operator
        psibar = psibar + tp.apply_fermion(plan, pos, sigma, not create, sbar)
    # psi = y / ||y||, y = sum_k c_k q_k
    ybar = (psibar - torch.dot(psibar, psi) * psi) / ynorm
    m = tape0.m
    _, cbar = tape_combine(tape0, probe=ybar)
    # eigenpair of T: E0 = c^T T c, c = ground state of T; v = -(T - E0)^+ cbar on the
    # complement of c (device solve)
    v = E.tridiag_pinv_solve_batch(tape0.alpha[None, :m], tape0.beta[None, :m + 1], [m], e0_d, cvec[None],
                                   cbar[None, :m].contiguous())[0]
    dev = E.device()
    abar0 = e0bar * cvec ** 2 + v * cvec
    bbar0 = torch.zeros(m + 1, dtype=torch.float64, device=dev)
    if m > 1:
        bbar0[1:m] = 2.0 * e0bar * cvec[:-1] * cvec[1:] + v[:-1] * cvec[1:] + v[1:] * cvec[:-1]
    tape_reverse(tape0, abar0.contiguous(), bbar0, theta_bar, ext_coef=cvec, ext_vec=ybar)
    return theta_bar


class GreensFunctionAD(torch.autograd.Function):
    """G(z) of a fermionic model sector as a differentiable function of theta."""

    @staticmethod
    def forward(ctx, theta, spec, z):
        zt = E._as_dev_c128(z)
        g = torch.zeros_like(zt)
        ctx.saved = _gf_forward(theta, spec, zt, g)
        return g

    @staticmethod
    def backward(ctx, gbar):
        return _gf_backward(ctx.saved, gbar).to(gbar.device), None, None


# ------------------------------------------------------------------------------------------
# batched native tape: B problems of one structure per launch (csrc/ed_adjoint_batch.cu)
# ------------------------------------------------------------------------------------------


def structure_plan(n_sites: int, bonds, sign_width: int, n_up: int, n_dn: int) -> E.Plan:
    """Plan of a sector with t = 1 on every bond and eps = U = 0: its hop coefficients are the
    fermionic signs, the structure shared by every parameter set."""
    z = np.zeros(n_sites)
    return E.Plan.fermion(n_sites, z, z, [(i, j, 1.0) for (i, j) in bonds], n_up, n_dn, sign_width)


@dataclass
class BatchTape:
    """B taped Lanczos runs of one structure: alpha[B, K], beta[B, K+1], checkpoints
    [slot, 2, B, D], the tape lengths m[b] and the shared workspace."""
    plan: E.Plan
    thetas: torch.Tensor
    diag: torch.Tensor
    alpha: torch.Tensor
    beta: torch.Tensor
    ckpt: torch.Tensor
    m: list
    K: int
    c: int
    work: torch.Tensor


def batch_diag(plan: E.Plan, thetas: torch.Tensor) -> torch.Tensor:
    B = thetas.shape[0]
    diag = torch.empty((B, plan.dim), dtype=torch.float64, device=E.device())
    N.check(N.lib().ed_batch_diag(plan.handle, B, N.ptr(thetas), N.ptr(diag), E._stream()))
    return diag


def batch_matvec(plan: E.Plan, thetas: torch.Tensor, diag: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    """y[b] = H(theta_b) x[b]."""
    y = torch.empty_like(x)
    N.check(N.lib().ed_batch_matvec_params(plan.handle, thetas.shape[0], N.ptr(thetas), N.ptr(diag), N.ptr(x),
                                           N.ptr(y), E._stream()))
    return y


def batch_tape_forward(plan: E.Plan, thetas: torch.Tensor, diag: torch.Tensor, starts: torch.Tensor, max_steps: int,
                       c: int = 16, tol: float = 0.0, check_every: int = 10,
                       breakdown: float = 1e-13) -> BatchTape:
    B = thetas.shape[0]
    K = int(min(max_steps, plan.dim))
    nb = C.c_size_t()
    N.check(N.lib().ed_batch_tape_workspace(plan.handle, B, K, int(c), C.byref(nb)))
    work = torch.empty(int(nb.value), dtype=torch.uint8, device=E.device())
    alpha = torch.empty((B, K), dtype=torch.float64, device=E.device())
    beta = torch.empty((B, K + 1), dtype=torch.float64, device=E.device())
    ckpt = torch.empty(((K + c - 1) // c, 2, B, plan.dim), dtype=torch.float64, device=E.device())
    steps = (C.c_int * B)()
    st = starts.to(dtype=torch.float64).contiguous()
    N.check(N.lib().ed_batch_lanczos_tape(plan.handle, B, N.ptr(thetas), N.ptr(diag), N.ptr(st), K, int(c),
                                          float(tol), int(check_every), float(breakdown), N.ptr(work), work.numel(),
                                          N.ptr(alpha), N.ptr(beta), N.ptr(ckpt), steps, E._stream()))
    return BatchTape(plan, thetas, diag, alpha, beta, ckpt, [int(v) for v in steps], K, int(c), work)


def _hm(tape: BatchTape):
    return (C.c_int * len(tape.m))(*tape.m)


def batch_tape_combine(tape: BatchTape, coef: torch.Tensor | None = None, probe: torch.Tensor | None = None):
    """Replays B tapes: (rows sum_k coef[b, k] q_k[b] or None, dots[b, k] = q_k[b] . probe[b] or None)."""
    p, B = tape.plan, len(tape.m)
    out = torch.empty((B, p.dim), dtype=torch.float64, device=E.device()) if coef is not None else None
    dots = torch.zeros((B, tape.K), dtype=torch.float64, device=E.device()) if probe is not None else None
    cf = coef.to(dtype=torch.float64).contiguous() if coef is not None else None
    pr = probe.to(dtype=torch.float64).contiguous() if probe is not None else None
    N.check(N.lib().ed_batch_tape_combine(p.handle, B, N.ptr(tape.thetas), N.ptr(tape.diag), _hm(tape), tape.K, tape.c,
                                          N.ptr(tape.alpha), N.ptr(tape.beta), N.ptr(tape.ckpt), N.ptr(cf), N.ptr(out),
                                          N.ptr(pr), N.ptr(dots), N.ptr(tape.work), tape.work.numel(), E._stream()))
    return out, dots


def batch_tape_reverse(tape: BatchTape, abar: torch.Tensor, bbar: torch.Tensor, theta_bar: torch.Tensor,
                       ext_coef: torch.Tensor | None = None, ext_vec: torch.Tensor | None = None) -> torch.Tensor:
    """Reverse sweep of B tapes: theta_bar[b] += dL/dtheta_b; returns dL/dstart [B, D]."""
    p, B = tape.plan, len(tape.m)
    ab = abar.to(dtype=torch.float64).contiguous()
    bb = bbar.to(dtype=torch.float64).contiguous()
    ec = ext_coef.to(dtype=torch.float64).contiguous() if ext_coef is not None else None
    ev = ext_vec.to(dtype=torch.float64).contiguous() if ext_vec is not None else None
    sbar = torch.empty((B, p.dim), dtype=torch.float64, device=E.device())
    N.check(N.lib().ed_batch_tape_reverse(p.handle, B, N.ptr(tape.thetas), N.ptr(tape.diag), _hm(tape), tape.K,
                                          tape.c, N.ptr(tape.alpha), N.ptr(tape.beta), N.ptr(tape.ckpt), N.ptr(ab),
                                          N.ptr(bb), N.ptr(ec), N.ptr(ev), N.ptr(tape.work), tape.work.numel(),
                                          N.ptr(theta_bar), N.ptr(sbar), E._stream()))
    return sbar


def batch_cf(tape: BatchTape, n2: np.ndarray, e0: np.ndarray, sign: int, zt: torch.Tensor, g: torch.Tensor) -> None:
    """g[b] += the continued fraction of tape b (norm^2 n2[b], shift e0[b]), every problem in
    one launch."""
    B, dev = len(tape.m), E.device()
    m_d = torch.tensor(tape.m, dtype=torch.int32, device=dev)
    n2_d = torch.as_tensor(np.asarray(n2, dtype=np.float64)).to(dev)
    e0_d = torch.as_tensor(np.asarray(e0, dtype=np.float64)).to(dev)
    N.check(N.lib().ed_batch_cf(B, N.ptr(tape.alpha), tape.K, N.ptr(tape.beta), tape.K + 1, N.ptr(m_d), N.ptr(n2_d),
                                N.ptr(e0_d), int(sign), N.ptr(torch.view_as_real(zt)), zt.numel(),
                                N.ptr(torch.view_as_real(g)), E._stream()))


def batch_cf_adjoint(tape: BatchTape, n2: np.ndarray, e0: np.ndarray, sign: int, zt: torch.Tensor,
                     gbar: torch.Tensor):
    """cf_adjoint of every tape of the batch: (abar[B, K], bbar[B, K+1], e0bar[B])."""
    B, dev = len(tape.m), E.device()
    abar = torch.zeros((B, tape.K), dtype=torch.float64, device=dev)
    bbar = torch.zeros((B, tape.K + 1), dtype=torch.float64, device=dev)
    scal = torch.zeros((B, 2), dtype=torch.float64, device=dev)
    mmax = max(tape.m) if tape.m else 0
    if mmax == 0:
        return abar, bbar, scal[:, 0]
    m_d = torch.tensor(tape.m, dtype=torch.int32, device=dev)
    n2_d = torch.as_tensor(np.asarray(n2, dtype=np.float64)).to(dev)
    e0_d = torch.as_tensor(np.asarray(e0, dtype=np.float64)).to(dev)
    gb = gbar.to(dtype=torch.complex128).contiguous()
    N.check(N.lib().ed_batch_cf_adjoint(B, N.ptr(tape.alpha), tape.K, N.ptr(tape.beta), tape.K + 1, N.ptr(m_d), mmax,
                                        N.ptr(n2_d), N.ptr(e0_d), int(sign), N.ptr(torch.view_as_real(zt)), zt.numel(),
                                        N.ptr(torch.view_as_real(gb)), N.ptr(abar), N.ptr(bbar), N.ptr(scal),
                                        E._stream()))
    return abar, bbar, scal[:, 0]


def _apply_fermion_rows(src: E.Plan, dst: E.Plan, pos: int, sigma: int, create: bool, X: torch.Tensor) -> torch.Tensor:
    """c^dag (create) or c applied to every row of X [B, D_src] -> [B, D_dst]."""
    B = X.shape[0]
    Y = torch.empty((B, dst.dim), dtype=torch.float64, device=E.device())
    N.check(N.lib().ed_apply_fermion(src.handle, dst.handle, int(pos), int(sigma), int(bool(create)), 0,
                                     N.ptr(X.contiguous()), N.ptr(Y), B, src.dim, dst.dim, E._stream()))
    return Y


def _gf_forward_batch(thetas: torch.Tensor, spec, zt: torch.Tensor, g: torch.Tensor):
    n_sites, bonds, width, (nu, nd), pos, sigma, m0, mgf, c, seed = spec
    B = thetas.shape[0]
    th = thetas.detach().to(dtype=torch.float64).contiguous()
    dev = E.device()
    plan = structure_plan(n_sites, bonds, width, nu, nd)
    diag = batch_diag(plan, th)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    v0 = torch.rand(plan.dim, generator=gen, dtype=torch.float64).to(dev)
    tape0 = batch_tape_forward(plan, th, diag, v0.expand(B, -1), m0, c, tol=1e-12)
    e0_d, cvec = E.tridiag_lowest_batch(tape0.alpha, tape0.beta, tape0.m)
    e0 = e0_d.cpu().numpy()
    Y, _ = batch_tape_combine(tape0, coef=cvec)
    ynorm = torch.linalg.norm(Y, dim=1)
    psi = Y / ynorm[:, None]
    parts = []
    for delta, create, sign in ((1, True, 1), (-1, False, -1)):
        tu, td = (nu + delta, nd) if sigma == 1 else (nu, nd + delta)
        if not (0 <= tu <= n_sites and 0 <= td <= n_sites):
            parts.append(None)
            continue
        tp = structure_plan(n_sites, bonds, width, tu, td)
        start = _apply_fermion_rows(plan, tp, pos, sigma, create, psi)
        tape = batch_tape_forward(tp, th, batch_diag(tp, th), start, mgf, c)
        n2 = tape.beta[:, 0].cpu().numpy() ** 2
        batch_cf(tape, n2, e0, sign, zt, g)
        parts.append((tp, tape, sign, create, n2))
    return (plan, tape0, e0_d, cvec, e0, ynorm, psi, zt, parts, spec)


def _gf_backward_batch(saved, gbar: torch.Tensor) -> torch.Tensor:
    plan, tape0, e0_d, cv, e0, ynorm, psi, zt, parts, spec = saved
    n_sites, bonds = spec[0], spec[1]
    B = psi.shape[0]
    dev = E.device()
    P = 2 * n_sites + len(bonds)
    theta_bar = torch.zeros((B, P), dtype=torch.float64, device=dev)
    e0bar = torch.zeros(B, dtype=torch.float64, device=dev)
    psibar = torch.zeros_like(psi)
    gb = gbar.to(dev).contiguous()
    pos, sigma = spec[4], spec[5]
    for part in parts:
        if part is None:
            continue
        tp, tape, sign, create, n2 = part
        Ab, Bb, eb = batch_cf_adjoint(tape, n2, e0, sign, zt, gb)
        e0bar += eb
        sbar = batch_tape_reverse(tape, Ab, Bb, theta_bar)
        psibar = psibar + _apply_fermion_rows(tp, plan, pos, sigma, not create, sbar)
    ybar = (psibar - torch.sum(psibar * psi, dim=1, keepdim=True) * psi) / ynorm[:, None]
    _, cbar = batch_tape_combine(tape0, probe=ybar)
    # v_b = -(T_b - E0_b)^+ cbar_b for every problem in one launch (device solves)
    vs = E.tridiag_pinv_solve_batch(tape0.alpha, tape0.beta, tape0.m, e0_d, cv, cbar.contiguous())
    K = tape0.K
    A0 = torch.zeros((B, K), dtype=torch.float64, device=dev)
    B0 = torch.zeros((B, K + 1), dtype=torch.float64, device=dev)
    for b in range(B):
        m = tape0.m[b]
        cvec = cv[b, :m]
        v = vs[b, :m]
        A0[b, :m] = e0bar[b] * cvec ** 2 + v * cvec
        if m > 1:
            B0[b, 1:m] = 2.0 * e0bar[b] * cvec[:-1] * cvec[1:] + v[:-1] * cvec[1:] + v[1:] * cvec[:-1]
    batch_tape_reverse(tape0, A0, B0, theta_bar, ext_coef=cv.contiguous(), ext_vec=ybar)
    return theta_bar


class GreensFunctionADBatch(torch.autograd.Function):
    """G(z) of B problems with the same structure (rows of theta), every Lanczos step of all
    problems in one launch per kernel."""

    @staticmethod
    def forward(ctx, thetas, spec, z):
        zt = E._as_dev_c128(z)
        g = torch.zeros((thetas.shape[0], zt.numel()), dtype=torch.complex128, device=E.device())
        ctx.saved = _gf_forward_batch(thetas, spec, zt, g)
        return g

    @staticmethod
    def backward(ctx, gbar):
        return _gf_backward_batch(ctx.saved, gbar).to(gbar.device), None, None


def greens_function_ad(theta: torch.Tensor, n_sites: int, bonds, sector, z, pos: int = 0, sigma: int = 1,
                       sign_width: int | None = None, gs_steps: int = 200, gf_levels: int = 200, ckpt: int = 16,
                       seed: int = 0) -> torch.Tensor:
    """Differentiable T=0 G(z) of a fermionic model sector; theta = [eps(N), U(N), t(nb)]."""
    spec = (n_sites, [tuple(b) for b in bonds], n_sites if sign_width is None else sign_width, tuple(sector), pos,
            sigma, gs_steps, gf_levels, ckpt, seed)
    return GreensFunctionAD.apply(theta, spec, z)


def greens_function_ad_batch(thetas: torch.Tensor, n_sites: int, bonds, sector, z, pos: int = 0, sigma: int = 1,
                             sign_width: int | None = None, gs_steps: int = 200, gf_levels: int = 200,
                             ckpt: int = 16, seed: int = 0) -> torch.Tensor:
    """Differentiable T=0 G(z) of B models with one structure (thetas[B, P], rows as in
    greens_function_ad) -> [B, n_z]. Each problem follows the arithmetic of greens_function_ad;
    every Lanczos step of all B problems runs as one launch per kernel (batched tape)."""
    spec = (n_sites, [tuple(b) for b in bonds], n_sites if sign_width is None else sign_width, tuple(sector), pos,
            sigma, gs_steps, gf_levels, ckpt, seed)
    if thetas.dim() != 2:
        raise ValueError("thetas must be [B, P]")
    if thetas.shape[1] != 2 * n_sites + len(spec[1]):
        raise ValueError("thetas must have 2 * n_sites + n_bonds columns")
    return GreensFunctionADBatch.apply(thetas, spec, z)


def siam_parameters(u, eps_imp, eps_bath, v, mu=None):
    """theta of a SIAM (anderson.py:147-158) as a differentiable torch function of
    (u, eps_imp, eps_bath[nb], v[nb]); returns (theta, n_sites, bonds, sign_width=0)."""
    nb = eps_bath.numel()
    mu = u / 2 if mu is None else mu
    eps = torch.cat([torch.reshape(eps_imp - mu, (1,)), eps_bath])
    uu = torch.cat([torch.reshape(u, (1,)), torch.zeros(nb, dtype=eps.dtype, device=eps.device)])
    theta = torch.cat([eps, uu, v])
    bonds = [(0, j + 1) for j in range(nb)]
    return theta, nb + 1, bonds, 0
