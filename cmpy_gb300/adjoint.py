"""Adjoint (reverse-mode) zero-temperature Green's function behind torch.autograd.

No reference counterpart: cmpy has no derivatives. Its use is fitting Anderson bath
parameters (cmpy/models/anderson.py:24-164) for the DMFT loop (cmpy/dmft/twosite.py:103-172).

Forward, for a sector (n_up, n_dn) of a fermionic model with parameters
theta = [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}] (the plan's order):
  1. ground-state Lanczos (m0 steps) -> T0 -> lowest eigenpair (E0, c) -> psi0 = Q c/||Q c||;
  2. phi = c^dag_{pos,sigma} psi0, chi = c_{pos,sigma} psi0;
  3. Lanczos of phi in the (n+1) sector and of chi in the (n-1) sector;
  4. G(z) = CF_particle(z) + CF_hole(z)  (continued fractions, z' = +-z + E0).
Every Lanczos run stores only its scalars and the Krylov vectors q_k at k = 0 (mod c)
(with q_{k-1}); the backward pass recomputes each segment of c vectors from its checkpoint
with the stored (alpha, beta) (no reductions) and sweeps the adjoint recurrence backwards
through it. Memory: about 2m/c + c vectors per run instead of m.

Backward (exact reverse of the computed recurrences):
  * continued fraction: dG/dalpha_l, dG/dbeta_l, dG/dnorm^2, dG/dE0 by the chain through
    t_l = z' - alpha_l - beta_{l+1}^2 / t_{l+1};
  * Lanczos step k (w = H q_k, alpha = q.w, r = w - alpha q_k - beta_k q_{k-1},
    beta_{k+1} = ||r||, q_{k+1} = r / beta_{k+1}) reversed, with
    theta_bar += wbar_k^T (dH/dtheta) q_k (ed_param_sandwich) and qbar_k += H wbar_k;
  * Ritz vector and tridiagonal eigenpair: Tbar = Ebar c c^T + v c^T, v = -(T - E0)^+ cbar.
Costs: forward = m0 + m_p + m_h matvecs; backward = one matvec per step for the segment
recompute plus one for H wbar, i.e. about 2x the forward.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import engine as E

__all__ = ["LanczosTape", "lanczos_taped", "lanczos_reverse", "greens_function_ad", "GreensFunctionAD",
           "siam_parameters"]


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
# taped Lanczos (FP64): scalars + checkpoints
# ------------------------------------------------------------------------------------------


@dataclass
class LanczosTape:
    alpha: torch.Tensor   # [m]
    beta: torch.Tensor    # [m+1]; beta[0] = ||start||, beta[k] couplings, beta[m] residual
    ckpt: dict            # k -> (q_{k-1} or None, q_k) for k = 0 (mod c)
    c: int
    m: int


def _lowest_ritz_residual(alpha, beta):
    m = len(alpha)
    a = torch.stack(alpha).cpu().numpy()
    b = torch.stack(beta).cpu().numpy()
    T = np.diag(a) + np.diag(b[1:m], 1) + np.diag(b[1:m], -1)
    w, V = np.linalg.eigh(T)
    return abs(b[m] * V[m - 1, 0]), w[0]


def lanczos_taped(plan: E.Plan, start: torch.Tensor, m: int, c: int = 16, breakdown: float = 1e-13,
                  tol: float = 0.0, check_every: int = 10) -> LanczosTape:
    """Plain Lanczos from `start` keeping (alpha, beta) and checkpoints every c steps. With
    tol > 0 it stops once the lowest Ritz pair has residual <= tol * max(1, |E|) (before
    ghost copies of the converged value appear in T).

    The recurrence runs in blocks of `check_every` steps without host synchronisation; the
    breakdown test (beta_{k+1} <= breakdown * (|alpha_k| + beta_k)) and the convergence test
    read the block's scalars once. Steps computed after a breakdown inside a block are
    discarded, so the tape is the same as with a per-step test."""
    s = start.reshape(-1)
    b0 = torch.linalg.norm(s)
    q = s / b0
    qp = None
    alpha, beta = [], [b0]
    ckpt = {}
    m = int(min(m, plan.dim))
    blk = max(1, int(check_every))
    stop = None
    k = 0
    while k < m and stop is None:
        k_end = min(m, k + blk)
        for kk in range(k, k_end):
            if kk % c == 0:
                ckpt[kk] = (qp, q)
            w = plan.matvec(q)
            a = torch.dot(q, w)
            r = w - a * q
            if qp is not None:
                r = r - beta[kk] * qp
            bn = torch.linalg.norm(r)
            alpha.append(a)
            beta.append(bn)
            qp, q = q, r / bn  # inf/nan after an exact breakdown: those steps are dropped below
        a_h = torch.stack(alpha[k:k_end]).cpu().numpy()
        b_h = torch.stack(beta[k:k_end + 1]).cpu().numpy()
        for j in range(k, k_end):
            scale = abs(a_h[j - k]) + (b_h[j - k] if j > 0 else 0.0)
            if not b_h[j - k + 1] > breakdown * scale:
                stop = j + 1
                break
        if stop is None and tol > 0 and k_end % blk == 0:
            res, e = _lowest_ritz_residual(alpha, beta)
            if res <= tol * max(1.0, abs(e)):
                stop = k_end
        k = k_end
    mm = stop if stop is not None else len(alpha)
    ckpt = {kk: v for kk, v in ckpt.items() if kk < mm}
    return LanczosTape(torch.stack(alpha[:mm]), torch.stack(beta[:mm + 1]), ckpt, c, mm)


def _segment(plan, tape: LanczosTape, k0: int, k1: int):
    """q_{k0-1} .. q_{k1} recomputed from the checkpoint at k0 with the stored scalars; the
    vector after the last step (never used by the Green's function) is left at zero."""
    qp, q = tape.ckpt[k0]
    qs = {k0 - 1: qp, k0: q}
    for k in range(k0, k1):
        if k + 1 >= tape.m:
            qs[k + 1] = torch.zeros_like(q)
            continue
        w = plan.matvec(qs[k])
        r = w - tape.alpha[k] * qs[k]
        if k > 0:
            r = r - tape.beta[k] * qs[k - 1]
        qs[k + 1] = r / tape.beta[k + 1]
    return qs


def lanczos_reverse(plan: E.Plan, tape: LanczosTape, abar: torch.Tensor, bbar: torch.Tensor,
                    qbar_ext: dict | None, theta_bar: torch.Tensor) -> torch.Tensor:
    """Reverse sweep of the taped recurrence. abar[m], bbar[m+1] (bbar[0]: adjoint of the
    start norm), qbar_ext: extra adjoints of q_k (k -> vector). Accumulates the parameter
    gradient into theta_bar and returns the adjoint of the start vector."""
    m = tape.m
    abar = abar.clone()
    bbar = bbar.clone()
    qbar = {}  # adjoints of q_k, filled as the sweep descends
    if qbar_ext:
        for k, v in qbar_ext.items():
            qbar[k] = v.clone()
    seg_starts = sorted(tape.ckpt)
    for s0 in reversed(seg_starts):
        s1 = min(s0 + tape.c, m)
        qs = _segment(plan, tape, s0, s1)  # q_{s0-1} .. q_{s1}
        for k in range(s1 - 1, s0 - 1, -1):
            qk, qkp1 = qs[k], qs[k + 1]
            bk1 = tape.beta[k + 1]
            qb_next = qbar.pop(k + 1, None)
            # q_{k+1} = r_k / beta_{k+1} ; beta_{k+1} = ||r_k||
            if qb_next is not None:
                rbar = qb_next / bk1
                bbar[k + 1] = bbar[k + 1] - torch.dot(qb_next, qkp1) / bk1
            else:
                rbar = torch.zeros_like(qk)
            rbar = rbar + bbar[k + 1] * qkp1
            # r_k = w_k - alpha_k q_k - beta_k q_{k-1}
            w = plan.matvec(qk)
            abar[k] = abar[k] - torch.dot(rbar, qk)
            qb = qbar.get(k, torch.zeros_like(qk)) - tape.alpha[k] * rbar
            if k > 0:
                bbar[k] = bbar[k] - torch.dot(rbar, qs[k - 1])
                qbar[k - 1] = qbar.get(k - 1, torch.zeros_like(qk)) - tape.beta[k] * rbar
            # alpha_k = q_k . w_k
            wbar = rbar + abar[k] * qk
            qb = qb + abar[k] * w
            # w_k = H q_k
            sandwich(plan, wbar, qk, theta_bar)
            qb = qb + plan.matvec(wbar)
            qbar[k] = qb
    q0 = tape.ckpt[0][1]
    qb0 = qbar.get(0, torch.zeros_like(q0))
    b0 = tape.beta[0]
    # q_0 = s / ||s||, beta_0 = ||s||
    return (qb0 - torch.dot(qb0, q0) * q0) / b0 + bbar[0] * q0


# ------------------------------------------------------------------------------------------
# continued fraction with its derivatives
# ------------------------------------------------------------------------------------------


def cf_eval(alpha, beta, n2, z, e0, sign):
    """G(z) and the per-level quantities needed for its derivatives (torch, complex128)."""
    m = alpha.numel()
    zp = sign * z + e0
    ts = [None] * m
    t = zp - alpha[m - 1]
    ts[m - 1] = t
    for l in range(m - 2, -1, -1):
        t = zp - alpha[l] - beta[l + 1] ** 2 / t
        ts[l] = t
    g = sign * n2 / ts[0]
    return g, ts


def cf_adjoint(alpha, beta, n2, z, e0, sign, gbar):
    """Adjoints (abar[m], bbar[m+1] with bbar[0] for sqrt(n2), e0bar) of
    L = Re sum conj(gbar) G."""
    m = alpha.numel()
    g, ts = cf_eval(alpha, beta, n2, z, e0, sign)
    u = -sign * n2 / ts[0] ** 2  # dG/dt_0
    abar = torch.zeros(m, dtype=torch.float64, device=alpha.device)
    bbar = torch.zeros(m + 1, dtype=torch.float64, device=alpha.device)
    dz = torch.zeros_like(u)
    cg = torch.conj(gbar)
    for l in range(m):
        dz = dz + u  # dt_l/dz' = 1
        abar[l] = torch.real(torch.sum(cg * (-u)))
        if l + 1 < m:
            bb = beta[l + 1]
            bbar[l + 1] = torch.real(torch.sum(cg * (u * (-2.0 * bb / ts[l + 1]))))
            u = u * (bb * bb) / ts[l + 1] ** 2
    e0bar = torch.real(torch.sum(cg * dz))
    n2bar = torch.real(torch.sum(cg * (sign / ts[0])))
    bbar[0] = n2bar * 2.0 * torch.sqrt(n2)  # norm adjoint
    return g, abar, bbar, e0bar


# ------------------------------------------------------------------------------------------
# the autograd function
# ------------------------------------------------------------------------------------------


class GreensFunctionAD(torch.autograd.Function):
    """G(z) of a fermionic model sector as a differentiable function of theta."""

    @staticmethod
    def forward(ctx, theta, spec, z):
        n_sites, bonds, width, (nu, nd), pos, sigma, m0, mgf, c, seed = spec
        plan = plan_from_params(theta, n_sites, bonds, width, nu, nd)
        gen = torch.Generator(device="cpu").manual_seed(seed)
        v0 = torch.rand(plan.dim, generator=gen, dtype=torch.float64).to(E.device())
        tape0 = lanczos_taped(plan, v0, m0, c, tol=1e-12)
        m = tape0.m
        T = torch.diag(tape0.alpha) + torch.diag(tape0.beta[1:m], 1) + torch.diag(tape0.beta[1:m], -1)
        w, V = torch.linalg.eigh(T)
        e0 = w[0]
        cvec = V[:, 0]
        # Ritz vector (segments recomputed from checkpoints)
        y = torch.zeros(plan.dim, dtype=torch.float64, device=E.device())
        for s0 in sorted(tape0.ckpt):
            s1 = min(s0 + tape0.c, m)
            qs = _segment(plan, tape0, s0, s1)
            for k in range(s0, s1):
                y = y + cvec[k] * qs[k]
        ynorm = torch.linalg.norm(y)
        psi = y / ynorm
        zt = E._as_dev_c128(z)
        g = torch.zeros_like(zt)
        parts = []
        for delta, create, sign in ((1, True, 1), (-1, False, -1)):
            tu, td = (nu + delta, nd) if sigma == 1 else (nu, nd + delta)
            if not (0 <= tu <= n_sites and 0 <= td <= n_sites):
                parts.append(None)
                continue
            tp = plan_from_params(theta, n_sites, bonds, width, tu, td)
            start = plan.apply_fermion(tp, pos, sigma, create, psi)
            if torch.linalg.norm(start).item() == 0.0:
                parts.append(None)
                continue
            tape = lanczos_taped(tp, start, mgf, c)
            n2 = tape.beta[0] ** 2
            gp, _ = cf_eval(tape.alpha, tape.beta, n2, zt, e0, sign)
            g = g + gp
            parts.append((tp, tape, sign, create))
        ctx.saved = (plan, tape0, cvec, w, ynorm, psi, e0, zt, parts, spec)
        return g

    @staticmethod
    def backward(ctx, gbar):
        plan, tape0, cvec, w, ynorm, psi, e0, zt, parts, spec = ctx.saved
        n_sites, bonds, width, (nu, nd), pos, sigma, m0, mgf, c, seed = spec
        P = 2 * n_sites + len(bonds)
        theta_bar = torch.zeros(P, dtype=torch.float64, device=E.device())
        e0bar = torch.zeros((), dtype=torch.float64, device=E.device())
        psibar = torch.zeros_like(psi)
        for part in parts:
            if part is None:
                continue
            tp, tape, sign, create = part
            n2 = tape.beta[0] ** 2
            _, abar, bbar, eb = cf_adjoint(tape.alpha, tape.beta, n2, zt, e0, sign, gbar)
            e0bar = e0bar + eb
            sbar = lanczos_reverse(tp, tape, abar, bbar, None, theta_bar)
            # start = c^dag psi (or c psi): its adjoint maps back with the opposite operator
            psibar = psibar + tp.apply_fermion(plan, pos, sigma, not create, sbar)
        # psi = y / ||y||, y = sum_k c_k q_k
        ybar = (psibar - torch.dot(psibar, psi) * psi) / ynorm
        m = tape0.m
        # c_bar_k = q_k . ybar and the external q_bar_k = c_k ybar, segment by segment
        cbar = torch.zeros(m, dtype=torch.float64, device=E.device())
        for s0 in sorted(tape0.ckpt):
            s1 = min(s0 + tape0.c, m)
            qs = _segment(plan, tape0, s0, s1)
            for k in range(s0, s1):
                cbar[k] = torch.dot(qs[k], ybar)
        # eigenpair of T: E0 = c^T T c, c = ground state of T
        T = torch.diag(tape0.alpha) + torch.diag(tape0.beta[1:m], 1) + torch.diag(tape0.beta[1:m], -1)
        cb = cbar - torch.dot(cbar, cvec) * cvec
        A = T - w[0] * torch.eye(m, dtype=torch.float64, device=E.device())
        # v = -(T - E0)^+ cb on the complement of c (add c c^T to make the system regular)
        v = -torch.linalg.solve(A + torch.outer(cvec, cvec), cb)
        v = v - torch.dot(v, cvec) * cvec
        abar0 = e0bar * cvec ** 2 + v * cvec
        bbar0 = torch.zeros(m + 1, dtype=torch.float64, device=E.device())
        if m > 1:
            bbar0[1:m] = 2.0 * e0bar * cvec[:-1] * cvec[1:] + v[:-1] * cvec[1:] + v[1:] * cvec[:-1]
        qext = {k: cvec[k] * ybar for k in range(m)}
        lanczos_reverse(plan, tape0, abar0, bbar0, qext, theta_bar)
        return theta_bar.to(gbar.device), None, None


def greens_function_ad(theta: torch.Tensor, n_sites: int, bonds, sector, z, pos: int = 0, sigma: int = 1,
                       sign_width: int | None = None, gs_steps: int = 200, gf_levels: int = 200, ckpt: int = 16,
                       seed: int = 0) -> torch.Tensor:
    """Differentiable T=0 G(z) of a fermionic model sector; theta = [eps(N), U(N), t(nb)]."""
    spec = (n_sites, [tuple(b) for b in bonds], n_sites if sign_width is None else sign_width, tuple(sector), pos,
            sigma, gs_steps, gf_levels, ckpt, seed)
    return GreensFunctionAD.apply(theta, spec, z)


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
