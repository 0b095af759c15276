"""Torch (FP64, on the device) restatement of the taped Lanczos, its reverse sweep and the
continued-fraction adjoint, step by step in plain tensor operations. Test infrastructure:
the native tape (ed_lanczos_tape / ed_tape_combine / ed_tape_reverse / ed_cf_adjoint) is
checked against it."""

from dataclasses import dataclass

import numpy as np
import torch

from cmpy_gb300.adjoint import sandwich


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


def lanczos_taped(plan, start: torch.Tensor, m: int, c: int = 16, breakdown: float = 1e-13,
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


def lanczos_reverse(plan, tape: LanczosTape, abar: torch.Tensor, bbar: torch.Tensor,
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
