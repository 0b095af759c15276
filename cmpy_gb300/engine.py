"""Device-side objects of the engine: plans (one Hamiltonian sector on one GPU) and thin
wrappers of the C ABI. Everything here runs on the current CUDA device through
libcmpy_ed.so; tensors are torch CUDA tensors.
"""

from __future__ import annotations

import ctypes as C
import math
import threading
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np
import torch

from . import _native as N

__all__ = [
    "device",
    "Plan",
    "basis_plan",
    "enumerate_states",
    "rank_states",
    "LanczosResult",
    "lanczos",
    "lanczos_coeffs",
    "tridiag_lowest",
    "tridiag_lowest_batch",
    "tridiag_pinv_solve_batch",
    "continued_fraction",
    "lehmann_accumulate",
    "csr_matvec",
    "coo_onsite",
    "coo_inter",
    "coo_hopping",
]


def launch_count() -> int:
    """Kernels launched by libcmpy_ed.so so far in this process."""
    return int(N.lib().ed_launch_count())


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("cmpy_gb300 needs a CUDA GPU (GB300, sm_103a); there is no CPU fallback")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return N.stream_handle()


def _as_dev_f64(x) -> torch.Tensor:
    dev = device()
    if isinstance(x, torch.Tensor):
        t = x.to(device=dev, dtype=torch.float64)
    else:
        t = torch.as_tensor(np.asarray(x, dtype=np.float64)).to(dev)
    return t.contiguous()


def _as_dev_states(states) -> torch.Tensor:
    dev = device()
    if isinstance(states, torch.Tensor):
        return states.to(device=dev, dtype=torch.int64).contiguous()
    return torch.as_tensor(np.asarray(states, dtype=np.int64).reshape(-1)).to(dev).contiguous()


# ------------------------------------------------------------------------------------------
# basis
# ------------------------------------------------------------------------------------------


def sector_size(n_sites: int, n: int | None) -> int:
    return int(N.lib().ed_sector_size(int(n_sites), -1 if n is None else int(n)))


def enumerate_states(n_sites: int, n: int | None) -> torch.Tensor:
    """Ascending states with popcount n (all 2^n_sites for n=None) as an int64 CUDA tensor."""
    L = N.lib()
    nn = -1 if n is None else int(n)
    count = int(L.ed_sector_size(int(n_sites), nn))
    if count < 0:
        raise ValueError("sector too large")
    out = torch.empty(max(count, 0), dtype=torch.int64, device=device())
    if count > 0:
        N.check(L.ed_enumerate(int(n_sites), nn, N.ptr(out), count, _stream()))
    return out


def rank_states(states) -> torch.Tensor:
    st = _as_dev_states(states)
    out = torch.empty_like(st)
    if st.numel():
        N.check(N.lib().ed_rank(N.ptr(st), st.numel(), N.ptr(out), _stream()))
    return out


# ------------------------------------------------------------------------------------------
# plans
# ------------------------------------------------------------------------------------------


class Plan:
    """One Hamiltonian sector resident on the current device (an ed_plan handle).

    ``kind`` is "fermion" (Hubbard / Anderson, up-major many-body index) or "spin".
    """

    def __init__(self, handle: int, kind: str, key=None):
        self._h = C.c_void_p(handle)
        self.kind = kind
        self.key = key
        self.device_index = torch.cuda.current_device()
        info = N.PlanInfo()
        N.check(N.lib().ed_plan_get_info(self._h, C.byref(info)))
        self.info = info
        self.dim = int(info.dim)
        self.num_up = int(info.num_up)
        self.num_dn = int(info.num_dn)
        self.n_sites = int(info.n_sites)
        self.n_up = int(info.n_up)
        self.n_dn = int(info.n_dn)
        self.hnorm_bound = float(info.hnorm_bound)

    # -- construction ------------------------------------------------------------------------
    @classmethod
    def fermion(
        cls,
        n_sites: int,
        eps: Sequence[float],
        u: Sequence[float],
        bonds: Iterable[tuple[int, int, float]],
        n_up: int,
        n_dn: int,
        sign_width: int | None = None,
    ) -> "Plan":
        bonds = list(bonds)
        eps_a, eps_p = N.f64_array(eps)
        u_a, u_p = N.f64_array(u)
        if len(eps_a) != n_sites or len(u_a) != n_sites:
            raise ValueError("eps and u need one value per site")
        s1_a, s1_p = N.i32_array([b[0] for b in bonds])
        s2_a, s2_p = N.i32_array([b[1] for b in bonds])
        t_a, t_p = N.f64_array([b[2] for b in bonds])
        m = N.FermionModel()
        m.n_sites = n_sites
        m.n_bonds = len(bonds)
        m.sign_width = n_sites if sign_width is None else int(sign_width)
        m.h_eps, m.h_u = eps_p, u_p
        m.h_bond_site1, m.h_bond_site2, m.h_bond_hop = s1_p, s2_p, t_p
        h = C.c_void_p()
        device()
        N.check(N.lib().ed_plan_create_fermion(C.byref(m), int(n_up), int(n_dn), C.byref(h), _stream()))
        key = ("fermion", n_sites, tuple(eps_a.tolist()), tuple(u_a.tolist()), tuple(map(tuple, bonds)),
               m.sign_width, n_up, n_dn)
        return cls(h.value, "fermion", key)

    @classmethod
    def spin(cls, n_sites: int, pairs: Iterable[tuple[int, int, float, float]], n_up: int) -> "Plan":
        pairs = list(pairs)
        p1_a, p1_p = N.i32_array([p[0] for p in pairs])
        p2_a, p2_p = N.i32_array([p[1] for p in pairs])
        j_a, j_p = N.f64_array([p[2] for p in pairs])
        jz_a, jz_p = N.f64_array([p[3] for p in pairs])
        m = N.SpinModel()
        m.n_sites = n_sites
        m.n_pairs = len(pairs)
        m.h_pos1, m.h_pos2, m.h_j, m.h_jz = p1_p, p2_p, j_p, jz_p
        h = C.c_void_p()
        device()
        N.check(N.lib().ed_plan_create_spin(C.byref(m), int(n_up), C.byref(h), _stream()))
        return cls(h.value, "spin", ("spin", n_sites, tuple(map(tuple, pairs)), n_up))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                with torch.cuda.device(self.device_index):
                    N.lib().ed_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def _dev(self):
        return torch.cuda.device(self.device_index)

    # -- basis views -------------------------------------------------------------------------
    def up_states(self) -> torch.Tensor:
        return enumerate_states(self.n_sites, self.n_up)

    def dn_states(self) -> torch.Tensor:
        if self.kind != "fermion":
            raise ValueError("spin plans have one state list")
        return enumerate_states(self.n_sites, self.n_dn)

    # -- Hamiltonian application ----------------------------------------------------------------
    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        with self._dev():
            x = _as_dev_f64(x).reshape(-1)
            if x.numel() != self.dim:
                raise ValueError(f"vector of length {x.numel()} for a sector of dimension {self.dim}")
            y = torch.empty_like(x) if out is None else out
            N.check(N.lib().ed_matvec(self._h, N.ptr(x), N.ptr(y), _stream()))
            return y

    def matmat(self, X: torch.Tensor) -> torch.Tensor:
        """H X for X of shape (D, k) (columns are vectors)."""
        with self._dev():
            X = _as_dev_f64(X)
            if X.ndim != 2 or X.shape[0] != self.dim:
                raise ValueError("expected a (D, k) matrix")
            Xc = X.t().contiguous()  # k vectors contiguous
            Y = torch.empty_like(Xc)
            N.check(N.lib().ed_matmat(self._h, N.ptr(Xc), N.ptr(Y), Xc.shape[0], self.dim, _stream()))
            return Y.t()

    @property
    def fixed_point(self) -> int:
        """Input mantissa bits of the sector's integer matvec, 0 if it has none."""
        return int(N.lib().ed_plan_fixed_point(self._h))

    @property
    def matvec_variant(self) -> int:
        """Fixed-point matvec the plan uses: 7 = single-pass kernel with the dn states renumbered
        by hop count (default where it fits), 3/2/1 = single-pass kernels in the sector's order,
        5 = banded two-pass sweep, 6 = two-pass stripes (5 and 6 on request; 5, 6 and 7 keep the
        Lanczos vectors in a renumbered basis), 0 = none (FP64 matvec)."""
        return int(N.lib().ed_plan_matvec_variant(self._h))

    def set_matvec_variant(self, variant: int) -> None:
        """Choose the fixed-point matvec variant (0 = automatic) for comparisons and timing."""
        N.check(N.lib().ed_plan_set_matvec_variant(self._h, int(variant)))

    def set_wait_limit(self, polls: int) -> None:
        """Polls of a first bulk-copy wait in the fixed-point matvec before it gives up and the
        solve reports ED_ERR_TIMEOUT (0 = default, -1 = give up without polling)."""
        N.check(N.lib().ed_plan_set_wait_limit(self._h, int(polls)))

    def matvec_fixed(self, xm: torch.Tensor, ex: int) -> tuple[torch.Tensor, int]:
        """Exact integer H*x for x = xm * 2^ex (int64 mantissas); returns (wm, ew)."""
        with self._dev():
            xm = xm.to(device=device(), dtype=torch.int64).contiguous().reshape(-1)
            wm = torch.empty_like(xm)
            ew = C.c_int32()
            N.check(N.lib().ed_matvec_fixed(self._h, N.ptr(xm), int(ex), N.ptr(wm), C.byref(ew), None, _stream()))
            return wm, int(ew.value)

    def dense(self) -> torch.Tensor:
        with self._dev():
            out = torch.empty((self.dim, self.dim), dtype=torch.float64, device=device())
            N.check(N.lib().ed_dense(self._h, N.ptr(out), _stream()))
            return out

    def diagonal(self) -> torch.Tensor:
        with self._dev():
            out = torch.empty(self.dim, dtype=torch.float64, device=device())
            N.check(N.lib().ed_diagonal(self._h, N.ptr(out), _stream()))
            return out

    def coo(self) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """Reference-ordered triplets (rows, cols, vals) of the whole model."""
        with self._dev():
            L = N.lib()
            nnz = C.c_int64()
            N.check(L.ed_coo_plan(self._h, None, None, None, 0, C.byref(nnz), _stream()))
            n = int(nnz.value)
            rows = torch.empty(n, dtype=torch.int64, device=device())
            cols = torch.empty(n, dtype=torch.int64, device=device())
            vals = torch.empty(n, dtype=torch.float64, device=device())
            if n:
                N.check(L.ed_coo_plan(self._h, N.ptr(rows), N.ptr(cols), N.ptr(vals), n, C.byref(nnz), _stream()))
            return rows, cols, vals

    def apply_fermion(self, target: "Plan", pos: int, sigma: int, create: bool, x: torch.Tensor,
                      jw_sign: bool = False) -> torch.Tensor:
        """c^dag (create) or c on site pos, spin sigma (1 up, 2 dn), into the target sector.
        x: (D,) or (D, k)."""
        with self._dev():
            x = _as_dev_f64(x)
            vec = x.ndim == 1
            X = x.reshape(self.dim, -1).t().contiguous()
            k = X.shape[0]
            Y = torch.empty((k, target.dim), dtype=torch.float64, device=device())
            N.check(N.lib().ed_apply_fermion(self._h, target.handle, int(pos), int(sigma), int(bool(create)),
                                             int(bool(jw_sign)), N.ptr(X), N.ptr(Y), k, self.dim, target.dim,
                                             _stream()))
            return Y.reshape(-1) if vec else Y.t()


def apply_fermion_batch(plans, targets, pos: int, sigma: int, create: bool, x: torch.Tensor, x_offsets,
                        jw_sign: bool = False):
    """c^dag (create) or c on site pos, spin sigma, for many problems in one native call:
    problem i maps x[x_offsets[i] : x_offsets[i] + plans[i].dim] into its target sector.
    Returns (y, y_offsets): one buffer holding every target vector, problem i at
    y[y_offsets[i] : y_offsets[i] + targets[i].dim]."""
    n = len(plans)
    if len(targets) != n or len(x_offsets) != n:
        raise ValueError("plans, targets and x_offsets must have the same length")
    dims = np.array([t.dim for t in targets], dtype=np.int64)
    y_off = np.zeros(n, dtype=np.int64)
    if n > 1:
        y_off[1:] = np.cumsum(dims)[:-1]
    y = torch.empty(int(dims.sum()), dtype=torch.float64, device=device())
    if n == 0:
        return y, y_off
    xo = np.ascontiguousarray(x_offsets, dtype=np.int64)
    x = _as_dev_f64(x).reshape(-1)
    if np.any(xo + np.array([p.dim for p in plans], dtype=np.int64) > x.numel()):
        raise ValueError("a source vector runs past the end of x")
    arr_p = (C.c_void_p * n)(*[p.handle.value for p in plans])
    arr_t = (C.c_void_p * n)(*[t.handle.value for t in targets])
    N.check(N.lib().ed_apply_fermion_batch(arr_p, arr_t, n, int(pos), int(sigma), int(bool(create)),
                                           int(bool(jw_sign)), N.ptr(x), xo.ctypes.data, N.ptr(y),
                                           y_off.ctypes.data, _stream()))
    return y, y_off


_basis_plans: dict = {}
_basis_lock = threading.Lock()


def basis_plan(n_sites: int, n_up: int, n_dn: int) -> Plan:
    """Plan with the sector basis only (no Hamiltonian terms), used by c^dag / c."""
    key = (torch.cuda.current_device(), n_sites, n_up, n_dn)
    with _basis_lock:
        p = _basis_plans.get(key)
        if p is None:
            p = Plan.fermion(n_sites, [0.0] * n_sites, [0.0] * n_sites, [], n_up, n_dn)
            _basis_plans[key] = p
    return p


# ------------------------------------------------------------------------------------------
# COO segments (project_* generators of cmpy/operators.py)
# ------------------------------------------------------------------------------------------


def _coo_call(fn, *args) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    nnz = C.c_int64()
    N.check(fn(*args, None, None, None, 0, C.byref(nnz), _stream()))
    n = int(nnz.value)
    rows = torch.empty(n, dtype=torch.int64, device=device())
    cols = torch.empty(n, dtype=torch.int64, device=device())
    vals = torch.empty(n, dtype=torch.float64, device=device())
    if n:
        N.check(fn(*args, N.ptr(rows), N.ptr(cols), N.ptr(vals), n, C.byref(nnz), _stream()))
    return rows, cols, vals


def coo_onsite(up_states, dn_states, eps):
    up, dn = _as_dev_states(up_states), _as_dev_states(dn_states)
    e, ep = N.f64_array(np.atleast_1d(eps))
    return _coo_call(N.lib().ed_coo_onsite, N.ptr(up), up.numel(), N.ptr(dn), dn.numel(), ep, len(e))


def coo_inter(up_states, dn_states, u):
    up, dn = _as_dev_states(up_states), _as_dev_states(dn_states)
    e, ep = N.f64_array(np.atleast_1d(u))
    return _coo_call(N.lib().ed_coo_inter, N.ptr(up), up.numel(), N.ptr(dn), dn.numel(), ep, len(e))


def coo_hopping(up_states, dn_states, width, site1, site2, hop):
    up, dn = _as_dev_states(up_states), _as_dev_states(dn_states)
    return _coo_call(N.lib().ed_coo_hopping, N.ptr(up), up.numel(), N.ptr(dn), dn.numel(), int(width),
                     int(site1), int(site2), float(hop))


def fixed_from_f64(x, m_bits: int = 56) -> tuple[torch.Tensor, int]:
    """Block-fixed-point encoding of an FP64 vector: (int64 mantissas, exponent)."""
    xt = _as_dev_f64(x).reshape(-1)
    xm = torch.empty(xt.numel(), dtype=torch.int64, device=xt.device)
    e = C.c_int32()
    N.check(N.lib().ed_fixed_from_f64(N.ptr(xt), xt.numel(), int(m_bits), N.ptr(xm), C.byref(e), _stream()))
    return xm, int(e.value)


def fixed_to_f64(xm: torch.Tensor, exp: int) -> torch.Tensor:
    xm = xm.to(device=device(), dtype=torch.int64).contiguous()
    out = torch.empty(xm.numel(), dtype=torch.float64, device=xm.device)
    N.check(N.lib().ed_fixed_to_f64(N.ptr(xm), xm.numel(), int(exp), N.ptr(out), _stream()))
    return out


def csr_matvec(rowptr: torch.Tensor, cols: torch.Tensor, vals: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    n = rowptr.numel() - 1
    y = torch.empty(n, dtype=torch.float64, device=x.device)
    N.check(N.lib().ed_csr_matvec(n, N.ptr(rowptr), N.ptr(cols), N.ptr(vals), N.ptr(x), N.ptr(y), _stream()))
    return y


# ------------------------------------------------------------------------------------------
# Lanczos / Green's functions
# ------------------------------------------------------------------------------------------


@dataclass
class LanczosResult:
    energy: float
    residual: float
    steps: int
    converged: int
    alpha: torch.Tensor
    beta: torch.Tensor
    vector: torch.Tensor | None
    matvec_ms: float = 0.0
    matvecs: int = 0


def lanczos(plan: Plan, max_steps: int = 250, reorth: bool = False, want_vector: bool = True,
            tol: float = 0.0, check_every: int = 0, v0: torch.Tensor | None = None, seed: int = 0,
            workspace: torch.Tensor | None = None, profile: bool = False,
            arithmetic: str = "auto") -> LanczosResult:
    """Lanczos ground state of a plan, entirely on the device.

    arithmetic: "auto" (block-fixed-point vectors when the sector allows it), "f64" or
    "fixed" (error if the sector has no integer matvec)."""
    L = N.lib()
    prm = N.LanczosParams()
    prm.max_steps = int(max_steps)
    prm.reorth = int(bool(reorth))
    prm.check_every = int(check_every)
    prm.want_vector = int(bool(want_vector))
    prm.tol = float(tol)
    prm.seed = int(seed)
    prm.profile = int(bool(profile))
    prm.arithmetic = {"auto": 0, "f64": 1, "fixed": 2}[arithmetic]
    with plan._dev():
        nb = C.c_size_t()
        N.check(L.ed_lanczos_workspace(plan.handle, C.byref(prm), C.byref(nb)))
        if workspace is None or workspace.numel() < nb.value:
            workspace = torch.empty(int(nb.value), dtype=torch.uint8, device=device())
        alpha = torch.empty(prm.max_steps, dtype=torch.float64, device=device())
        beta = torch.empty(prm.max_steps + 1, dtype=torch.float64, device=device())
        vec = torch.empty(plan.dim, dtype=torch.float64, device=device()) if want_vector else None
        v0t = _as_dev_f64(v0).reshape(-1) if v0 is not None else None
        res = N.LanczosResult()
        N.check(L.ed_lanczos(plan.handle, C.byref(prm), N.ptr(v0t), N.ptr(workspace), nb.value, N.ptr(alpha),
                             N.ptr(beta), N.ptr(vec), C.byref(res), _stream()))
        m = int(res.steps)
        return LanczosResult(float(res.energy), float(res.residual), m, int(res.converged), alpha[:m],
                             beta[: m + 1], vec, float(res.matvec_ms), int(res.matvecs))


def lanczos_coeffs(plan: Plan, start: torch.Tensor, max_steps: int = 200,
                   workspace: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor, float]:
    """(alpha[m], beta[m+1], ||start||) of the Krylov space of `start` (no basis stored)."""
    L = N.lib()
    prm = N.LanczosParams()
    prm.max_steps = int(max_steps)
    with plan._dev():
        nb = C.c_size_t()
        N.check(L.ed_lanczos_workspace(plan.handle, C.byref(prm), C.byref(nb)))
        if workspace is None or workspace.numel() < nb.value:
            workspace = torch.empty(int(nb.value), dtype=torch.uint8, device=device())
        s = _as_dev_f64(start).reshape(-1)
        alpha = torch.empty(prm.max_steps, dtype=torch.float64, device=device())
        beta = torch.empty(prm.max_steps + 1, dtype=torch.float64, device=device())
        steps = C.c_int()
        nrm = C.c_double()
        N.check(L.ed_lanczos_coeffs(plan.handle, prm.max_steps, N.ptr(s), N.ptr(workspace), nb.value, N.ptr(alpha),
                                    N.ptr(beta), C.byref(steps), C.byref(nrm), _stream()))
        m = int(steps.value)
        return alpha[:m], beta[: m + 1], float(nrm.value)


def lanczos_coeffs_multi(runs, max_steps: int = 200) -> list[tuple[torch.Tensor, torch.Tensor, float]]:
    """lanczos_coeffs for several independent (plan, start) pairs in one call: with fixed-point
    plans their steps interleave on separate streams (one run's kernels fill the SMs the other
    leaves idle); the results equal separate lanczos_coeffs calls."""
    runs = list(runs)
    if not runs:
        return []
    L = N.lib()
    prm = N.LanczosParams()
    prm.max_steps = int(max_steps)
    n = len(runs)
    with runs[0][0]._dev():
        keep, starts, works, sizes, alphas, betas = [], [], [], [], [], []
        for plan, start in runs:
            nb = C.c_size_t()
            N.check(L.ed_lanczos_workspace(plan.handle, C.byref(prm), C.byref(nb)))
            w = torch.empty(max(int(nb.value), 1), dtype=torch.uint8, device=device())
            s = _as_dev_f64(start).reshape(-1).contiguous()
            a = torch.empty(prm.max_steps, dtype=torch.float64, device=device())
            b = torch.empty(prm.max_steps + 1, dtype=torch.float64, device=device())
            keep += [w, s, a, b]
            starts.append(N.ptr(s))
            works.append(N.ptr(w))
            sizes.append(int(nb.value))
            alphas.append(N.ptr(a))
            betas.append(N.ptr(b))
        P = C.c_void_p
        h_plans = (P * n)(*[p.handle for p, _ in runs])
        h_steps = (C.c_int * n)()
        h_norm = (C.c_double * n)()
        N.check(L.ed_lanczos_coeffs_multi(n, h_plans, prm.max_steps, (P * n)(*starts), (P * n)(*works),
                                          (C.c_size_t * n)(*sizes), (P * n)(*alphas), (P * n)(*betas), h_steps,
                                          h_norm, _stream()))
        out = []
        for i in range(n):
            m = int(h_steps[i])
            out.append((keep[4 * i + 2][:m], keep[4 * i + 3][: m + 1], float(h_norm[i])))
        return out


def tridiag_lowest(alpha, beta, want_vector: bool = True):
    """Lowest eigenpair of the tridiagonal (alpha[0..m), beta[1..m)) on the device."""
    a = _as_dev_f64(alpha).reshape(-1)
    b = _as_dev_f64(beta).reshape(-1)
    m = a.numel()
    if b.numel() < m:
        raise ValueError("beta needs at least len(alpha) entries (beta[0] unused)")
    val = torch.empty(1, dtype=torch.float64, device=device())
    vec = torch.empty(m, dtype=torch.float64, device=device()) if want_vector else None
    N.check(N.lib().ed_tridiag_lowest(N.ptr(a), N.ptr(b), m, N.ptr(val), N.ptr(vec), _stream()))
    return float(val.item()), vec


def tridiag_lowest_batch(alpha: torch.Tensor, beta: torch.Tensor, m) -> tuple[torch.Tensor, torch.Tensor]:
    """Lowest eigenpairs of B tridiagonals in one launch: alpha [B, lda], beta [B, ldb] (row b
    uses alpha[b, :m[b]], beta[b, 1:m[b]]). Returns (values [B], vectors [B, lda]) on the device."""
    a = _as_dev_f64(alpha).contiguous()
    b = _as_dev_f64(beta).contiguous()
    B, lda = a.shape
    mm = torch.as_tensor(np.asarray(m, dtype=np.int32)).to(device())
    max_m = int(np.max(np.asarray(m))) if B else 1
    vals = torch.empty(B, dtype=torch.float64, device=device())
    vecs = torch.zeros((B, lda), dtype=torch.float64, device=device())
    N.check(N.lib().ed_tridiag_lowest_batch(N.ptr(a), lda, N.ptr(b), b.shape[1], N.ptr(mm), B, max_m, N.ptr(vals),
                                            N.ptr(vecs), lda, _stream()))
    return vals, vecs


def dense_eigh_batch(mats) -> list[tuple[torch.Tensor, torch.Tensor]]:
    """Every eigenpair of each real symmetric matrix in `mats` (square tensors), one call for
    the batch: [(eigenvalues ascending [n], eigenvectors as columns [n, n])] on the device.
    The hand-written FP64 solver (Householder, Sturm multisection, inverse iteration)."""
    ms = [_as_dev_f64(a) for a in mats]
    if not ms:
        return []
    sizes = [int(a.shape[0]) for a in ms]
    if any(a.dim() != 2 or a.shape[0] != a.shape[1] or a.shape[0] < 1 for a in ms):
        raise ValueError("dense_eigh_batch takes non-empty square matrices")
    B, nmax = len(ms), max(sizes)
    A = torch.zeros((B, nmax, nmax), dtype=torch.float64, device=device())
    for b, a in enumerate(ms):
        A[b, : sizes[b], : sizes[b]] = a
    W = torch.empty((B, nmax), dtype=torch.float64, device=device())
    Z = torch.zeros((B, nmax, nmax), dtype=torch.float64, device=device())
    hn = (C.c_int * B)(*sizes)
    N.check(N.lib().ed_dense_eigh_batch(N.ptr(A), nmax, nmax * nmax, hn, B, nmax, N.ptr(W), N.ptr(Z), nmax,
                                        nmax * nmax, _stream()))
    return [(W[b, : sizes[b]], Z[b, : sizes[b], : sizes[b]].t()) for b in range(B)]


def dense_eigh(a: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """(eigenvalues ascending, eigenvectors as columns) of one real symmetric matrix."""
    return dense_eigh_batch([a])[0]


def tridiag_eigh(alpha: torch.Tensor, beta: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Every eigenpair of the tridiagonal (alpha[0..m), beta[1..m)): (eigenvalues ascending,
    eigenvectors as columns [m, m]) on the device."""
    a = _as_dev_f64(alpha).contiguous().reshape(-1)
    b = _as_dev_f64(beta).contiguous().reshape(-1)
    m = a.numel()
    if b.numel() < m:
        raise ValueError("beta needs m entries (beta[0] unused)")
    w = torch.empty(m, dtype=torch.float64, device=device())
    z = torch.zeros((m, m), dtype=torch.float64, device=device())
    N.check(N.lib().ed_tridiag_eigh(N.ptr(a), N.ptr(b), m, N.ptr(w), N.ptr(z), m, _stream()))
    return w, z.t()


def tridiag_pinv_solve_batch(alpha: torch.Tensor, beta: torch.Tensor, m, e0: torch.Tensor, c: torch.Tensor,
                             rhs: torch.Tensor) -> torch.Tensor:
    """v_b = -(T_b - e0_b)^+ rhs_b on the complement of c_b for B tridiagonals (c_b the unit
    lowest eigenvector of T_b, e0_b its eigenvalue); rows as in tridiag_lowest_batch."""
    a = _as_dev_f64(alpha).contiguous()
    b = _as_dev_f64(beta).contiguous()
    cc = _as_dev_f64(c).contiguous()
    r = _as_dev_f64(rhs).contiguous()
    e = _as_dev_f64(e0).contiguous()
    B = a.shape[0]
    mm = torch.as_tensor(np.asarray(m, dtype=np.int32)).to(device())
    max_m = int(np.max(np.asarray(m))) if B else 1
    out = torch.zeros_like(r)
    N.check(N.lib().ed_tridiag_pinv_solve_batch(N.ptr(a), a.shape[1], N.ptr(b), b.shape[1], N.ptr(mm), B, max_m,
                                                N.ptr(e), N.ptr(cc), cc.shape[1], N.ptr(r), N.ptr(out), r.shape[1],
                                                _stream()))
    return out


def _as_dev_c128(z) -> torch.Tensor:
    dev = device()
    if isinstance(z, torch.Tensor):
        t = z.to(device=dev, dtype=torch.complex128)
    else:
        t = torch.as_tensor(np.asarray(z, dtype=np.complex128)).to(dev)
    return t.contiguous().reshape(-1)


def continued_fraction(alpha, beta, norm2: float, z, e0: float = 0.0, sign: int = 1,
                       out: torch.Tensor | None = None) -> torch.Tensor:
    """sign * norm2 / (z' - a0 - b1^2/(z' - a1 - ...)), z' = sign*z + e0 (complex128 on device)."""
    a = _as_dev_f64(alpha)
    b = _as_dev_f64(beta)
    zt = _as_dev_c128(z)
    acc = out is not None
    g = out if acc else torch.empty_like(zt)
    N.check(N.lib().ed_gf_continued_fraction(N.ptr(a), N.ptr(b), a.numel(), float(norm2), float(e0), int(sign),
                                             N.ptr(torch.view_as_real(zt)), zt.numel(),
                                             N.ptr(torch.view_as_real(g)), int(acc), _stream()))
    return g


def tevo_sum(lam, w, e0: float, sign: int, times, out: torch.Tensor | None = None) -> torch.Tensor:
    """-i*sign * sum_k w_k exp(-i sign (lam_k - e0) t) for every t (complex128 on device)."""
    la = _as_dev_f64(lam).reshape(-1)
    wt = _as_dev_f64(w).reshape(-1)
    tt = _as_dev_f64(times).reshape(-1)
    if la.numel() != wt.numel():
        raise ValueError("lam and w must have the same length")
    acc = out is not None
    g = out if acc else torch.empty(tt.numel(), dtype=torch.complex128, device=device())
    N.check(N.lib().ed_tevo_sum(N.ptr(la), N.ptr(wt), la.numel(), float(e0), int(sign), N.ptr(tt), tt.numel(),
                                N.ptr(torch.view_as_real(g)), int(acc), _stream()))
    return g


def laplace_t2z(times, gf_t, z, method: str = "lin") -> torch.Tensor:
    """int_{t_0}^{t_last} e^{izt} g(t) dt of samples g(t_j) (piecewise-linear "lin" or "trapz")."""
    tt = _as_dev_f64(times).reshape(-1)
    gt = _as_dev_c128(gf_t).reshape(-1)
    zt = _as_dev_c128(z).reshape(-1)
    if tt.numel() != gt.numel():
        raise ValueError("times and gf_t must have the same length")
    m = {"lin": 0, "trapz": 1}[method]
    out = torch.empty_like(zt)
    N.check(N.lib().ed_laplace_t2z(N.ptr(tt), N.ptr(torch.view_as_real(gt)), tt.numel(),
                                   N.ptr(torch.view_as_real(zt)), zt.numel(), m, N.ptr(torch.view_as_real(out)),
                                   _stream()))
    return out


def lehmann_accumulate(evals, evals_p1, overlap, beta: float, emin: float, z, g: torch.Tensor) -> torch.Tensor:
    e = _as_dev_f64(evals)
    ep = _as_dev_f64(evals_p1)
    ov = _as_dev_f64(overlap)
    zt = _as_dev_c128(z)
    if ov.shape != (ep.numel(), e.numel()):
        raise ValueError("overlap must be (len(evals_p1), len(evals))")
    N.check(N.lib().ed_lehmann_accumulate(N.ptr(e), e.numel(), N.ptr(ep), ep.numel(), N.ptr(ov), float(beta),
                                          float(emin), N.ptr(torch.view_as_real(zt)), zt.numel(),
                                          N.ptr(torch.view_as_real(g)), _stream()))
    return g
