"""Batched form: many sectors or realisations solved in one persistent launch.

No reference counterpart — cmpy solves sector after sector (cmpy/exactdiag.py:24-43, and
gf_lehmann at exactdiag.py:215-245). Here every problem is a fixed-point sector plan, and one
launch of ``ed_batch_lanczos`` runs all their Lanczos recurrences (one CTA per problem, a
device work queue, largest first). The launch configuration (threads per CTA, CTAs per SM) is
picked by the autotuner ``ed_batch_tune``; repeated batched sequences can be replayed from a
CUDA graph (``BatchGraph``).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _native as N
from . import engine as E

__all__ = ["Batch", "BatchResult", "groundstate_all_sectors", "groundstates", "greens_functions_batched",
           "BatchGraph"]


# tuned launch configurations: (device, problem dimensions, tune steps) -> (threads,
# ctas_per_sm, cluster_size, ms)
_tune_cache: dict = {}


@dataclass
class BatchResult:
    energy: torch.Tensor      # [n]
    steps: torch.Tensor       # [n] int32
    residual: torch.Tensor    # [n]
    alpha: torch.Tensor       # [n, K]
    beta: torch.Tensor        # [n, K+1]; beta[:, 0] = start norm
    vectors: list | None      # ground states (views into one buffer) when requested


class Batch:
    """A set of fixed-point sector plans solved together."""

    def __init__(self, plans: Sequence[E.Plan]):
        self.plans = list(plans)  # keep the plans alive
        arr = (C.c_void_p * len(self.plans))(*[p.handle.value for p in self.plans])
        h = C.c_void_p()
        N.check(N.lib().ed_batch_create(arr, len(self.plans), C.byref(h)))
        self._h = h
        self.n = len(self.plans)
        self.dims = [p.dim for p in self.plans]
        self.device_index = torch.cuda.current_device()
        self._ws = torch.empty(0, dtype=torch.uint8, device=E.device())
        self.threads = 0
        self.ctas_per_sm = 0
        self.cluster_size = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().ed_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def workspace(self, max_steps: int, threads: int = 0, ctas_per_sm: int = 0, cluster_size: int = 0) -> torch.Tensor:
        nb = C.c_size_t()
        N.check(N.lib().ed_batch_workspace(self._h, int(max_steps), int(threads), int(ctas_per_sm), int(cluster_size),
                                           C.byref(nb)))
        if self._ws.numel() < nb.value:
            self._ws = torch.empty(int(nb.value), dtype=torch.uint8, device=E.device())
        return self._ws

    def _outputs(self, K):
        dev = E.device()
        return (torch.empty((self.n, K), dtype=torch.float64, device=dev),
                torch.empty((self.n, K + 1), dtype=torch.float64, device=dev),
                torch.empty(self.n, dtype=torch.float64, device=dev),
                torch.empty(self.n, dtype=torch.float64, device=dev),
                torch.empty(self.n, dtype=torch.int32, device=dev))

    def tune(self, tune_steps: int = 40):
        """Pick threads per CTA, CTAs per SM and the cluster size per problem by timing the
        candidates; returns (threads, ctas_per_sm, cluster_size, ms). The choice is cached per
        device and problem-dimension list, so batches of the same shape tune once."""
        key = (self.device_index, tuple(self.dims), int(tune_steps))
        hit = _tune_cache.get(key)
        if hit is not None:
            self.threads, self.ctas_per_sm, self.cluster_size = hit[:3]
            return hit
        # size the workspace for the largest candidate grid
        best = 0
        for t, ps, cs in ((128, 4, 1), (256, 2, 1), (256, 4, 1), (512, 1, 1), (512, 2, 1), (1024, 1, 1),
                          (512, 2, 2), (1024, 1, 2), (512, 2, 4), (1024, 1, 4), (512, 2, 8), (1024, 1, 8)):
            nb = C.c_size_t()
            N.check(N.lib().ed_batch_workspace(self._h, int(tune_steps), t, ps, cs, C.byref(nb)))
            best = max(best, nb.value)
        if self._ws.numel() < best:
            self._ws = torch.empty(int(best), dtype=torch.uint8, device=E.device())
        a, b, e, r, s = self._outputs(tune_steps)
        th, ps, cs, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        N.check(N.lib().ed_batch_tune(self._h, int(tune_steps), N.ptr(self._ws), self._ws.numel(), N.ptr(a), N.ptr(b),
                                      N.ptr(e), N.ptr(r), N.ptr(s), C.byref(th), C.byref(ps), C.byref(cs),
                                      C.byref(ms), E._stream()))
        self.threads, self.ctas_per_sm, self.cluster_size = int(th.value), int(ps.value), int(cs.value)
        _tune_cache[key] = (self.threads, self.ctas_per_sm, self.cluster_size, float(ms.value))
        return _tune_cache[key]

    def lanczos(self, max_steps: int = 300, tol: float = 1e-12, check_every: int = 10, seed: int = 0,
                starts: Sequence[torch.Tensor] | None = None, want_vector: bool = False,
                out: BatchResult | None = None) -> BatchResult:
        """Ground states (and optionally vectors) of every problem. Asynchronous: the result
        tensors are filled on the current stream."""
        K = int(max_steps)
        ws = self.workspace(K, self.threads, self.ctas_per_sm, self.cluster_size)
        if out is None:
            a, b, e, r, s = self._outputs(K)
            vecs = None
            if want_vector:
                vbuf = torch.empty(sum(self.dims), dtype=torch.float64, device=E.device())
                offs = np.concatenate([[0], np.cumsum(self.dims)[:-1]]).astype(np.int64)
                vecs = [vbuf[o:o + d] for o, d in zip(offs, self.dims)]
                self._voff = torch.as_tensor(offs).to(E.device())
                self._vbuf = vbuf
            out = BatchResult(e, s, r, a, b, vecs)
        starts_ptr = None
        if starts is not None:
            st = [E._as_dev_f64(x).reshape(-1) for x in starts]
            if [x.numel() for x in st] != self.dims:
                raise ValueError("start vectors must match the problem dimensions")
            self._starts_keep = st
            self._starts_dev = torch.as_tensor(np.array([x.data_ptr() for x in st], dtype=np.int64)).to(E.device())
            starts_ptr = self._starts_dev.data_ptr()
        N.check(N.lib().ed_batch_lanczos(
            self._h, K, float(tol), int(check_every), int(seed), starts_ptr, int(bool(want_vector)), N.ptr(ws),
            ws.numel(), N.ptr(out.alpha), N.ptr(out.beta), N.ptr(out.energy), N.ptr(out.residual), N.ptr(out.steps),
            N.ptr(self._vbuf) if want_vector else None, N.ptr(self._voff) if want_vector else None,
            int(self.threads), int(self.ctas_per_sm), int(self.cluster_size), E._stream()))
        return out


def batch_cf(res: BatchResult, e0: torch.Tensor, sign: int, z, g: torch.Tensor | None = None) -> torch.Tensor:
    """Add the continued fraction of every problem of a batch result to g[n, nz]."""
    zt = E._as_dev_c128(z)
    n, K = res.alpha.shape
    if g is None:
        g = torch.zeros((n, zt.numel()), dtype=torch.complex128, device=zt.device)
    N.check(N.lib().ed_batch_gf_continued_fraction(n, K, N.ptr(res.alpha), N.ptr(res.beta), N.ptr(res.steps),
                                                   N.ptr(E._as_dev_f64(e0)), int(sign),
                                                   N.ptr(torch.view_as_real(zt)), zt.numel(),
                                                   N.ptr(torch.view_as_real(g)), E._stream()))
    return g


def groundstate_all_sectors(model, max_steps: int = 300, tol: float = 1e-12, check_every: int = 10,
                            tune: bool = True, want_vector: bool = False):
    """Ground state of every (n_up, n_dn) sector of a model in one persistent launch (the
    batched counterpart of cmpy's compute_groundstate, exactdiag.py:24-43).
    Returns (fillings, BatchResult)."""
    fillings = list(model.basis.iter_fillings())
    plans = [model.plan(nu, nd) for nu, nd in fillings]
    b = Batch(plans)
    if tune:
        b.tune(min(40, max_steps))
    res = b.lanczos(max_steps=max_steps, tol=tol, check_every=check_every, want_vector=want_vector)
    return fillings, res, b


def groundstates(plans: Sequence[E.Plan], max_steps: int = 300, tol: float = 1e-12, check_every: int = 10,
                 want_vector: bool = True, tune: bool = True):
    b = Batch(plans)
    if tune:
        b.tune(min(40, max_steps))
    return b.lanczos(max_steps=max_steps, tol=tol, check_every=check_every, want_vector=want_vector), b


def greens_functions_batched(models, sectors, z, pos: int = 0, sigma: int = 1, gs_steps: int = 300,
                             gf_levels: int = 200, tol: float = 1e-12, tune: bool = True):
    """Zero-temperature G(z) of many models (e.g. disorder realisations), each in its own
    sector: batched ground states with vectors, c^dag / c on every ground state, batched
    Lanczos coefficients in the neighbouring sectors and a batched continued fraction.
    Returns (energies [n], G [n, nz])."""
    # the ground-state sector and its two neighbours of every model, from one descriptor each
    trip = []
    for m, (nu, nd) in zip(models, sectors):
        want = [(nu, nd)]
        for delta in (1, -1):
            tu, td = (nu + delta, nd) if sigma == 1 else (nu, nd + delta)
            want.append((tu, td) if (0 <= tu <= m.num_sites and 0 <= td <= m.num_sites) else None)
        trip.append(m.plans(want))
    plans = [t[0] for t in trip]
    gs, gb = groundstates(plans, gs_steps, tol, 10, True, tune)
    # host offsets of the ground states in the batch's vector buffer
    gs_off = np.zeros(len(plans), dtype=np.int64)
    if len(plans) > 1:
        gs_off[1:] = np.cumsum(gb.dims)[:-1]
    zt = E._as_dev_c128(z)
    g = torch.zeros((len(plans), zt.numel()), dtype=torch.complex128, device=zt.device)
    for slot, (delta, create, sign) in enumerate(((1, True, 1), (-1, False, -1)), start=1):
        idx = [i for i, t in enumerate(trip) if t[slot] is not None]
        tplans = [trip[i][slot] for i in idx]
        if not tplans:
            continue
        # c^dag / c on every ground state in one native call
        ybuf, y_off = E.apply_fermion_batch([plans[i] for i in idx], tplans, pos, sigma, create, gb._vbuf,
                                            gs_off[idx])
        starts = [ybuf[o:o + t.dim] for o, t in zip(y_off.tolist(), tplans)]
        b = Batch(tplans)
        if tune:
            b.tune(min(40, gf_levels))
        res = b.lanczos(max_steps=gf_levels, tol=0.0, check_every=0, starts=starts)
        part = batch_cf(res, gs.energy[idx], sign, zt)
        g[idx] += part
    return gs.energy, g


class BatchGraph:
    """Captures one batched Lanczos launch (and its queue reset) in a CUDA graph for replay."""

    def __init__(self, batch: Batch, **kw):
        self.batch = batch
        self.kw = kw
        batch.lanczos(**kw)  # warm-up: sizes the workspace and outputs outside the capture
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        self.out = None
        with torch.cuda.graph(self.graph):
            self.out = batch.lanczos(**kw)

    def replay(self) -> BatchResult:
        self.graph.replay()
        return self.out
