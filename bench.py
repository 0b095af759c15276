#!/usr/bin/env python
"""Benchmark of the plain exact-diagonalisation path on one GB300 (or N replicas).

Workload (one "step"): 1D Hubbard ring of 14 sites, periodic, t=1, U=4, mu=U/2, half filling
n_up = n_dn = 7 (dimension 3432^2 = 11,778,624, FP64 vectors of 94 MB):
  * Lanczos ground state, 250 steps, Ritz vector formed on the device;
  * continued-fraction local Green's function on site 0 (spin up), 200 Lanczos levels for the
    electron part (8,7) and the hole part (6,7), on 4096 real frequencies in [-10, 10] with
    eta = 0.02 and 2048 Matsubara frequencies at beta = 50.
Metric: H*v GB/s — algorithmic matvec bytes (16 * D per H*v: x read once, y written once) of
all H*v in the step divided by the step time — plus the ground-state time. Inputs are
synthetic and deterministic (seeded start vector). The Krylov store of one step (23.6 GB) is
far larger than L2, so no extra L2 flush is needed between steps.

``--impl reference`` times the reference's CPU path (COO triplets -> scipy CSR -> H*v) on a
bounded row sample of the same sector with the oracle's restatement of the reference
arithmetic, using all host threads.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SITES, N_UP, N_DN = 14, 7, 7
U, T, MU = 4.0, 1.0, 2.0
LZ_STEPS, GF_LEVELS = 250, 200
N_REAL, N_MATS, ETA, BETA = 4096, 2048, 0.02, 50.0
METRIC = "H·v GB/s & GS time, 14-site Hubbard; batched & adjoint vs plain, same GPU, 1e-10"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and adjoint measurements")
    ap.add_argument("--matvec-only", type=int, default=0,
                    help="time N fixed-point matvecs of the 14-site sector alone (kernel profiling)")
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES), default=None,
                    help="run one small single-kernel workload once (for ncu captures) and exit")
    return ap.parse_args()


def run_matvec_only(n: int):
    """N fixed-point Lanczos steps of the 14-site (7,7) sector per matvec variant (7 = single-pass
    with renumbered dn states, 6 = two-pass stripes, 5 = banded two-pass sweep, 3 = single-pass),
    the matvec launches timed with CUDA events on the launching stream (one JSON line per
    variant)."""
    import torch

    from cmpy_gb300 import engine as E

    bonds = [(i, j, T) for i, j in sorted(ring_bonds(N_SITES))]
    plan = E.Plan.fermion(N_SITES, [-MU] * N_SITES, [U] * N_SITES, bonds, N_UP, N_DN)
    v0 = torch.rand(plan.dim, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))
    peak, _ = peaks()
    kernels = {7: "k_bfp_hub_matvec3 (dn renumbered, per-chunk lists)", 6: "k_stripe_up + k_stripe_dn",
               5: "k_sweep_up + k_sweep_dn", 3: "k_bfp_hub_matvec3"}
    for var in (7, 6, 5, 3):
        plan.set_matvec_variant(var)
        if plan.matvec_variant != var:
            continue
        E.lanczos(plan, max_steps=4, want_vector=False, v0=v0)  # warm-up
        r = E.lanczos(plan, max_steps=n, want_vector=False, v0=v0, profile=True)
        us = 1e3 * r.matvec_ms / max(r.matvecs, 1)
        gbs = 16.0 * plan.dim / (us * 1e-6) / 1e9
        print(json.dumps({"variant": var, "kernels": kernels[var],
                          "dim": plan.dim, "matvecs": r.matvecs, "matvec_us": round(us, 2), "gbs": round(gbs, 1),
                          "frac": round(gbs / peak, 4), "alpha0": float(r.alpha[0]), "energy": r.energy}), flush=True)
    plan.set_matvec_variant(0)


def case_gf14(steps: int = 12) -> None:
    """Particle-sector Lanczos of the 14-site Hubbard ring (U=4, mu=2, t=1), sector (8,7),
    D = 10,306,296, from a seeded uniform start vector, 12 steps in block fixed point (three
    rotating vectors, ~0.5 GB on the device): the update kernel and the integer matvec of the
    benchmark step without its 23.6 GB Krylov store."""
    import torch

    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(14, True), inter=4.0, mu=2.0, hop=1.0)
    p = m.plan(8, 7)
    g = torch.Generator(device="cuda").manual_seed(3)
    s = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    a, b, _ = E.lanczos_coeffs(p, s, max_steps=steps)
    torch.cuda.synchronize()
    print(f"gf14: {a.numel()} steps, alpha_0 = {float(a[0]):.12f}")


def case_adjoint64(n: int = 64) -> None:
    """The batched part of the `adjoint` extra: 64 SIAMs with 1 impurity + 9 bath sites,
    sector (5,5), 1024 Matsubara frequencies at beta=100, seeded bath parameters (numpy
    default_rng(5)); forward and backward once."""
    import torch

    from cmpy_gb300.adjoint import greens_function_ad_batch, siam_parameters

    rng = np.random.default_rng(5)
    z = 1j * (2 * np.arange(1024) + 1) * np.pi / 100.0
    eb = torch.tensor(rng.uniform(-2, 2, (n, 9)), dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor(rng.uniform(0.1, 0.6, (n, 9)), dtype=torch.float64, device="cuda", requires_grad=True)
    u = torch.tensor(4.0, dtype=torch.float64, device="cuda")
    e_imp = torch.tensor(0.0, dtype=torch.float64, device="cuda")
    rows = [siam_parameters(u, e_imp, eb[i], v[i]) for i in range(n)]
    th = torch.stack([r[0] for r in rows])
    n_sites, bonds, width = rows[0][1], rows[0][2], rows[0][3]
    g = greens_function_ad_batch(th, n_sites, bonds, (5, 5), z, sign_width=width, gs_steps=250, gf_levels=150,
                                 ckpt=16)
    torch.sum(torch.abs(g) ** 2).backward()
    torch.cuda.synchronize()
    print(f"adjoint64: |grad| = {float(eb.grad.abs().sum() + v.grad.abs().sum()):.6f}")


def case_sweep10() -> None:
    """The `batched_sweep` workload (all 121 sectors of the 10-site Hubbard ring, U=6, mu=3,
    t=1; 300 steps, tol 1e-12, tested every 10 steps) in one batched launch with a fixed
    configuration (512 threads, 2 CTAs per SM, clusters of 4 CTAs), run twice (the second
    launch is the one to capture)."""
    import torch

    from cmpy_gb300.batched import Batch
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(10, True), inter=6.0, mu=3.0, hop=1.0)
    plans = [m.plan(nu, nd) for nu, nd in m.basis.iter_fillings()]
    b = Batch(plans)
    b.threads, b.ctas_per_sm, b.cluster_size = 512, 2, 4
    for _ in range(2):
        r = b.lanczos(max_steps=300, tol=1e-12, check_every=10)
    torch.cuda.synchronize()
    print(f"sweep10: {len(plans)} sectors, E0 = {float(r.energy.min()):.12f}")


def case_gs14(steps: int = 250) -> None:
    """The benchmark's ground-state run alone: 14-site ring (7,7), 250 block-fixed-point Lanczos
    steps with the Ritz vector (Krylov store 23.6 GB), then the final tridiagonal eigenpair and
    Ritz kernels; twice (the first run warms the plan and the workspace)."""
    import torch

    from cmpy_gb300 import engine as E

    bonds = [(i, j, T) for i, j in sorted(ring_bonds(N_SITES))]
    plan = E.Plan.fermion(N_SITES, [-MU] * N_SITES, [U] * N_SITES, bonds, N_UP, N_DN)
    v0 = torch.rand(plan.dim, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))
    for _ in range(2):
        r = E.lanczos(plan, max_steps=steps, want_vector=True, v0=v0)
    torch.cuda.synchronize()
    print(json.dumps({"case": "gs14", "steps": r.steps, "energy": r.energy}))


def case_chain6() -> None:
    """The 6-site open chain workload (U=4, mu=2, t=1): ground state of (3,3) and the T=0
    Lehmann G at 512 frequencies, whose dense eigenpairs of the (4,3) and (2,3) sectors (order
    300 each, one batch) are the dense eigensolver's kernels; three times (the first warms
    the plans)."""
    for _ in range(3):
        out = run_chain6()
    print(json.dumps({"case": "chain6", "ms": out["ms"], "energy": out["gs_energy"]}))


PROFILE_CASES = {"gf14": case_gf14, "adjoint64": case_adjoint64, "sweep10": case_sweep10, "gs14": case_gs14,
                 "chain6": case_chain6}


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def frequencies():
    w = np.linspace(-10.0, 10.0, N_REAL) + 1j * ETA
    iwn = 1j * (2 * np.arange(N_MATS) + 1) * np.pi / BETA
    return np.concatenate([w, iwn])


def ring_bonds(n):
    return [(i, (i + 1) % n) if i < (i + 1) % n else ((i + 1) % n, i) for i in range(n)]


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------


def run_ours(args, rank, world, dist):
    import torch

    from cmpy_gb300 import engine as E

    dev_index = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev_index)
    bonds = [(i, j, T) for i, j in sorted(ring_bonds(N_SITES))]
    eps = [-MU] * N_SITES
    uu = [U] * N_SITES
    plan = E.Plan.fermion(N_SITES, eps, uu, bonds, N_UP, N_DN)
    plan_p = E.Plan.fermion(N_SITES, eps, uu, bonds, N_UP + 1, N_DN)
    plan_m = E.Plan.fermion(N_SITES, eps, uu, bonds, N_UP - 1, N_DN)
    D, Dp, Dm = plan.dim, plan_p.dim, plan_m.dim
    z = frequencies()
    zt = torch.as_tensor(z).cuda()
    gen = torch.Generator(device="cuda").manual_seed(1234 + rank)
    v0 = torch.rand(D, dtype=torch.float64, device="cuda", generator=gen)
    ws = torch.empty(0, dtype=torch.uint8, device="cuda")
    # workspace sized once (Krylov store for the ground state)
    res0 = None

    def step(v0_dev, profile):
        nonlocal ws
        r = E.lanczos(plan, max_steps=LZ_STEPS, want_vector=True, v0=v0_dev, workspace=ws if ws.numel() else None,
                      profile=profile)
        g = torch.zeros_like(zt)
        phi = plan.apply_fermion(plan_p, 0, 1, True, r.vector)
        chi = plan.apply_fermion(plan_m, 0, 1, False, r.vector)
        # the particle and the hole run in one call (their steps interleave on the GPU)
        (a, b, nrm), (a2, b2, nrm2) = E.lanczos_coeffs_multi([(plan_p, phi), (plan_m, chi)], max_steps=GF_LEVELS)
        E.continued_fraction(a, b, nrm * nrm, zt, e0=r.energy, sign=1, out=g)
        E.continued_fraction(a2, b2, nrm2 * nrm2, zt, e0=r.energy, sign=-1, out=g)
        return r, g, (a.numel(), a2.numel())

    # allocate the workspace once and reuse it
    import ctypes as C

    from cmpy_gb300 import _native as N

    prm = N.LanczosParams()
    prm.max_steps, prm.want_vector = LZ_STEPS, 1
    nb = C.c_size_t()
    N.check(N.lib().ed_lanczos_workspace(plan.handle, C.byref(prm), C.byref(nb)))
    ws = torch.empty(int(nb.value), dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        res0, g0, lv = step(v0, False)
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    stream = torch.cuda.current_stream()
    mv_ms, mv_n, gs_ms = 0.0, 0, 0.0
    launches0 = E.launch_count()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev_index) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        levels = []
        for _ in range(args.steps):
            r, g, lv = step(v0, True)
            mv_ms += r.matvec_ms
            mv_n += r.matvecs
            levels.append((r.steps, lv))
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = E.launch_count() - launches0
    elapsed = e0.elapsed_time(e1) / 1e3  # s
    # ground-state part alone (separately timed, same device-resident inputs)
    g0e, g1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0e.record(stream)
    rgs = E.lanczos(plan, max_steps=LZ_STEPS, want_vector=True, v0=v0, workspace=ws)
    g1e.record(stream)
    torch.cuda.synchronize()
    gs_ms = g0e.elapsed_time(g1e)

    # matvecs per step and bytes
    mv_per_step = [s + la + lb for s, (la, lb) in levels]
    bytes_per_step = [16.0 * (D * s + Dp * la + Dm * lb) for s, (la, lb) in levels]
    t_max = elapsed
    if dist is not None:
        import torch.distributed as tdist

        tt = torch.tensor([elapsed], dtype=torch.float64, device="cuda")
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * sum(bytes_per_step) / t_max / 1e9

    # e2e: public API with host buffers (pinned start vector in, GS vector and G(z) out)
    h_v0 = torch.empty(D, dtype=torch.float64, pin_memory=True)
    h_v0.copy_(v0.cpu())
    h_z = torch.as_tensor(z).pin_memory()
    h_psi = torch.empty(D, dtype=torch.float64, pin_memory=True)
    h_g = torch.empty(len(z), dtype=torch.complex128, pin_memory=True)
    barrier()
    torch.cuda.synchronize()
    x0 = torch.cuda.Event(enable_timing=True)
    x1 = torch.cuda.Event(enable_timing=True)
    x0.record(stream)
    for _ in range(args.steps):
        vd = h_v0.to("cuda", non_blocking=True)
        zd = h_z.to("cuda", non_blocking=True)
        r = E.lanczos(plan, max_steps=LZ_STEPS, want_vector=True, v0=vd, workspace=ws)
        g = torch.zeros_like(zd)
        phi = plan.apply_fermion(plan_p, 0, 1, True, r.vector)
        chi = plan.apply_fermion(plan_m, 0, 1, False, r.vector)
        (a, b, nrm), (a2, b2, nrm2) = E.lanczos_coeffs_multi([(plan_p, phi), (plan_m, chi)], max_steps=GF_LEVELS)
        E.continued_fraction(a, b, nrm * nrm, zd, e0=r.energy, sign=1, out=g)
        E.continued_fraction(a2, b2, nrm2 * nrm2, zd, e0=r.energy, sign=-1, out=g)
        h_psi.copy_(r.vector, non_blocking=True)
        h_g.copy_(g, non_blocking=True)
    x1.record(stream)
    torch.cuda.synchronize()
    e2e_s = x0.elapsed_time(x1) / 1e3
    if dist is not None:
        import torch.distributed as tdist

        tt = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e_value = world * sum(bytes_per_step) / e2e_s / 1e9
    h2d = D * 8 + len(z) * 16
    d2h = D * 8 + len(z) * 16

    peak, peak_kind = peaks()
    achieved = (16.0 * D * mv_n) / (mv_ms / 1e3) / 1e9 if mv_ms > 0 else None
    traffic = matvec_traffic()
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_max / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "arithmetic": ("int64 block fixed point (56-bit mantissas, one exponent per vector) for the Krylov vectors "
                       "and H*v; FP64 for alpha, beta, the tridiagonal solve and the continued fraction"),
        "data": "synthetic (deterministic model, seeded uniform start vector)",
        "config": {
            "workload": "hubbard_ring14_half_filling_gs250_cf200",
            "n_sites": N_SITES, "sector": [N_UP, N_DN], "dim": D, "U": U, "t": T, "mu": MU,
            "lanczos_steps": LZ_STEPS, "gf_levels": GF_LEVELS, "n_real_freq": N_REAL, "eta": ETA,
            "n_matsubara": N_MATS, "beta": BETA, "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (23.6 GB Krylov store per step)",
        },
        "gs_time_ms": round(gs_ms, 3),
        "gs_energy": rgs.energy,
        "matvecs_per_step": mv_per_step[0] if mv_per_step else None,
        "matvecs_per_s": round(world * sum(mv_per_step) / t_max, 1),
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None,
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4) if achieved else None,
            "traffic": traffic,
            "kernel": (f"k_bfp_hub_matvec3 (integer H·v, matvec variant {plan.matvec_variant}"
                       f"{': dn states renumbered by hop count' if plan.matvec_variant == 7 else ''}, "
                       "16*D bytes per launch)"),
            "peak_source": f"{peak_kind} (hbm_gbs, burst copy)",
            "matvec_us": round(mv_ms / mv_n * 1e3, 2) if mv_n else None,
        },
        "e2e": {"value": round(e2e_value, 3), "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    return out


def _timed(fn):
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = fn()
    e1.record()
    torch.cuda.synchronize()
    return out, e0.elapsed_time(e1)


def run_batched_sweep():
    """Batched sweep: all 121 sectors of the 10-site Hubbard ring (t=1, U=6, mu=3) — one persistent
    batched launch vs per-sector plain launches, same residual tolerance (E0 to 1e-10)."""
    import torch

    from cmpy_gb300 import engine as E
    from cmpy_gb300.batched import Batch
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(10, True), inter=6.0, mu=3.0, hop=1.0)
    fillings = list(m.basis.iter_fillings())
    plans = [m.plan(a, b) for a, b in fillings]
    b = Batch(plans)
    th, ps, cs, _ = b.tune(40)
    b.lanczos(max_steps=300, tol=1e-12, check_every=10)  # warm
    res, t_batch = _timed(lambda: b.lanczos(max_steps=300, tol=1e-12, check_every=10))
    e_batch = res.energy.cpu().numpy()

    def plain():
        return [E.lanczos(p, max_steps=min(300, p.dim), want_vector=False, tol=1e-12, check_every=10).energy
                for p in plans]

    plain()
    e_plain, t_plain = _timed(plain)
    e_plain = np.array(e_plain)
    i = int(np.argmin(e_batch))
    return {
        "workload": "hubbard_ring10_U6_all_121_sectors",
        "batched_ms": round(t_batch, 3),
        "plain_per_sector_ms": round(t_plain, 3),
        "speedup": round(t_plain / t_batch, 2),
        "gs_energy": float(e_batch[i]),
        "gs_sector": list(fillings[i]),
        "max_rel_diff_vs_plain": float(np.max(np.abs(e_batch - e_plain) / np.maximum(1.0, np.abs(e_plain)))),
        "tuned": {"threads": th, "ctas_per_sm": ps, "cluster_size": cs},
        "launches": "1 persistent batched kernel vs per-sector Lanczos sequences",
    }


def _dense_lehmann(plan_gs, plan_t, psi, e0, z, create: bool):
    """T=0 Lehmann sum of one neighbouring sector from its dense eigenpairs (device eigh):
    the accuracy check of the continued fractions on the real axis."""
    import torch

    H = plan_t.dense()
    w, V = torch.linalg.eigh(H)
    phi = plan_gs.apply_fermion(plan_t, 0, 1, create, psi)
    amp = (V.T @ phi) ** 2
    zt = torch.as_tensor(z).cuda()
    if create:
        return (amp[None, :] / (zt[:, None] - (w[None, :] - e0))).sum(1)
    return (amp[None, :] / (zt[:, None] + (w[None, :] - e0))).sum(1)


def run_disorder_batch(n_real: int = 512, n_freq: int = 1024, n_dense: int = 8):
    """Batched disorder: realisations of the 8-site Anderson-Hubbard chain (eps ~ U[-1,1],
    U=4, t=1, mu=2, n_up, n_dn ~ U{2..5}, numpy default_rng(2024)); ground state + G(w) at
    n_freq real frequencies in [-8, 8] (eta = 0.05) and 256 Matsubara points (beta = 10) each.
    2000 Lanczos levels (no reorthogonalisation) converge the continued fractions on the real
    axis (1000 leave up to ~1e-6 in slowly converging realisations); the accuracy is checked against dense-eigh Lehmann sums on `n_dense` realisations
    (the largest sectors first) and against the per-realisation runs."""
    import torch

    from cmpy_gb300.batched import greens_functions_batched
    from cmpy_gb300.exactdiag import gf_continued_fraction, groundstate_sector
    from cmpy_gb300.models import ChainLattice, HubbardModel

    rng = np.random.default_rng(2024)
    lat = ChainLattice(8, False)
    models = [HubbardModel(lat, inter=4.0, eps=rng.uniform(-1, 1, 8), mu=2.0, hop=1.0) for _ in range(n_real)]
    sectors = [(int(a), int(b)) for a, b in rng.integers(2, 6, size=(n_real, 2))]
    n_mats = 256
    z = np.concatenate([np.linspace(-8, 8, n_freq) + 0.05j, 1j * (2 * np.arange(n_mats) + 1) * np.pi / 10.0])
    levels = 2000
    for m_, s_ in zip(models, sectors):  # plans (setup, untimed)
        for d in (-1, 0, 1):
            m_.plan(s_[0] + d, s_[1])
    # warm-up on the full set: the launch configurations are tuned (once per batch shape, cached)
    greens_functions_batched(models, sectors, z, gf_levels=levels)
    (eb, gb), t_batch = _timed(lambda: greens_functions_batched(models, sectors, z, gf_levels=levels))
    n_plain = min(n_real, 64)

    def plain():
        out = []
        for m_, (a, b) in zip(models[:n_plain], sectors[:n_plain]):
            e0, psi = groundstate_sector(m_, a, b, max_steps=300, tol=1e-12)
            out.append((e0, psi, gf_continued_fraction(m_, z, a, b, e0, psi, n_lev=levels)))
        return out

    plain()
    pl, t_plain = _timed(plain)
    gdiff = max(float(np.max(np.abs(gb[i].cpu().numpy()[:n_freq] - pl[i][2][:n_freq]))) for i in range(n_plain))
    gdiff_m = max(float(np.max(np.abs(gb[i].cpu().numpy()[n_freq:] - pl[i][2][n_freq:]))) for i in range(n_plain))
    ediff = max(abs(float(eb[i]) - pl[i][0]) / abs(pl[i][0]) for i in range(n_plain))
    # dense check: the largest sectors among the plain sample
    order = sorted(range(n_plain), key=lambda i: -models[i].plan(*sectors[i]).dim)[:n_dense]
    derr = 0.0
    for i in order:
        m_, (a, b) = models[i], sectors[i]
        e0, psi = pl[i][0], pl[i][1]
        g_d = _dense_lehmann(m_.plan(a, b), m_.plan(a + 1, b), psi, e0, z, True)
        g_d = g_d + _dense_lehmann(m_.plan(a, b), m_.plan(a - 1, b), psi, e0, z, False)
        derr = max(derr, float(torch.max(torch.abs(gb[i] - g_d))))
    return {
        "workload": f"anderson_hubbard_chain8_{n_real}_realisations_gs_gf{n_freq}",
        "batched_ms": round(t_batch, 3),
        "plain_ms_extrapolated": round(t_plain * n_real / n_plain, 3),
        "plain_sample": n_plain,
        "speedup": round(t_plain * n_real / n_plain / t_batch, 2),
        "max_rel_energy_diff": ediff,
        "max_abs_gf_diff_matsubara": gdiff_m,
        "max_abs_gf_diff_real_axis": gdiff,
        "max_abs_gf_err_vs_dense_eigh": derr,
        "dense_checked": [list(sectors[i]) for i in order],
        "eta": 0.05,
        "n_matsubara": n_mats,
        "gf_levels": levels,
    }


def run_adjoint(n_siam: int = 64, n_freq: int = 1024, n_single: int = 8):
    """Adjoint: SIAMs with 1 impurity + 9 bath sites (star), U=4, eps_d=-U/2, sector (5,5)
    (eps_bath ~ U[-2,2], V ~ U[0.1,0.6], numpy default_rng(5)); G_imp(i w_n) on n_freq
    Matsubara frequencies (beta=100) and the adjoint gradient of a least-squares loss against a
    target hybridisation with 30 poles, w.r.t. bath energies and V. Single problems (forward /
    backward cost, after one warm-up) and all n_siam SIAMs at once (batched tape)."""
    import torch

    from cmpy_gb300.adjoint import greens_function_ad, greens_function_ad_batch, siam_parameters

    rng = np.random.default_rng(5)
    ek = rng.uniform(-2, 2, 30)
    z = 1j * (2 * np.arange(n_freq) + 1) * np.pi / 100.0
    gt = torch.as_tensor(1.0 / (z - np.sum(0.3**2 / (z[:, None] - ek[None, :]), axis=1))).cuda()
    eb = torch.tensor(rng.uniform(-2, 2, (n_siam, 9)), dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor(rng.uniform(0.1, 0.6, (n_siam, 9)), dtype=torch.float64, device="cuda", requires_grad=True)
    u = torch.tensor(4.0, dtype=torch.float64, device="cuda")
    e_imp = torch.tensor(0.0, dtype=torch.float64, device="cuda")
    kw = dict(gs_steps=250, gf_levels=150, ckpt=16)

    def thetas():
        rows = [siam_parameters(u, e_imp, eb[i], v[i]) for i in range(n_siam)]
        return torch.stack([r[0] for r in rows]), rows[0][1], rows[0][2], rows[0][3]

    th, n_sites, bonds, width = thetas()
    fwd, bwd = [], []
    for s in range(n_single + 1):  # the first is a warm-up (lazy kernel loading), not timed
        g, tf = _timed(lambda: greens_function_ad(th[s % n_siam], n_sites, bonds, (5, 5), z, sign_width=width, **kw))
        loss = torch.sum(torch.abs(g - gt) ** 2)
        _, tb = _timed(lambda: loss.backward(retain_graph=True))
        if s > 0:
            fwd.append(tf)
            bwd.append(tb)
    eb.grad = None
    v.grad = None
    th, n_sites, bonds, width = thetas()
    greens_function_ad_batch(th[:2], n_sites, bonds, (5, 5), z, sign_width=width, **kw)  # warm-up
    gall, tbf = _timed(lambda: greens_function_ad_batch(th, n_sites, bonds, (5, 5), z, sign_width=width, **kw))
    lall = torch.sum(torch.abs(gall - gt) ** 2)
    _, tbb = _timed(lambda: lall.backward())
    return {
        "workload": f"siam_1p9_sector55_matsubara{n_freq}_beta100",
        "single_timed": n_single,
        "forward_ms": round(float(np.mean(fwd)), 2),
        "backward_ms": round(float(np.mean(bwd)), 2),
        "backward_over_forward": round(float(np.mean(bwd) / np.mean(fwd)), 3),
        "batch_siams": n_siam,
        "batch_forward_ms": round(tbf, 1),
        "batch_backward_ms": round(tbb, 1),
        "batch_gradients_per_s": round(n_siam * 1e3 / (tbf + tbb), 1),
        "single_gradients_per_s": round(1e3 / float(np.mean(fwd) + np.mean(bwd)), 1),
    }


def run_heisenberg(steps: int = 300):
    """Heisenberg ring N=20, Sz=0 (D=184,756) with per-bond couplings J_ij = 1 + 0.1*N(0,1)
    (numpy default_rng(0), bond (i, i+1 mod 20) in order); `steps` Lanczos steps with full
    reorthogonalisation (CGS2) and the Ritz vector. Vector 1.48 MB: L2-resident, latency bound."""
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import ChainLattice, HeisenbergModel

    n = 20
    rng = np.random.default_rng(0)
    J = np.zeros((n, n))
    for i in range(n):
        k = (i + 1) % n
        J[i, k] = J[k, i] = 1.0 + 0.1 * rng.standard_normal()
    m = HeisenbergModel(ChainLattice(n, True), j=J, jz=J)
    p = m.plan(0)
    D = p.dim
    run = lambda: E.lanczos(p, max_steps=steps, reorth=True, want_vector=True, tol=0.0)  # noqa: E731
    run()
    r, t = _timed(run)
    rp = E.lanczos(p, max_steps=steps, reorth=True, want_vector=True, tol=0.0, profile=True)
    plain = E.lanczos(p, max_steps=steps, reorth=False, want_vector=False, tol=1e-12, check_every=10)
    k = r.steps
    reorth_bytes = sum(2 * 2 * 8 * D * (j + 1) for j in range(k))  # CGS2: 2 passes x (dots + axpy)
    return {
        "workload": "heisenberg_ring20_sz0_randomJ_fullreorth",
        "dim": D,
        "steps": k,
        "total_ms": round(t, 3),
        "ms_per_step": round(t / max(k, 1), 4),
        "matvec_us": round(1e3 * rp.matvec_ms / max(rp.matvecs, 1), 2),
        "matvec_gbs": round(16 * D * rp.matvecs / (rp.matvec_ms * 1e-3) / 1e9, 1) if rp.matvec_ms > 0 else None,
        "reorth_plus_matvec_gbs": round((reorth_bytes + 16 * D * k) / (t * 1e-3) / 1e9, 1),
        "gs_energy": r.energy,
        "residual": r.residual,
        "rel_diff_vs_no_reorth": abs(r.energy - plain.energy) / abs(plain.energy),
    }


def matvec_traffic():
    """DRAM bytes per matvec launch from the committed ncu summary (profiles/), if any."""
    f = ROOT / "profiles" / "k_bfp_hub_matvec3_hubbard14.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ------------------------------------------------------------------------------------------
# CPU reference path (oracle restatement of the reference's COO -> scipy CSR -> H*v)
# ------------------------------------------------------------------------------------------


def cpu_sample(up_rows: int):
    """Reference triplets of the first `up_rows` up-rows of the 14-site (7,7) sector as a CSR
    block (rows = origins). Returns (csr, x, build_s)."""
    import scipy.sparse as sp

    from oracle import ed_oracle as O

    t0 = time.perf_counter()
    up = O.sector_states(N_SITES, N_UP)
    dn = O.sector_states(N_SITES, N_DN)
    eps, uu, bonds, width = O.hubbard_descriptor(N_SITES, [list(b) for b in sorted(ring_bonds(N_SITES))], inter=U,
                                                 hop=T, mu=MU)
    r, c, v = O.coo_fermion_rows(up, dn, eps, uu, bonds, width, up_rows)
    nd = len(dn)
    csr = sp.csr_matrix((v, (r, c)), shape=(up_rows * nd, len(up) * nd))
    build = time.perf_counter() - t0
    x = np.random.default_rng(0).random(len(up) * nd)
    return csr, x, build


def cpu_matvec_rate(csr, x, seconds: float):
    """H*v GB/s of the sample on one host core (scipy's sparse product holds the GIL; this
    process has used the GPU, so no worker processes are forked here: the all-core figure is
    the --impl reference line)."""
    csr @ x
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        csr @ x
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return 16.0 * csr.shape[0] / dt / 1e9, dt


def cpu_baseline_line(seconds: float = 8.0):
    up_rows = 96
    csr, x, build = cpu_sample(up_rows)
    gbs, dt = cpu_matvec_rate(csr, x, seconds)
    return {
        "value": round(gbs, 4),
        "unit": "GB/s",
        "cores": 1,
        "kind": "port",
        "sample": (f"reference COO (oracle restatement) of the first {up_rows} of 3432 up-rows of the 14-site (7,7) "
                   f"sector -> scipy CSR ({csr.nnz} nnz) -> H*v on one core; COO+CSR build {build:.2f} s "
                   f"for the sample ({build * 3432 / up_rows:.0f} s extrapolated to the sector)"),
    }


def _pool_csr_matvec(H, nproc: int):
    """y = H x over `nproc` row blocks of a scipy CSR matrix in forked worker processes (scipy's
    sparse product holds the GIL, so threads would not run in parallel). x and y live in
    anonymous shared memory created before the fork; the blocks are sliced before the fork
    and shared copy-on-write. Only for processes that have made no GPU call (fork).
    Returns (matvec, close)."""
    import mmap
    import multiprocessing as mp

    n = H.shape[0]
    bx, by = mmap.mmap(-1, n * 8), mmap.mmap(-1, n * 8)
    x = np.frombuffer(bx, dtype=np.float64)
    y = np.frombuffer(by, dtype=np.float64)
    cuts = np.linspace(0, n, nproc + 1).astype(int)
    blocks = [H[cuts[i]:cuts[i + 1]] for i in range(nproc)]
    ctx = mp.get_context("fork")

    def worker(i, conn):
        a, b = int(cuts[i]), int(cuts[i + 1])
        while conn.recv():
            y[a:b] = blocks[i] @ x
            conn.send(1)

    conns, procs = [], []
    for i in range(nproc):
        parent, child = ctx.Pipe()
        pr = ctx.Process(target=worker, args=(i, child), daemon=True)
        pr.start()
        conns.append(parent)
        procs.append(pr)

    def mv(v):
        x[:] = np.asarray(v, dtype=np.float64).reshape(-1)
        for c in conns:
            c.send(1)
        for c in conns:
            c.recv()
        return y  # shared buffer: valid until the next call (eigsh copies it out at once)

    def close():
        for c in conns:
            c.send(0)
        for pr in procs:
            pr.join(timeout=10)

    return mv, close


def run_reference(args, rank, world):
    """The reference's CPU path for the 14-site (7,7) sector on this machine's host cores: the
    reference triplets (the oracle's bit-exact restatement of cmpy/operators.py project_* and
    cmpy/models/hubbard.py _ham_data, kind "port": the reference itself is Python that cannot
    run here) -> scipy CSR -> eigsh(k=1, which="SA") as in cmpy/exactdiag.py:37, timed once in
    full (gs_time_s). Each step then times `reps` full-sector CSR H*v (the operation the
    Lanczos/ARPACK iteration repeats), row-blocked over all host threads: the line's value is
    that H*v GB/s (16 bytes per element, as for the GPU arm)."""
    if rank != 0:
        return None
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from oracle import ed_oracle as O

    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    up = O.sector_states(N_SITES, N_UP)
    dn = O.sector_states(N_SITES, N_DN)
    eps, uu, bonds, width = O.hubbard_descriptor(N_SITES, [list(b) for b in sorted(ring_bonds(N_SITES))], inter=U,
                                                 hop=T, mu=MU)
    D = len(up) * len(dn)
    t0 = time.perf_counter()
    r, c, v = O.coo_fermion(up, dn, eps, uu, bonds, width)
    n_trip = int(r.size)
    t1 = time.perf_counter()
    H = sp.csr_matrix((v, (r, c)), shape=(D, D))
    del r, c, v
    t2 = time.perf_counter()
    mv, close = _pool_csr_matvec(H, threads)
    count = [0]

    def counted(x):
        count[0] += 1
        return mv(x)

    op = sla.LinearOperator((D, D), matvec=counted, dtype=np.float64)
    v0 = np.random.default_rng(0).random(D)
    e0 = float(sla.eigsh(op, k=1, which="SA", tol=1e-12, v0=v0, return_eigenvectors=False)[0])
    t3 = time.perf_counter()
    x = np.random.default_rng(1).random(D)
    reps = 4
    for _ in range(args.warmup):
        for _ in range(reps):
            mv(x)
    t4 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(reps):
            mv(x)
    el = time.perf_counter() - t4
    close()
    gbs = 16.0 * D * reps * args.steps / el / 1e9
    sample = (f"full 14-site (7,7) sector: {n_trip} reference triplets (oracle restatement, one thread, "
              f"{t1 - t0:.1f} s) -> scipy CSR ({H.nnz} nnz, {t2 - t1:.1f} s) -> eigsh with the CSR matvec in "
              f"{threads} processes by row blocks ({count[0]} H*v, {t3 - t2:.1f} s); each step {reps} full-sector H*v")
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": round(gbs, 4),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(el / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (deterministic model, seeded start vector)",
        "config": {"workload": "hubbard_ring14_half_filling_gs250_cf200", "n_sites": N_SITES, "sector": [N_UP, N_DN],
                   "dim": D, "U": U, "t": T, "mu": MU, "parallelism": f"{threads} host processes"},
        "same_config": True,
        "gs_time_s": round(t3 - t0, 2),
        "gs_parts_s": {"coo_build": round(t1 - t0, 2), "csr_build": round(t2 - t1, 2), "eigsh": round(t3 - t2, 2)},
        "gs_energy": e0,
        "eigsh_matvecs": count[0],
        "cpu_baseline": {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(gbs, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_chain6():
    """The small correctness workload, timed: 6-site open Hubbard chain, t=1,
    U=4, mu=2, sector (3,3): Lanczos ground state (tol 1e-12) and the T=0 Lehmann Green's
    function on site 0, spin up, at 512 real frequencies in [-8, 8] with eta = 0.05."""
    import torch

    from cmpy_gb300.exactdiag import gf_lehmann_zero_temperature, groundstate_sector
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(6), inter=4.0, mu=2.0, hop=1.0)
    z = np.linspace(-8, 8, 512) + 0.05j

    def run():
        e0, psi = groundstate_sector(m, 3, 3, max_steps=200, tol=1e-12)
        return e0, gf_lehmann_zero_temperature(m, z, e0, psi, 3, 3, pos=0)

    run()
    (e0, g), ms = _timed(run)
    torch.cuda.synchronize()
    return {"workload": "hubbard_chain6_sector33_gs_lehmann512", "ms": round(ms, 3), "gs_energy": e0,
            "g_norm_check": float(-np.sum(g.imag) * (z[1].real - z[0].real) / np.pi)}


def cpu_baseline_heisenberg():
    """The reference's CPU path for the Heisenberg N=20 configuration (same couplings as
    run_heisenberg): its triplets (the oracle's restatement of cmpy/models/heisenberg.py:19-40
    with per-bond J) -> scipy CSR -> eigsh(k=1, which="SA", tol=1e-12) as in
    cmpy/exactdiag.py:37, one host core, timed in full."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from oracle import ed_oracle as O

    n = 20
    rng = np.random.default_rng(0)
    J = np.zeros((n, n))
    for i in range(n):
        k = (i + 1) % n
        J[i, k] = J[k, i] = 1.0 + 0.1 * rng.standard_normal()
    t0 = time.perf_counter()
    states = O.sector_states(n, n // 2)
    neighbors = [[(q - 1) % n, (q + 1) % n] for q in range(n)]
    r, c, v = O.coo_heisenberg(states, O.heisenberg_pairs(neighbors, j=J, jz=J))
    D = len(states)
    H = sp.csr_matrix((v, (r, c)), shape=(D, D))
    t1 = time.perf_counter()
    e0 = float(sla.eigsh(H, k=1, which="SA", tol=1e-12, v0=np.random.default_rng(1).random(D),
                         return_eigenvectors=False)[0])
    t2 = time.perf_counter()
    return {"kind": "port", "cores": 1, "gs_time_s": round(t2 - t0, 3),
            "gs_parts_s": {"coo_csr_build": round(t1 - t0, 3), "eigsh": round(t2 - t1, 3)}, "gs_energy": e0,
            "sample": "full configuration: reference triplets (oracle restatement) -> scipy CSR -> eigsh on one core"}


def cpu_baseline_chain6():
    """The reference's CPU path for the 6-site chain workload (same model as run_chain6): dense sector
    Hamiltonians from its triplets, numpy.linalg.eigh of the (3,3) sector for the ground state
    and of the (4,3) and (2,3) sectors for the T=0 Lehmann sum at 512 frequencies
    (cmpy/exactdiag.py:46-57, 215-245), one host core."""
    from oracle import ed_oracle as O

    n = 6
    bonds = [[i, i + 1] for i in range(n - 1)]
    eps, uu, bnd, width = O.hubbard_descriptor(n, bonds, inter=4.0, hop=1.0, mu=2.0)
    z = np.linspace(-8, 8, 512) + 0.05j

    def dense(nu, nd):
        up, dn = O.sector_states(n, nu), O.sector_states(n, nd)
        return up, dn, O.dense_from_coo(len(up) * len(dn), *O.coo_fermion(up, dn, eps, uu, bnd, width))

    def run():
        up, dn, H = dense(3, 3)
        w, V = np.linalg.eigh(H)
        psi = V[:, 0]
        upp, dnp, Hp = dense(4, 3)
        upm, dnm, Hm = dense(2, 3)
        cd = O.apply_fermion(up, dn, upp, dn, 0, O.UP, True, psi)
        cm = O.apply_fermion(up, dn, upm, dn, 0, O.UP, False, psi)
        return w[0], O.gf_zero_temperature_dense(None, Hp, Hm, cd, cm, w[0], z)

    run()
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        e0, g = run()
    ms = 1e3 * (time.perf_counter() - t0) / reps
    return {"kind": "port", "cores": 1, "ms": round(ms, 3), "gs_energy": float(e0),
            "sample": "full configuration: reference triplets (oracle restatement) -> dense eigh of three sectors "
                      "-> Lehmann sum at 512 frequencies, one host core, mean of 5"}


def run_f64_matvec(steps: int = 20):
    """The FP64 matvec fallback: the 14-site (7,7) ring with t = 0.7 (not a dyadic hop, so the
    sector has no integer matvec), matvec launches timed inside an FP64 Lanczos run."""
    from cmpy_gb300 import engine as E

    bonds = [(i, j, 0.7) for i, j in sorted(ring_bonds(N_SITES))]
    plan = E.Plan.fermion(N_SITES, [-MU] * N_SITES, [U] * N_SITES, bonds, N_UP, N_DN)
    assert plan.fixed_point == 0
    E.lanczos(plan, max_steps=3, want_vector=False)
    r = E.lanczos(plan, max_steps=steps, want_vector=False, profile=True)
    us = 1e3 * r.matvec_ms / max(r.matvecs, 1)
    return {"workload": "hubbard_ring14_sector77_t0.7_fp64", "kernel": "k_hub_matvec_f64", "matvec_us": round(us, 2),
            "gbs": round(16.0 * plan.dim / (us * 1e-6) / 1e9, 1)}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.matvec_only:
        run_matvec_only(args.matvec_only)
        return
    if args.profile_case:
        PROFILE_CASES[args.profile_case]()
        return
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        tdist.init_process_group("nccl")
        dist = tdist
    out = run_ours(args, rank, world, dist)
    if rank == 0:
        if not args.no_cpu_baseline and world == 1:
            out["cpu_baseline"] = cpu_baseline_line()
        else:
            out["cpu_baseline"] = None
        if not args.no_extras and world == 1:
            for key, fn in (("batched_sweep", run_batched_sweep), ("batched_disorder", run_disorder_batch),
                            ("adjoint", run_adjoint), ("heisenberg20", run_heisenberg), ("chain6_gs_lehmann512", run_chain6),
                            ("matvec_f64_t07", run_f64_matvec)):
                try:
                    out[key] = fn()
                except Exception as exc:  # keep the headline line even if an extra fails
                    out[key] = {"error": f"{type(exc).__name__}: {exc}"}
            # the reference's CPU path beside the two small configurations (cpu_baseline leg)
            if not args.no_cpu_baseline:
                for key, fn in (("heisenberg20", cpu_baseline_heisenberg), ("chain6_gs_lehmann512", cpu_baseline_chain6)):
                    if isinstance(out.get(key), dict) and "error" not in out[key]:
                        try:
                            out[key]["cpu_baseline"] = fn()
                        except Exception as exc:
                            out[key]["cpu_baseline"] = {"error": f"{type(exc).__name__}: {exc}"}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
