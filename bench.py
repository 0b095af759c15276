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
    return ap.parse_args()


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
        a, b, nrm = E.lanczos_coeffs(plan_p, phi, max_steps=GF_LEVELS)
        E.continued_fraction(a, b, nrm * nrm, zt, e0=r.energy, sign=1, out=g)
        chi = plan.apply_fermion(plan_m, 0, 1, False, r.vector)
        a2, b2, nrm2 = E.lanczos_coeffs(plan_m, chi, max_steps=GF_LEVELS)
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
        a, b, nrm = E.lanczos_coeffs(plan_p, phi, max_steps=GF_LEVELS)
        E.continued_fraction(a, b, nrm * nrm, zd, e0=r.energy, sign=1, out=g)
        chi = plan.apply_fermion(plan_m, 0, 1, False, r.vector)
        a2, b2, nrm2 = E.lanczos_coeffs(plan_m, chi, max_steps=GF_LEVELS)
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
        "dtype": "f64",
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
            "kernel": "matvec (16*D bytes per launch)",
            "peak_source": f"{peak_kind} (hbm_gbs, burst copy)",
            "matvec_us": round(mv_ms / mv_n * 1e3, 2) if mv_n else None,
        },
        "e2e": {"value": round(e2e_value, 3), "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    return out


def matvec_traffic():
    """DRAM bytes per matvec launch from the committed ncu summary (profiles/), if any."""
    f = ROOT / "profiles" / "matvec_hubbard14.md"
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


def cpu_matvec_rate(csr, x, threads: int, seconds: float):
    """H*v GB/s of the sample with `threads` row blocks in parallel (scipy releases the GIL in
    its sparse kernels)."""
    from concurrent.futures import ThreadPoolExecutor

    n = csr.shape[0]
    cuts = np.linspace(0, n, threads + 1).astype(int)
    blocks = [csr[cuts[i]:cuts[i + 1]] for i in range(threads)]
    ex = ThreadPoolExecutor(max_workers=threads)

    def one():
        list(ex.map(lambda b: b @ x, blocks))

    one()
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        one()
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    ex.shutdown()
    return 16.0 * n / dt / 1e9, dt


def cpu_baseline_line(seconds: float = 8.0):
    threads = os.cpu_count() or 1
    up_rows = 96
    csr, x, build = cpu_sample(up_rows)
    gbs, dt = cpu_matvec_rate(csr, x, threads, seconds)
    return {
        "value": round(gbs, 4),
        "unit": "GB/s",
        "cores": threads,
        "kind": "port",
        "sample": (f"reference COO (oracle restatement) of the first {up_rows} of 3432 up-rows of the 14-site (7,7) "
                   f"sector -> scipy CSR ({csr.nnz} nnz) -> H*v over {threads} threads; COO+CSR build {build:.2f} s "
                   f"for the sample ({build * 3432 / up_rows:.0f} s extrapolated to the sector)"),
    }


def run_reference(args, rank, world):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    up_rows = 96
    csr, x, build = cpu_sample(up_rows)
    from concurrent.futures import ThreadPoolExecutor

    n = csr.shape[0]
    cuts = np.linspace(0, n, threads + 1).astype(int)
    blocks = [csr[cuts[i]:cuts[i + 1]] for i in range(threads)]
    ex = ThreadPoolExecutor(max_workers=threads)
    reps_per_step = 20

    def step():
        for _ in range(reps_per_step):
            list(ex.map(lambda b: b @ x, blocks))

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    ex.shutdown()
    gbs = 16.0 * n * reps_per_step * args.steps / el / 1e9
    D = 3432 * 3432
    mv_s = el / (reps_per_step * args.steps) * (D / n)
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
        "data": "synthetic",
        "config": {"workload": "hubbard_ring14_half_filling_gs250_cf200", "n_sites": N_SITES, "sector": [N_UP, N_DN],
                   "dim": D, "parallelism": "host threads"},
        "gs_time_s_extrapolated": round(250 * mv_s + build * 3432 / up_rows, 1),
        "cpu_baseline": {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{up_rows} of 3432 up-rows, {reps_per_step} H*v per step, scipy CSR over "
                                   f"{threads} threads"},
        "e2e": {"value": round(gbs, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
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
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
