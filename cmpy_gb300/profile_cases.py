"""Small, self-contained workloads for profiling single kernels (ncu captures want one kernel
on a few GB of device memory, not the whole benchmark step).

    python -m cmpy_gb300.profile_cases gf14        # Green's-function Lanczos of the 14-site ring
    python -m cmpy_gb300.profile_cases adjoint64   # batched adjoint, 64 SIAMs 1+9, forward + backward
    python -m cmpy_gb300.profile_cases sweep10     # batched ground states, all 121 sectors, 10-site ring

gf14: the particle-sector Lanczos of the 14-site Hubbard ring (U=4, mu=2, t=1), sector (8,7),
D = 10,306,296, from a seeded uniform start vector, 12 steps in block fixed point (three
rotating vectors, ~0.5 GB on the device): the update kernel and the integer matvec of the
benchmark step, without its 23.6 GB Krylov store.
adjoint64: the workload of the benchmark's `adjoint` extra (batched part): 64 SIAMs with
1 impurity + 9 bath sites, sector (5,5), 1024 Matsubara frequencies at beta=100, seeded bath
parameters (numpy default_rng(5)), forward and backward once.
sweep10: the benchmark's `batched_sweep` workload (all 121 sectors of the 10-site Hubbard ring,
U=6, mu=3, t=1; 300 steps, tol 1e-12, tested every 10 steps) in one batched launch with a
configuration the tuner picks on GB300 (512 threads, 2 CTAs per SM, clusters of 4 CTAs; its
other frequent pick, 1024 threads, 1 CTA per SM, clusters of 4, times within a few percent),
run twice (the second launch is the one to capture).
"""

from __future__ import annotations

import sys


def gf14(steps: int = 12) -> None:
    import torch

    from . import engine as E
    from .models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(14, True), inter=4.0, mu=2.0, hop=1.0)
    p = m.plan(8, 7)
    g = torch.Generator(device="cuda").manual_seed(3)
    s = torch.rand(p.dim, dtype=torch.float64, device="cuda", generator=g)
    a, b, _ = E.lanczos_coeffs(p, s, max_steps=steps)
    torch.cuda.synchronize()
    print(f"gf14: {a.numel()} steps, alpha_0 = {float(a[0]):.12f}")


def adjoint64(n: int = 64) -> None:
    import numpy as np
    import torch

    from .adjoint import greens_function_ad_batch, siam_parameters

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


def sweep10() -> None:
    import torch

    from .batched import Batch
    from .models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(10, True), inter=6.0, mu=3.0, hop=1.0)
    plans = [m.plan(nu, nd) for nu, nd in m.basis.iter_fillings()]
    b = Batch(plans)
    b.threads, b.ctas_per_sm, b.cluster_size = 512, 2, 4
    for _ in range(2):
        r = b.lanczos(max_steps=300, tol=1e-12, check_every=10)
    torch.cuda.synchronize()
    print(f"sweep10: {len(plans)} sectors, E0 = {float(r.energy.min()):.12f}")


CASES = {"gf14": gf14, "adjoint64": adjoint64, "sweep10": sweep10}

if __name__ == "__main__":
    if len(sys.argv) != 2 or sys.argv[1] not in CASES:
        sys.exit(f"usage: python -m cmpy_gb300.profile_cases {{{','.join(CASES)}}}")
    CASES[sys.argv[1]]()
