"""Ground-state energies of the benchmark sectors from the oracle's restatement of the
reference path: the reference triplets (bit-exact restatement of cmpy/operators.py and
cmpy/models, checked against the reference's own output in test_oracle_golden.py) summed into
a scipy CSR matrix, then scipy.sparse.linalg.eigsh(k=1, which="SA") as in
cmpy/exactdiag.py:37. CPU only; run once where memory allows (the 14-site sector holds
~206 M triplets, about 10 GB while the matrix is assembled):

    python tests/golden/make_e0_pins.py

Writes tests/golden/bench_e0.npz. The GPU tests compare the engine's energies with these
values; the 12-site value is also checked against the one measured by running the reference
itself (-30.920353562419).
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import ed_oracle as O  # noqa: E402


def ring(n):
    return [(i, (i + 1) % n) if i < (i + 1) % n else ((i + 1) % n, i) for i in range(n)]


def hubbard_ring_e0(n, nu, nd, u, mu, t=1.0):
    up, dn = O.sector_states(n, nu), O.sector_states(n, nd)
    eps, uu, bonds, width = O.hubbard_descriptor(n, ring(n), inter=u, hop=t, mu=mu)
    t0 = time.perf_counter()
    r, c, v = O.coo_fermion(up, dn, eps, uu, bonds, width)
    D = len(up) * len(dn)
    H = sp.csr_matrix((v, (r, c)), shape=(D, D))
    del r, c, v
    t1 = time.perf_counter()
    v0 = np.random.default_rng(0).random(D)
    w = sla.eigsh(H, k=1, which="SA", tol=0, v0=v0, return_eigenvectors=False)
    t2 = time.perf_counter()
    print(f"ring{n} ({nu},{nd}) U={u}: D={D} nnz={H.nnz} build {t1 - t0:.1f}s eigsh {t2 - t1:.1f}s E0={w[0]!r}",
          flush=True)
    return float(w[0]), int(H.nnz)


def heisenberg_ring_random_j_e0(n=20, seed=0):
    """Sz=0 sector of the spin-1/2 ring with J_ij = 1 + 0.1 N(0,1) per bond (i, i+1 mod n),
    drawn in bond order from numpy default_rng(seed); jz = J (the reference's normalisation,
    cmpy/models/heisenberg.py:19-40, with per-bond couplings)."""
    rng = np.random.default_rng(seed)
    J = np.zeros((n, n))
    for i in range(n):
        k = (i + 1) % n
        J[i, k] = J[k, i] = 1.0 + 0.1 * rng.standard_normal()
    states = O.sector_states(n, n // 2)
    neighbors = [[(p - 1) % n, (p + 1) % n] for p in range(n)]
    r, c, v = O.coo_heisenberg(states, O.heisenberg_pairs(neighbors, j=J, jz=J))
    D = len(states)
    H = sp.csr_matrix((v, (r, c)), shape=(D, D))
    v0 = np.random.default_rng(1).random(D)
    w = sla.eigsh(H, k=1, which="SA", tol=0, v0=v0, return_eigenvectors=False)
    print(f"heisenberg{n} Sz=0 random J: D={D} nnz={H.nnz} E0={w[0]!r}", flush=True)
    return float(w[0])


def main():
    out = {}
    out["ring12_66_U4_e0"], _ = hubbard_ring_e0(12, 6, 6, 4.0, 2.0)
    assert abs(out["ring12_66_U4_e0"] - (-30.920353562419)) < 1e-11, "12-site value differs from the reference run"
    out["ring10_55_U6_e0"], _ = hubbard_ring_e0(10, 5, 5, 6.0, 3.0)
    out["heis20_sz0_randomJ_e0"] = heisenberg_ring_random_j_e0()
    out["ring14_77_U4_e0"], nnz = hubbard_ring_e0(14, 7, 7, 4.0, 2.0)
    out["ring14_77_nnz"] = nnz
    np.savez(HERE / "bench_e0.npz", **{k: np.asarray(v) for k, v in out.items()})
    print("wrote", HERE / "bench_e0.npz")


if __name__ == "__main__":
    main()
