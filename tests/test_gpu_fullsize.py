"""Parity at the benchmark's full size (14-site Hubbard ring, t=1, U=4, mu=2, sector (7,7),
D = 11,778,624) through properties that do not depend on a dense oracle:

* the integer matvec is exactly symmetric: <x, H y> == <H x, y> in int64 arithmetic;
* every matvec variant (table in global memory, resident table, bulk-copied row pairs, the
  two-pass panel form, the banded two-pass sweep) gives the same integers;
* the ground-state energies of the benchmark sectors equal the oracle's reference triplets
  summed into a scipy CSR matrix and solved with eigsh (tests/golden/make_e0_pins.py) to 1e-10
  relative: 14-site ring (7,7), 12-site ring (6,6) (also the value measured on the reference
  itself), 10-site ring U=6 (5,5), Heisenberg ring N=20 with random couplings;
* the fixed-point Lanczos and the FP64 Lanczos (independent arithmetic) agree on E0 to 1e-10
  relative, and the Ritz vector has a small residual;
* the Green's function of site 0 obeys the sum rule (particle + hole weights = 1), is purely
  imaginary on the Matsubara axis (particle-hole symmetry of the half-filled ring) and has the
  1/(i w) tail.
"""

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _ring14():
    from cmpy_gb300.models import ChainLattice, HubbardModel

    return HubbardModel(ChainLattice(14, True), inter=4.0, mu=2.0, hop=1.0)


def test_integer_matvec_exactly_symmetric(cuda):
    m = _ring14()
    p = m.plan(7, 7)
    assert p.fixed_point > 0
    gen = torch.Generator(device="cuda").manual_seed(11)
    # small integers: H x stays below 2^20 and <x, H y> below 2^52, exact in int64
    x = torch.randint(-1024, 1025, (p.dim,), dtype=torch.int64, device="cuda", generator=gen)
    y = torch.randint(-1024, 1025, (p.dim,), dtype=torch.int64, device="cuda", generator=gen)
    hx, ew = p.matvec_fixed(x, 0)
    hy, _ = p.matvec_fixed(y, 0)
    assert ew == 0  # t, U and mu are integers here: W = H x exactly
    assert torch.sum(x * hy).item() == torch.sum(hx * y).item()
    # and it is the FP64 operator
    ref = p.matvec(x.to(torch.float64))
    assert torch.equal(hx.to(torch.float64), ref)


_VARIANT_SCRIPT = r"""
import json, sys, torch
sys.path.insert(0, sys.argv[1])
from cmpy_gb300.models import ChainLattice, HubbardModel
m = HubbardModel(ChainLattice(14, True), inter=4.0, mu=2.0, hop=1.0)
p = m.plan(7, 7)
gen = torch.Generator(device="cuda").manual_seed(5)
x = torch.randint(-2**40, 2**40, (p.dim,), dtype=torch.int64, device="cuda", generator=gen)
w, _ = p.matvec_fixed(x, 0)
print(json.dumps({"sum": int(torch.sum(w).item()), "sq": float(torch.sum((w.to(torch.float64) / 2**40) ** 2).item()),
                  "head": [int(v) for v in w[:8].tolist()], "tail": [int(v) for v in w[-8:].tolist()]}))
"""


def test_matvec_variants_identical(cuda):
    """Each variant in its own process (the variant is chosen once per process)."""
    outs = {}
    for v in ("1", "2", "3", "4", "5", "6", "7"):
        env = dict(os.environ, CMPY_ED_MATVEC=v)
        r = subprocess.run([sys.executable, "-c", _VARIANT_SCRIPT, str(ROOT)], env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs[v] = json.loads(r.stdout.strip().splitlines()[-1])
    for v in ("2", "3", "4", "5", "6", "7"):
        assert outs[v] == outs["1"], v


def test_groundstate_fixed_vs_f64(cuda):
    from cmpy_gb300 import engine as E

    p = _ring14().plan(7, 7)
    rf = E.lanczos(p, max_steps=250, want_vector=True, tol=1e-12, check_every=10, arithmetic="fixed")
    rd = E.lanczos(p, max_steps=250, want_vector=False, tol=1e-12, check_every=10, arithmetic="f64")
    assert abs(rf.energy - rd.energy) <= 1e-10 * abs(rd.energy)
    psi = rf.vector
    assert abs(torch.linalg.norm(psi).item() - 1.0) < 1e-12
    res = torch.linalg.norm(p.matvec(psi) - rf.energy * psi).item()
    assert res < 1e-6 * abs(rf.energy)


def test_greens_function_sum_rule_and_symmetry(cuda):
    from cmpy_gb300.exactdiag import gf_continued_fraction, groundstate_sector

    m = _ring14()
    e0, psi = groundstate_sector(m, 7, 7, max_steps=250, tol=1e-12)
    beta = 10.0
    iwn = 1j * (2 * np.arange(256) + 1) * np.pi / beta
    g, coeffs = gf_continued_fraction(m, iwn, 7, 7, e0, psi, pos=0, n_lev=200, return_coeffs=True)
    n_p = coeffs["particle"][2] ** 2
    n_h = coeffs["hole"][2] ** 2
    assert abs(n_p + n_h - 1.0) < 1e-10  # <c c^dag> + <c^dag c> = 1
    assert abs(n_p - 0.5) < 1e-8  # half filling: <n_0,up> = 1/2
    assert np.max(np.abs(g.real)) < 1e-6 * np.max(np.abs(g))  # particle-hole symmetry
    assert abs(iwn[-1] * g[-1] - 1.0) < 1e-3  # 1/(i w) tail
    assert np.all(g.imag < 0)


def test_benchmark_energies_vs_oracle_eigsh(cuda, golden):
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import ChainLattice, HeisenbergModel, HubbardModel

    pins = golden["bench_e0"]
    r14 = E.lanczos(_ring14().plan(7, 7), max_steps=250, want_vector=False)
    assert abs(r14.energy - float(pins["ring14_77_U4_e0"])) <= 1e-10 * abs(float(pins["ring14_77_U4_e0"]))
    r12 = E.lanczos(HubbardModel(ChainLattice(12, True), inter=4.0, mu=2.0).plan(6, 6), max_steps=250,
                    want_vector=False, tol=1e-12, check_every=10)
    assert abs(r12.energy - float(pins["ring12_66_U4_e0"])) <= 1e-10 * 30.92
    assert abs(float(pins["ring12_66_U4_e0"]) - (-30.920353562419)) < 1e-11  # reference run
    r10 = E.lanczos(HubbardModel(ChainLattice(10, True), inter=6.0, mu=3.0).plan(5, 5), max_steps=250,
                    want_vector=False, tol=1e-12, check_every=10)
    assert abs(r10.energy - float(pins["ring10_55_U6_e0"])) <= 1e-10 * 34.25
    n = 20
    rng = np.random.default_rng(0)
    J = np.zeros((n, n))
    for i in range(n):
        k = (i + 1) % n
        J[i, k] = J[k, i] = 1.0 + 0.1 * rng.standard_normal()
    ph = HeisenbergModel(ChainLattice(n, True), j=J, jz=J).plan(0)
    rh = E.lanczos(ph, max_steps=300, reorth=True, want_vector=False, tol=0.0)
    e_h = float(pins["heis20_sz0_randomJ_e0"])
    assert abs(rh.energy - e_h) <= 1e-10 * abs(e_h)
