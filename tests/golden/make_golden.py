"""Generate golden vectors by running the unmodified reference (cmpy) on small inputs.

Run in a container that has the reference checkout:

    python tests/golden/make_golden.py [--reference /root/reference]

It imports cmpy through oracle.refshim (stubs for numba/matplotlib/colorcet/gftool/lattpy;
numba's JIT off, as in the reference's CI) and writes ``tests/golden/*.npz``. The GPU machine
never runs this script; tests only read the .npz files it produced.
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle.refshim import StubLattice, import_reference  # noqa: E402


def chain(n, periodic):
    lat = StubLattice()
    lat.periodic = periodic
    return lat.build(n)


def triplets(model, sector):
    data, idx = model.hamiltonian_data(sector.up_states, sector.dn_states)
    return np.asarray(idx[0], np.int64), np.asarray(idx[1], np.int64), np.asarray(data, np.float64)


def main(ref_path):
    R = import_reference(ref_path)
    out = {}

    # 1. sector enumeration: Basis.get_states (cmpy/basis.py:668-676), with and without init_sectors
    for N in range(1, 9):
        b = R.basis.Basis(N)
        bi = R.basis.Basis(N, init_sectors=True)
        for n in list(range(N + 1)) + [None]:
            key = f"states_N{N}_n{'all' if n is None else n}"
            out[key] = np.asarray(b.get_states(n), dtype=np.int64)
            alt = np.asarray(bi.get_states(n), dtype=np.int64)
            assert np.array_equal(out[key], alt)
    np.savez_compressed(HERE / "basis.npz", **out)

    # 2. COO triplets + dense H + reference matvec on seeded vectors
    rng = np.random.default_rng(1234)
    coo = {}

    def record(name, model, n_up, n_dn):
        sec = model.get_sector(n_up, n_dn)
        r, c, v = triplets(model, sec)
        coo[f"{name}_rows"], coo[f"{name}_cols"], coo[f"{name}_vals"] = r, c, v
        hop = model.hamilton_operator(sector=sec)
        x = rng.standard_normal(sec.size)
        coo[f"{name}_x"] = x
        coo[f"{name}_y"] = np.asarray(hop._matvec(x), np.float64)  # y[col] += val * x[row]
        if sec.size <= 1200:
            coo[f"{name}_dense"] = model.hamiltonian(sector=sec)

    m2 = R.models.HubbardModel(2, [[0, 1]], inter=2.0, eps=1.0, hop=1.0)
    record("hub2_11", m2, 1, 1)
    c6 = chain(6, False)
    m6 = R.models.HubbardModel(6, c6.neighbor_pairs(True)[0], inter=4.0, mu=2.0, hop=1.0)
    for nu, nd in [(3, 3), (3, 2), (4, 3), (2, 3), (0, 1), (6, 6)]:
        record(f"chain6_U4_{nu}{nd}", m6, nu, nd)
    r5 = chain(5, True)
    eps5 = rng.uniform(-1, 1, 5)
    coo["ring5_eps"] = eps5
    m5 = R.models.HubbardModel(5, r5.neighbor_pairs(True)[0], inter=3.0, eps=eps5, mu=1.5, hop=0.7)
    for nu, nd in [(2, 3), (3, 2), (1, 1), (0, 2), (5, 4)]:
        record(f"ring5_dis_{nu}{nd}", m5, nu, nd)
    eb = np.array([-1.0, 0.5, 1.2, -0.3])
    vv = np.array([0.3, 0.5, 0.2, 0.45])
    coo["siam_eps_bath"], coo["siam_v"] = eb, vv
    ms = R.models.SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=eb, v=vv)
    for nu, nd in [(2, 2), (3, 2), (2, 1), (5, 5)]:
        record(f"siam_{nu}{nd}", ms, nu, nd)

    # Heisenberg: full space (s=None) and Sz sectors of a 6-site ring
    for n, periodic, s_list, jj, jz in [(4, False, [None, 0.0, 1.0], 1.0, None), (6, True, [0.0, 1.0], 1.3, 0.7)]:
        lat = chain(n, periodic)
        mh = R.models.HeisenbergModel(lat, j=jj, jz=jz)
        for s in s_list:
            states = mh.get_states(s)
            data, (rows, cols) = mh.hamiltonian_data(states)
            tag = f"heis{n}{'p' if periodic else 'o'}_s{'all' if s is None else s}"
            coo[f"{tag}_rows"] = np.asarray(rows, np.int64)
            coo[f"{tag}_cols"] = np.asarray(cols, np.int64)
            coo[f"{tag}_vals"] = np.asarray(data, np.float64)
            coo[f"{tag}_states"] = np.asarray(states, np.int64)
            hop = mh.hamilton_operator(s)
            x = rng.standard_normal(len(states))
            coo[f"{tag}_x"] = x
            coo[f"{tag}_y"] = np.asarray(hop._matvec(x), np.float64)
            coo[f"{tag}_dense"] = mh.hamiltonian(s)

    # standalone projectors on odd inputs (zero hop, negative-zero energies, partial lists)
    up = np.asarray(R.basis.Basis(5).get_states(2), np.int64)
    dn = np.asarray(R.basis.Basis(5).get_states(3), np.int64)
    for tag, gen in [
        ("proj_onsite_mixed", R.operators.project_onsite_energy(up, dn, np.array([0.0, -0.0, 1.5, 0.0, -2.25]))),
        ("proj_inter_site", R.operators.project_hubbard_inter(up, dn, np.array([1.0, 0.0, 2.0, 0.0, 3.0]))),
        ("proj_hop_zero", R.operators.project_hopping(up, dn, 5, 1, 4, 0.0)),
        ("proj_hop_w3", R.operators.project_hopping(up, dn, 3, 0, 4, -0.6)),
        ("proj_hop_sub", R.operators.project_hopping(up[:7], dn[2:9], 5, 0, 3, 1.1)),
    ]:
        trip = np.array(list(gen), dtype=object).reshape(-1, 3)
        coo[f"{tag}_rows"] = trip[:, 0].astype(np.int64)
        coo[f"{tag}_cols"] = trip[:, 1].astype(np.int64)
        coo[f"{tag}_vals"] = trip[:, 2].astype(np.float64)
    coo["proj_up"], coo["proj_dn"] = up, dn
    np.savez_compressed(HERE / "coo.npz", **coo)

    # 3. creation / annihilation operators (UP channel; the reference's DN variant raises)
    ops = {}
    b4 = R.basis.Basis(4)
    for (nu, nd) in [(2, 1), (1, 2), (0, 0)]:
        sec = b4.get_sector(nu, nd)
        sp1 = b4.upper_sector(nu, nd, R.basis.UP)
        x = rng.standard_normal(sec.size)
        ops[f"cdag_x_{nu}{nd}"] = x
        for pos in range(4):
            cd = R.operators.CreationOperator(sec, sp1, pos, R.basis.UP)
            ops[f"cdag_{nu}{nd}_p{pos}"] = np.asarray(cd.matvec(x)).real.astype(np.float64)
            an = R.operators.AnnihilationOperator(sp1, sec, pos, R.basis.UP)
            xp = rng.standard_normal(sp1.size)
            ops[f"c_x_{nu}{nd}_p{pos}"] = xp
            ops[f"c_{nu}{nd}_p{pos}"] = np.asarray(an.matvec(xp)).real.astype(np.float64)
    np.savez_compressed(HERE / "fermion_ops.npz", **ops)

    # 4. ground state over all sectors and the thermal Lehmann Green's function
    ed = {}
    gs = R.exactdiag.compute_groundstate(m6)
    ed["chain6_U4_E0"] = np.float64(gs.energy)
    ed["chain6_U4_sector"] = np.array([gs.n_up, gs.n_dn])
    c4 = chain(4, False)
    m4 = R.models.HubbardModel(4, c4.neighbor_pairs(True)[0], inter=2.0, mu=1.0, hop=1.0)
    z = np.linspace(-4, 4, 96) + 0.1j
    for beta in (5.0, 40.0):
        for pos in (0, 2):
            d = R.exactdiag.gf_lehmann(m4, z, beta=beta, pos=pos)
            tag = f"chain4_U2_b{int(beta)}_p{pos}"
            ed[f"{tag}_gf"] = np.asarray(d.gf)
            ed[f"{tag}_occ"] = np.float64(d.occ)
            ed[f"{tag}_occ2"] = np.float64(d.occ_double)
            ed[f"{tag}_e0"] = np.float64(d.gs_energy)
    ed["chain4_z"] = z
    # config-1 style: 6-site open chain, site 0 up, 512 real frequencies, eta=0.05, beta=50
    z6 = np.linspace(-8, 8, 512) + 0.05j
    d6 = R.exactdiag.gf_lehmann(m6, z6, beta=50.0, pos=0)
    ed["chain6_z"] = z6
    ed["chain6_gf_b50"] = np.asarray(d6.gf)
    ed["chain6_occ_b50"] = np.float64(d6.occ)
    ed["chain6_e0_b50"] = np.float64(d6.gs_energy)
    # SIAM impurity Green's function via the model's own entry point (anderson.py:163-164)
    ms2 = R.models.SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=eb[:3], v=vv[:3], temp=0.1)
    zs = np.linspace(-5, 5, 64) + 0.2j
    ed["siam3_z"] = zs
    ed["siam3_gimp"] = np.asarray(ms2.impurity_gf(zs))
    ed["siam3_g0"] = np.asarray(ms2.impurity_gf0(zs))
    ed["siam3_delta"] = np.asarray(ms2.hybridization_func(zs))
    # tridiagonal ground state (exactdiag.py:368-375)
    a = rng.standard_normal(40)
    bb = np.abs(rng.standard_normal(39)) + 0.1
    e_t, v_t = R.exactdiag.lanczos_ground_state(a, bb)
    ed["tri_a"], ed["tri_b"], ed["tri_e"], ed["tri_v"] = a, bb, np.float64(e_t), v_t
    np.savez_compressed(HERE / "exactdiag.npz", **ed)

    # 5. real-time Green's functions (exactdiag.py:248-301, scipy expm_multiply inside); the
    #    ground state the reference used is stored so the engine evaluates the same input
    tv = {}
    for tag, model, t1, num in (("chain4_U2", m4, 20.0, 201), ("chain6_U4", m6, 8.0, 81), ("siam3", ms2, 10.0, 101)):
        gsr = R.exactdiag.compute_groundstate(model)
        times, gg = R.exactdiag.gf_greater(model, gsr, 0.0, t1, num, pos=0)
        _, gl = R.exactdiag.gf_lesser(model, gsr, 0.0, t1, num, pos=0)
        tv[f"{tag}_times"] = np.asarray(times)
        tv[f"{tag}_greater"] = np.asarray(gg)
        tv[f"{tag}_lesser"] = np.asarray(gl)
        tv[f"{tag}_e0"] = np.float64(gsr.energy)
        tv[f"{tag}_state"] = np.asarray(gsr.state, dtype=np.float64)
        tv[f"{tag}_sector"] = np.array([gsr.n_up, gsr.n_dn])
    np.savez_compressed(HERE / "tevo.npz", **tv)

    # 6. the G_ij draft lehmann_full.py:48-97 (a script module beside the package)
    import importlib.util

    spec = importlib.util.spec_from_file_location("lehmann_full", str(Path(ref_path) / "lehmann_full.py"))
    lf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(lf)
    lh = {}
    zl = np.linspace(-4, 4, 64) + 0.1j
    lh["z"] = zl
    for beta in (5.0, np.inf):
        for i, j in ((0, 0), (0, 1), (1, 2)):
            tag = f"chain4_U2_b{'inf' if not np.isfinite(beta) else int(beta)}_{i}{j}"
            lh[tag] = np.asarray(lf.greens_lehmann(m4, zl, beta, i, j))
    np.savez_compressed(HERE / "lehmann_full.npz", **lh)
    for f in sorted(HERE.glob("*.npz")):
        print(f"{f.name}: {f.stat().st_size / 1024:.1f} KiB")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    main(ap.parse_args().reference)
