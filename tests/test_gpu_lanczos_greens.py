"""GPU parity: Lanczos ground states against dense eigh and the reference, Green's functions
(thermal Lehmann, T=0 Lehmann, continued fraction) against the reference and the oracle.

Tolerances follow the engine's targets: ground-state energy 1e-10 relative, G(z) 1e-8 absolute.
"""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-8


def _hub_chain(N, periodic=False, **kw):
    from cmpy_gb300.models import ChainLattice, HubbardModel

    return HubbardModel(ChainLattice(N, periodic), **kw)


def _oracle_dense(model, nu, nd):
    eps, u, bonds, width = model.fermion_descriptor()
    N = model.num_sites
    up, dn = O.sector_states(N, nu), O.sector_states(N, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    return O.dense_from_coo(len(up) * len(dn), r, c, v)


def test_compute_groundstate_chain6(cuda, golden):
    from cmpy_gb300.exactdiag import compute_groundstate

    g = golden["exactdiag"]
    m = _hub_chain(6, inter=4.0, mu=2.0, hop=1.0)
    gs = compute_groundstate(m)
    assert (gs.n_up, gs.n_dn) == tuple(g["chain6_U4_sector"])
    assert abs(gs.energy - g["chain6_U4_E0"]) <= E_TOL * abs(g["chain6_U4_E0"])
    H = _oracle_dense(m, gs.n_up, gs.n_dn)
    r = H @ gs.state - gs.energy * gs.state
    assert np.linalg.norm(r) < 1e-9 * abs(gs.energy) and abs(np.linalg.norm(gs.state) - 1) < 1e-12


@pytest.mark.parametrize("reorth", [False, True])
@pytest.mark.parametrize("case", ["chain8_44", "ring8_43", "siam8_44", "ring10_55"])
def test_lanczos_vs_dense(cuda, case, reorth):
    from cmpy_gb300 import engine as E
    from cmpy_gb300.models import SingleImpurityAndersonModel

    if case == "chain8_44":
        m, (nu, nd) = _hub_chain(8, inter=4.0, mu=2.0), (4, 4)
    elif case == "ring8_43":
        m, (nu, nd) = _hub_chain(8, True, inter=6.0, mu=3.0, hop=-1.0), (4, 3)
    elif case == "ring10_55":
        m, (nu, nd) = _hub_chain(10, True, inter=6.0, mu=3.0), (5, 5)
    else:
        rng = np.random.default_rng(3)
        m = SingleImpurityAndersonModel(u=4.0, eps_bath=rng.uniform(-2, 2, 7), v=rng.uniform(0.1, 0.6, 7))
        nu, nd = 4, 4
    p = m.plan(nu, nd)
    res = E.lanczos(p, max_steps=min(300, p.dim), reorth=reorth, want_vector=True, tol=1e-12, check_every=10)
    if case == "ring10_55":
        ref = -34.254559411302544  # reference compute_groundstate, 10-site ring U=6 (probe value)
    else:
        ref = np.linalg.eigvalsh(_oracle_dense(m, nu, nd))[0]
    assert abs(res.energy - ref) <= E_TOL * abs(ref), (res.energy, ref)
    v = res.vector
    hv = p.matvec(v)
    assert torch.linalg.norm(hv - res.energy * v).item() < 1e-9 * abs(res.energy)
    assert abs(torch.linalg.norm(v).item() - 1) < 1e-12


def test_lanczos_small_and_breakdown(cuda):
    """Sectors smaller than the Krylov length stop at an invariant subspace exactly."""
    from cmpy_gb300 import engine as E

    m = _hub_chain(4, inter=2.0, mu=1.0)
    for nu, nd in [(0, 0), (1, 0), (1, 1), (2, 1), (4, 4)]:
        p = m.plan(nu, nd)
        res = E.lanczos(p, max_steps=50, want_vector=True)
        ref = np.linalg.eigvalsh(_oracle_dense(m, nu, nd))[0]
        assert res.steps <= p.dim
        assert abs(res.energy - ref) <= 1e-12 * max(1.0, abs(ref)), (nu, nd)


def test_lanczos_errors(cuda):
    from cmpy_gb300 import _native as N
    from cmpy_gb300 import engine as E

    m = _hub_chain(6, inter=4.0, mu=2.0)
    p = m.plan(3, 3)
    with pytest.raises(N.EDError) as ei:
        E.lanczos(p, max_steps=20, v0=torch.zeros(p.dim, dtype=torch.float64, device="cuda"))
    assert ei.value.status == N.ED_ERR_ZERO_VECTOR
    bad = torch.ones(p.dim, dtype=torch.float64, device="cuda")
    bad[3] = float("nan")
    with pytest.raises(N.EDError) as ei:
        E.lanczos(p, max_steps=20, v0=bad)
    assert ei.value.status == N.ED_ERR_NONFINITE
    with pytest.raises(ValueError):
        E.Plan.fermion(4, [0.0] * 4, [0.0] * 4, [(2, 1, 1.0)], 2, 2)
    with pytest.raises(N.EDError):
        E.Plan.fermion(4, [float("nan")] * 4, [0.0] * 4, [(0, 1, 1.0)], 2, 2)
    with pytest.raises(ValueError):
        E.Plan.fermion(4, [0.0] * 4, [0.0] * 4, [(0, 1, 1.0)], 5, 2)


def test_tridiag_golden(cuda, golden):
    from cmpy_gb300.exactdiag import lanczos_ground_state

    g = golden["exactdiag"]
    e, v = lanczos_ground_state(g["tri_a"], g["tri_b"])
    assert abs(e - g["tri_e"]) < 1e-12
    ref = g["tri_v"] * np.sign(g["tri_v"][np.argmax(np.abs(g["tri_v"]))])
    got = v * np.sign(v[np.argmax(np.abs(v))])
    np.testing.assert_allclose(got, ref, atol=1e-10)


@pytest.mark.parametrize("beta", [5, 40])
@pytest.mark.parametrize("pos", [0, 2])
def test_gf_lehmann_golden(cuda, golden, beta, pos):
    from cmpy_gb300.exactdiag import gf_lehmann

    g = golden["exactdiag"]
    m = _hub_chain(4, inter=2.0, mu=1.0, hop=1.0)
    d = gf_lehmann(m, g["chain4_z"], beta=float(beta), pos=pos)
    tag = f"chain4_U2_b{beta}_p{pos}"
    assert np.max(np.abs(d.gf - g[f"{tag}_gf"])) < G_TOL
    assert abs(d.occ - g[f"{tag}_occ"]) < 1e-10
    assert abs(d.occ_double - g[f"{tag}_occ2"]) < 1e-10
    assert abs(d.gs_energy - g[f"{tag}_e0"]) < 1e-10


def test_gf_lehmann_chain6_config(cuda, golden):
    from cmpy_gb300.exactdiag import gf_lehmann

    g = golden["exactdiag"]
    m = _hub_chain(6, inter=4.0, mu=2.0, hop=1.0)
    d = gf_lehmann(m, g["chain6_z"], beta=50.0, pos=0)
    assert np.max(np.abs(d.gf - g["chain6_gf_b50"])) < G_TOL
    assert abs(d.occ - g["chain6_occ_b50"]) < 1e-10


def test_siam_impurity_gf(cuda, golden):
    from cmpy_gb300.models import SingleImpurityAndersonModel

    g = golden["exactdiag"]
    eb = golden["coo"]["siam_eps_bath"][:3]
    vv = golden["coo"]["siam_v"][:3]
    m = SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=eb, v=vv, temp=0.1)
    assert np.max(np.abs(m.impurity_gf(g["siam3_z"]) - g["siam3_gimp"])) < G_TOL
    np.testing.assert_allclose(m.impurity_gf0(g["siam3_z"]), g["siam3_g0"], rtol=1e-14)
    zt = torch.as_tensor(g["siam3_z"]).cuda()
    np.testing.assert_allclose(m.hybridization_func(zt).cpu().numpy(), g["siam3_delta"], rtol=1e-13)


@pytest.mark.parametrize("case", ["chain6", "ring8"])
def test_gf_continued_fraction_vs_dense(cuda, case):
    """T=0 G(w+i eta) and G(i w_n) from the device CF agree with the dense-eigh Lehmann oracle.

    On the real axis (eta = 0.05) the fraction converges to 1e-8 once the levels resolve the
    poles that carry weight: 200 levels for the 6-site chain, ~1000 for the 8-site ring (1285
    weighted poles); Matsubara frequencies converge within 100 levels."""
    from cmpy_gb300.exactdiag import gf_continued_fraction, gf_lehmann_zero_temperature, groundstate_sector

    if case == "chain6":
        m, (nu, nd), n_lev = _hub_chain(6, inter=4.0, mu=2.0), (3, 3), 200
    else:
        m, (nu, nd), n_lev = _hub_chain(8, True, inter=4.0, mu=2.0), (4, 4), 1000
    e0, psi = groundstate_sector(m, nu, nd, max_steps=400, tol=1e-13)
    w = np.linspace(-8, 8, 512)
    beta = 50.0
    iwn = 1j * (2 * np.arange(256) + 1) * np.pi / beta
    z = np.concatenate([w + 0.05j, iwn])
    g_cf = gf_continued_fraction(m, z, nu, nd, e0, psi, pos=0, n_lev=n_lev)
    g_leh = gf_lehmann_zero_temperature(m, z, e0, psi, nu, nd, pos=0)
    # dense oracle
    N = m.num_sites
    psi_h = psi.cpu().numpy()
    up, dn = O.sector_states(N, nu), O.sector_states(N, nd)
    upp, upm = O.sector_states(N, nu + 1), O.sector_states(N, nu - 1)
    cd = O.apply_fermion(up, dn, upp, dn, 0, O.UP, True, psi_h)
    cm = O.apply_fermion(up, dn, upm, dn, 0, O.UP, False, psi_h)
    ref = O.gf_zero_temperature_dense(None, _oracle_dense(m, nu + 1, nd), _oracle_dense(m, nu - 1, nd), cd, cm, e0, z)
    assert np.max(np.abs(g_leh - ref)) < G_TOL
    assert np.max(np.abs(g_cf - ref)) < G_TOL
    # Matsubara axis converges with far fewer levels
    g_m = gf_continued_fraction(m, iwn, nu, nd, e0, psi, pos=0, n_lev=100)
    assert np.max(np.abs(g_m - ref[len(w):])) < G_TOL
    # sum rule: -Im G integrates to pi * <{c, c^dag}> = pi for large |w| behaviour 1/z
    zl = np.array([1e4j])
    assert abs(gf_continued_fraction(m, zl, nu, nd, e0, psi, n_lev=n_lev)[0] * zl[0] - 1.0) < 1e-6
