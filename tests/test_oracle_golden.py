"""The oracle (numpy restatement) against golden vectors from the unmodified reference.

This pins the oracle before any GPU result is compared with it: triplets and the
reference triplet matvec must match bit for bit, dense-eigh quantities to round-off.
"""

import numpy as np
import pytest

from oracle import ed_oracle as O
from oracle.refshim import chain_neighbors


def test_sector_states(golden):
    g = golden["basis"]
    for key, ref in g.items():
        _, N, n = key.split("_")
        N = int(N[1:])
        n = None if n == "nall" else int(n[1:])
        assert np.array_equal(O.sector_states(N, n), ref), key


def test_colex_rank_is_position():
    for N in range(1, 11):
        for n in range(N + 1):
            st = O.sector_states(N, n)
            assert np.array_equal(O.colex_rank(st), np.arange(len(st)))


def _hub(nsites, nbrs, **kw):
    return O.hubbard_descriptor(nsites, nbrs, **kw)


def _models(golden):
    g = golden["coo"]
    c6 = [[i, i + 1] for i in range(5)]
    r5 = sorted({tuple(sorted((i, (i + 1) % 5))) for i in range(5)})
    return {
        "hub2": _hub(2, [[0, 1]], inter=2.0, eps=1.0, hop=1.0),
        "chain6_U4": _hub(6, c6, inter=4.0, mu=2.0, hop=1.0),
        "ring5_dis": _hub(5, [list(p) for p in r5], inter=3.0, eps=g["ring5_eps"], mu=1.5, hop=0.7),
        "siam": O.siam_descriptor(4.0, 0.0, g["siam_eps_bath"], g["siam_v"]),
    }


SECTORS = {
    "hub2": [(1, 1)],
    "chain6_U4": [(3, 3), (3, 2), (4, 3), (2, 3), (0, 1), (6, 6)],
    "ring5_dis": [(2, 3), (3, 2), (1, 1), (0, 2), (5, 4)],
    "siam": [(2, 2), (3, 2), (2, 1), (5, 5)],
}
NSITES = {"hub2": 2, "chain6_U4": 6, "ring5_dis": 5, "siam": 5}


def _cases():
    for name, secs in SECTORS.items():
        for s in secs:
            yield name, s


@pytest.mark.parametrize("name,sector", list(_cases()))
def test_coo_fermion_bit_exact(golden, name, sector):
    g = golden["coo"]
    eps, u, bonds, width = _models(golden)[name]
    N = NSITES[name]
    up, dn = O.sector_states(N, sector[0]), O.sector_states(N, sector[1])
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    tag = f"{name}_{sector[0]}{sector[1]}" if name != "hub2" else "hub2_11"
    assert np.array_equal(r, g[f"{tag}_rows"])
    assert np.array_equal(c, g[f"{tag}_cols"])
    assert np.array_equal(v.view(np.int64), g[f"{tag}_vals"].view(np.int64))
    D = len(up) * len(dn)
    y = O.triplet_matvec(D, r, c, v, g[f"{tag}_x"])
    assert np.array_equal(y.view(np.int64), g[f"{tag}_y"].view(np.int64))
    if f"{tag}_dense" in g:
        assert np.array_equal(O.dense_from_coo(D, r, c, v), g[f"{tag}_dense"])


def test_projectors_odd_inputs(golden):
    g = golden["coo"]
    up, dn = g["proj_up"], g["proj_dn"]
    cases = {
        "proj_onsite_mixed": O.coo_onsite(up, dn, np.array([0.0, -0.0, 1.5, 0.0, -2.25])),
        "proj_inter_site": O.coo_inter(up, dn, np.array([1.0, 0.0, 2.0, 0.0, 3.0])),
        "proj_hop_zero": O.coo_hopping(up, dn, 5, 1, 4, 0.0),
        "proj_hop_w3": O.coo_hopping(up, dn, 3, 0, 4, -0.6),
        "proj_hop_sub": O.coo_hopping(up[:7], dn[2:9], 5, 0, 3, 1.1),
    }
    for tag, (r, c, v) in cases.items():
        assert np.array_equal(r, g[f"{tag}_rows"]), tag
        assert np.array_equal(c, g[f"{tag}_cols"]), tag
        assert np.array_equal(v.view(np.int64), g[f"{tag}_vals"].view(np.int64)), tag


@pytest.mark.parametrize("tag,n,periodic,j,jz,s", [
    ("heis4o_sall", 4, False, 1.0, None, None),
    ("heis4o_s0.0", 4, False, 1.0, None, 0.0),
    ("heis4o_s1.0", 4, False, 1.0, None, 1.0),
    ("heis6p_s0.0", 6, True, 1.3, 0.7, 0.0),
    ("heis6p_s1.0", 6, True, 1.3, 0.7, 1.0),
])
def test_coo_heisenberg_bit_exact(golden, tag, n, periodic, j, jz, s):
    g = golden["coo"]
    states = g[f"{tag}_states"]
    pairs = O.heisenberg_pairs(chain_neighbors(n, periodic), j, jz)
    r, c, v = O.coo_heisenberg(states, pairs)
    assert np.array_equal(r, g[f"{tag}_rows"])
    assert np.array_equal(c, g[f"{tag}_cols"])
    assert np.array_equal(v.view(np.int64), g[f"{tag}_vals"].view(np.int64))
    y = O.triplet_matvec(len(states), r, c, v, g[f"{tag}_x"])
    assert np.array_equal(y.view(np.int64), g[f"{tag}_y"].view(np.int64))
    assert np.array_equal(O.dense_from_coo(len(states), r, c, v), g[f"{tag}_dense"])


def test_fermion_ops_up(golden):
    g = golden["fermion_ops"]
    for nu, nd in [(2, 1), (1, 2), (0, 0)]:
        up, dn = O.sector_states(4, nu), O.sector_states(4, nd)
        up_p = O.sector_states(4, nu + 1)
        x = g[f"cdag_x_{nu}{nd}"]
        for pos in range(4):
            y = O.apply_fermion(up, dn, up_p, dn, pos, O.UP, True, x)
            assert np.array_equal(y, g[f"cdag_{nu}{nd}_p{pos}"])
            xp = g[f"c_x_{nu}{nd}_p{pos}"]
            y2 = O.apply_fermion(up_p, dn, up, dn, pos, O.UP, False, xp)
            assert np.array_equal(y2, g[f"c_{nu}{nd}_p{pos}"])


def _chain_dense(N, nbrs, **kw):
    eps, u, bonds, width = O.hubbard_descriptor(N, nbrs, **kw)

    def dense(nu, nd):
        up, dn = O.sector_states(N, nu), O.sector_states(N, nd)
        r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
        return O.dense_from_coo(len(up) * len(dn), r, c, v)

    return dense


@pytest.mark.parametrize("beta", [5, 40])
@pytest.mark.parametrize("pos", [0, 2])
def test_gf_lehmann_thermal(golden, beta, pos):
    g = golden["exactdiag"]
    dense = _chain_dense(4, [[0, 1], [1, 2], [2, 3]], inter=2.0, mu=1.0, hop=1.0)
    gf, occ, occ2, e0 = O.gf_lehmann_thermal(dense, lambda n: O.sector_states(4, n), 4, g["chain4_z"], float(beta),
                                             pos=pos)
    tag = f"chain4_U2_b{beta}_p{pos}"
    np.testing.assert_allclose(gf, g[f"{tag}_gf"], rtol=1e-11, atol=1e-12)
    assert abs(occ - g[f"{tag}_occ"]) < 1e-12
    assert abs(occ2 - g[f"{tag}_occ2"]) < 1e-12
    assert abs(e0 - g[f"{tag}_e0"]) < 1e-12


def test_ground_state_chain6(golden):
    g = golden["exactdiag"]
    dense = _chain_dense(6, [[i, i + 1] for i in range(5)], inter=4.0, mu=2.0, hop=1.0)
    nu, nd = g["chain6_U4_sector"]
    e0, _ = O.ground_state_dense(dense(int(nu), int(nd)))
    assert abs(e0 - g["chain6_U4_E0"]) <= 1e-12 * abs(e0)


def test_tridiag_lowest(golden):
    g = golden["exactdiag"]
    b = np.concatenate([[0.0], g["tri_b"]])
    assert abs(O.tridiag_lowest(g["tri_a"], b) - g["tri_e"]) < 1e-12


def test_cf_matches_dense_small():
    """Continued fraction of full-reorth Lanczos coefficients equals the dense resolvent."""
    rng = np.random.default_rng(0)
    A = rng.standard_normal((30, 30))
    H = A + A.T
    v = rng.standard_normal(30)
    a, b, nrm = O.lanczos_tridiag_dense(H, v, 30)
    z = np.linspace(-5, 5, 17) + 0.3j
    t = z - a[-1]
    for l in range(len(a) - 2, -1, -1):
        t = z - a[l] - b[l + 1] ** 2 / t
    cf = nrm**2 / t
    w, V = np.linalg.eigh(H)
    amp = (V.T @ v) ** 2
    exact = np.sum(amp[None, :] / (z[:, None] - w[None, :]), axis=1)
    np.testing.assert_allclose(cf, exact, rtol=1e-10, atol=1e-12)
