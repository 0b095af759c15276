"""GPU parity: sector enumeration and COO triplets against the reference's golden vectors
(bit-exact) and the oracle."""

import numpy as np
import pytest
import torch

from oracle import ed_oracle as O
from oracle.refshim import chain_neighbors

pytestmark = pytest.mark.gpu


def test_enumerate_golden(cuda, golden):
    from cmpy_gb300 import engine as E

    for key, ref in golden["basis"].items():
        _, N, n = key.split("_")
        N = int(N[1:])
        n = None if n == "nall" else int(n[1:])
        got = E.enumerate_states(N, n).cpu().numpy()
        assert np.array_equal(got, ref), key


@pytest.mark.parametrize("N", [14, 16, 20, 24])
def test_enumerate_large_properties(cuda, N):
    from cmpy_gb300 import engine as E

    for n in sorted({0, 1, N // 2, N - 1, N}):
        st = E.enumerate_states(N, n)
        from math import comb

        assert st.numel() == comb(N, n)
        if st.numel() > 1:
            assert bool(torch.all(st[1:] > st[:-1]))  # strictly ascending
        pc = torch.zeros_like(st)
        x = st.clone()
        for _ in range(N):
            pc += x & 1
            x >>= 1
        assert bool(torch.all(pc == n))
        assert bool(torch.all(st < (1 << N)))
        r = E.rank_states(st)
        assert torch.equal(r, torch.arange(st.numel(), device=st.device))


def test_basis_dropin(cuda, golden):
    from cmpy_gb300.basis import Basis, SpinBasis

    b = Basis(3)
    assert [format(s, "03b") for s in b.get_states(2)] == ["011", "101", "110"]
    assert list(b.get_states(None)) == list(range(8))
    bi = Basis(6, init_sectors=True)
    assert np.array_equal(bi.get_states(3), golden["basis"]["states_N6_n3"])
    sec = Basis(2).get_sector(1, 1)
    assert sec.state_labels() == ["⇅.", "↑↓", "↓↑", ".⇅"]
    assert Basis(2).get_sector(n_up=1).state_labels() == ["↑.", "⇅.", "↑↓", "⇅↓", ".↑", "↓↑", ".⇅", "↓⇅"]
    sb = SpinBasis(6)
    assert np.array_equal(np.asarray(sb.get_states(0.0)), O.sector_states(6, 3))
    with pytest.raises(ValueError):
        SpinBasis(5).get_states(0.0)


def _bitexact(got, ref):
    g = np.asarray(got)
    return g.shape == ref.shape and np.array_equal(g.view(np.int64) if g.dtype == np.float64 else g,
                                                   ref.view(np.int64) if ref.dtype == np.float64 else ref)


def _models(golden):
    from cmpy_gb300.models import ChainLattice, HubbardModel, SingleImpurityAndersonModel

    g = golden["coo"]
    return {
        "hub2": (HubbardModel(2, [[0, 1]], inter=2.0, eps=1.0, hop=1.0), [(1, 1)]),
        "chain6_U4": (HubbardModel(ChainLattice(6), inter=4.0, mu=2.0, hop=1.0),
                      [(3, 3), (3, 2), (4, 3), (2, 3), (0, 1), (6, 6)]),
        "ring5_dis": (HubbardModel(ChainLattice(5, True), inter=3.0, eps=g["ring5_eps"], mu=1.5, hop=0.7),
                      [(2, 3), (3, 2), (1, 1), (0, 2), (5, 4)]),
        "siam": (SingleImpurityAndersonModel(u=4.0, eps_imp=0.0, eps_bath=g["siam_eps_bath"], v=g["siam_v"]),
                 [(2, 2), (3, 2), (2, 1), (5, 5)]),
    }


def test_model_coo_bit_exact(cuda, golden):
    g = golden["coo"]
    for name, (model, sectors) in _models(golden).items():
        for nu, nd in sectors:
            tag = "hub2_11" if name == "hub2" else f"{name}_{nu}{nd}"
            sec = model.get_sector(nu, nd)
            vals, idx = model.hamiltonian_data(sec.up_states, sec.dn_states)
            assert _bitexact(idx[0], g[f"{tag}_rows"]), tag
            assert _bitexact(idx[1], g[f"{tag}_cols"]), tag
            assert _bitexact(vals, g[f"{tag}_vals"]), tag
            # the plan's whole-model generator gives the same triplets
            r, c, v = (a.cpu().numpy() for a in model.plan(nu, nd).coo())
            assert _bitexact(r, g[f"{tag}_rows"]) and _bitexact(c, g[f"{tag}_cols"]) and _bitexact(v, g[f"{tag}_vals"])
            if f"{tag}_dense" in g:
                assert np.array_equal(model.hamiltonian(nu, nd), g[f"{tag}_dense"]), tag


def test_projector_generators_bit_exact(cuda, golden):
    from cmpy_gb300 import operators as ops

    g = golden["coo"]
    up, dn = g["proj_up"], g["proj_dn"]
    cases = {
        "proj_onsite_mixed": ops.project_onsite_energy(up, dn, np.array([0.0, -0.0, 1.5, 0.0, -2.25])),
        "proj_inter_site": ops.project_hubbard_inter(up, dn, np.array([1.0, 0.0, 2.0, 0.0, 3.0])),
        "proj_hop_zero": ops.project_hopping(up, dn, 5, 1, 4, 0.0),
        "proj_hop_w3": ops.project_hopping(up, dn, 3, 0, 4, -0.6),
        "proj_hop_sub": ops.project_hopping(up[:7], dn[2:9], 5, 0, 3, 1.1),
    }
    for tag, gen in cases.items():
        trip = list(gen)
        r = np.array([t[0] for t in trip], dtype=np.int64)
        c = np.array([t[1] for t in trip], dtype=np.int64)
        v = np.array([t[2] for t in trip], dtype=np.float64)
        assert _bitexact(r, g[f"{tag}_rows"]), tag
        assert _bitexact(c, g[f"{tag}_cols"]), tag
        assert _bitexact(v, g[f"{tag}_vals"]), tag
    with pytest.raises(AssertionError):
        list(ops.project_hopping(up, dn, 5, 3, 1, 1.0))


@pytest.mark.parametrize("tag,n,periodic,j,jz,s", [
    ("heis4o_sall", 4, False, 1.0, None, None),
    ("heis4o_s0.0", 4, False, 1.0, None, 0.0),
    ("heis6p_s0.0", 6, True, 1.3, 0.7, 0.0),
    ("heis6p_s1.0", 6, True, 1.3, 0.7, 1.0),
])
def test_heisenberg_coo_and_dense(cuda, golden, tag, n, periodic, j, jz, s):
    from cmpy_gb300.models import ChainLattice, HeisenbergModel

    g = golden["coo"]
    m = HeisenbergModel(ChainLattice(n, periodic), j=j, jz=jz)
    r, c, v = (a.cpu().numpy() for a in m.plan(s).coo())
    assert _bitexact(r, g[f"{tag}_rows"]) and _bitexact(c, g[f"{tag}_cols"]) and _bitexact(v, g[f"{tag}_vals"])
    np.testing.assert_allclose(m.hamiltonian(s), g[f"{tag}_dense"], rtol=0, atol=1e-15)
    y = m.hamilton_operator(s).matvec(g[f"{tag}_x"])
    np.testing.assert_allclose(y, g[f"{tag}_y"], rtol=1e-14, atol=1e-14)


def test_coo_ring12_triplet_count(cuda):
    """12-site ring (6,6): the whole-model generator emits the reference's triplet count
    (13,737,108, counted by running the reference) and indexes inside the sector."""
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(12, True), inter=4.0, mu=2.0, hop=1.0)
    p = m.plan(6, 6)
    r, c, v = p.coo()
    # 13,737,108 triplets for the 12-site ring (6,6) (reference probe count)
    assert r.numel() == 13737108
    # row/col ranges and symmetry of the summed matrix diagonal count
    assert int(r.min()) == 0 and int(r.max()) == p.dim - 1 and int(c.max()) == p.dim - 1
