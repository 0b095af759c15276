"""Host-side logic of the drop-in API that needs no GPU (mirrors cmpy/tests/test_basis.py
and the model parameter handling)."""

import numpy as np
import pytest

from cmpy_gb300 import basis

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

settings.register_profile("cmpy_gb300", deadline=None)
settings.load_profile("cmpy_gb300")


@given(st.integers(0, 2**15))
def test_binstr(num):
    assert basis.binstr(num) == f"{num:b}"
    for width in [0, 5, 10, 15, 20]:
        assert basis.binstr(num, width) == f"{num:0{width}b}"


@given(st.integers(0, 2**15))
def test_binarr_binidx(num):
    for width in [None, 0, 5, 20]:
        ref = np.fromiter(f"{num:0{width or 0}b}"[::-1], dtype=np.int64)
        assert np.array_equal(basis.binarr(num, width), ref)
        assert basis.binidx(num, width) == list(np.where(ref)[0])


@given(st.integers(0, 2**15), st.integers(0, 2**15))
def test_overlap(a, b):
    ref = np.fromiter(f"{a & b:b}"[::-1], dtype=np.int64)
    assert np.array_equal(basis.overlap(a, b), ref)


@pytest.mark.parametrize("num,pos,res", [(0b0, 0, 0b1), (0b1, 0, None), (0b100, 0, 0b101), (0b100, 1, 0b110),
                                         (0b100, 2, None), (0b110, 0, 0b111), (0b110, 1, None)])
def test_create(num, pos, res):
    assert basis.create(num, pos) == res


@pytest.mark.parametrize("num,pos,res", [(0b0, 0, None), (0b1, 0, 0b0), (0b100, 2, 0b000), (0b110, 1, 0b100),
                                         (0b110, 2, 0b010), (0b110, 0, None)])
def test_annihilate(num, pos, res):
    assert basis.annihilate(num, pos) == res


@pytest.mark.parametrize("n_up", range(15))
@pytest.mark.parametrize("n_dn", range(15))
def test_upper_lower_sector(n_up, n_dn):
    N = 15
    assert basis.upper_sector(n_up, n_dn, basis.UP, N) == (None if n_up == N else (n_up + 1, n_dn))
    assert basis.upper_sector(n_up, n_dn, basis.DN, N) == (None if n_dn == N else (n_up, n_dn + 1))
    assert basis.lower_sector(n_up, n_dn, basis.UP) == (None if n_up == 0 else (n_up - 1, n_dn))
    assert basis.lower_sector(n_up, n_dn, basis.DN) == (None if n_dn == 0 else (n_up, n_dn - 1))


def test_state_labels():
    assert basis.state_label(1, 1) == "⇅"
    assert basis.state_label(1, 2) == "↑↓"
    assert basis.state_label(0, 0, 3) == "..."
    assert basis.State(3, 1, 2).label() == "⇅↑"


def test_basis_init_sizes():
    for n in range(0, 10):
        b = basis.Basis(n)
        assert b.num_spinstates == 2**n and b.size == 4**n and b.fillings == list(range(n + 1))


def test_model_parameters_and_descriptors():
    from cmpy_gb300.models import ChainLattice, HubbardModel, SingleImpurityAndersonModel

    latt = ChainLattice(6, periodic=True)
    m = HubbardModel(latt, inter=4.0, mu=2.0, hop=1.0)
    assert m.inter == 4.0 and m["mu"] == 2.0
    m.inter = 3.0
    assert m.params["inter"] == 3.0
    eps, u, bonds, width = m.fermion_descriptor()
    assert np.all(eps == -2.0) and np.all(u == 3.0) and width == 6
    assert bonds == [(0, 1, 1.0), (0, 5, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 4, 1.0), (4, 5, 1.0)]
    s = SingleImpurityAndersonModel(u=4.0, eps_bath=[-1.0, 1.0], v=[0.2, 0.3])
    eps, u, bonds, width = s.fermion_descriptor()
    assert list(eps) == [-2.0, -1.0, 1.0] and list(u) == [4.0, 0.0, 0.0] and width == 0
    assert bonds == [(0, 1, 0.2), (0, 2, 0.3)]
    z = np.array([0.5j, 1 + 0.1j])
    ref = np.sum(np.array([0.2, 0.3]) ** 2 / (z[:, None] - np.array([-1.0, 1.0])), axis=-1)
    np.testing.assert_allclose(s.hybridization_func(z), ref)
    with pytest.raises(ValueError):
        s.update_bath_energy([1.0])


def test_chain_lattice():
    from cmpy_gb300.models import ChainLattice

    assert ChainLattice(4).neighbors(0) == [1]
    assert ChainLattice(4, True).neighbors(0) == [1, 3]
    pairs, _ = ChainLattice(4, True).neighbor_pairs(True)
    assert pairs.tolist() == [[0, 1], [0, 3], [1, 2], [2, 3]]


def test_apply_fermion_batch_checks_lengths_before_any_device_work():
    """Mismatched plan / target / offset lists are rejected on the host."""
    from cmpy_gb300 import engine as E

    with pytest.raises(ValueError):
        E.apply_fermion_batch([object(), object()], [object()], 0, 1, True, None, [0, 1])
    with pytest.raises(ValueError):
        E.apply_fermion_batch([object()], [object()], 0, 1, True, None, [0, 1])


def test_model_plans_keeps_empty_slots():
    """plans() maps a None sector to None (no plan is built for it)."""
    from cmpy_gb300.models import ChainLattice, HubbardModel

    m = HubbardModel(ChainLattice(4, False), inter=2.0, mu=1.0)
    assert m.plans([None, None]) == [None, None]
