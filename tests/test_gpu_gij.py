"""GPU parity of the thermal G_ij (the completed lehmann_full.py:19-97) against the dense
oracle, the i = j reduction to the reference's gf_lehmann, and the ij symmetry."""

import numpy as np
import pytest

from oracle import ed_oracle as O

pytestmark = pytest.mark.gpu

DESC4 = O.hubbard_descriptor(4, [[0, 1], [1, 2], [2, 3]], inter=2.0, mu=1.0, hop=1.0)


def _m4():
    from cmpy_gb300.models import ChainLattice, HubbardModel

    return HubbardModel(ChainLattice(4, False), inter=2.0, mu=1.0, hop=1.0)


@pytest.mark.parametrize("ij", [(0, 1), (1, 2), (0, 3)])
def test_gij_vs_oracle(cuda, ij):
    from cmpy_gb300.exactdiag import gf_lehmann_offdiag

    z = np.linspace(-4, 4, 96) + 0.1j
    g = gf_lehmann_offdiag(_m4(), z, 5.0, *ij)
    ref = O.gf_offdiag_dense(4, DESC4, z, 5.0, *ij)
    assert np.max(np.abs(g - ref)) < 1e-10
    g2 = gf_lehmann_offdiag(_m4(), z, 5.0, ij[1], ij[0])
    assert np.max(np.abs(g - g2)) < 1e-12


def test_gii_equals_reference_gf_lehmann(cuda, golden):
    from cmpy_gb300.exactdiag import gf_lehmann_offdiag, greens_lehmann

    e = golden["exactdiag"]
    z = e["chain4_z"]
    for beta in (5.0, 40.0):
        for pos in (0, 2):
            ref = e[f"chain4_U2_b{int(beta)}_p{pos}_gf"]
            assert np.max(np.abs(gf_lehmann_offdiag(_m4(), z, beta, pos, pos) - ref)) < 1e-8
    # the unnormalised sum differs from the normalised one by the partition function only
    g_un = greens_lehmann(_m4(), z, 5.0, 0, 1)
    g_n = gf_lehmann_offdiag(_m4(), z, 5.0, 0, 1)
    ratio = g_un / g_n
    assert np.max(np.abs(ratio - ratio[0])) < 1e-9 * abs(ratio[0])
