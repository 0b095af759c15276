"""G_ij (lehmann_full.py:19-97): the oracle against the reference.

The reference's draft greens_lehmann is restated as written (its sector loop variable
shadows the site argument and the c^dag_j factor is commented out) and reproduces the
reference's output bit for bit; the completed G_ij oracle reduces to the reference's thermal
gf_lehmann for i = j."""

import numpy as np
import pytest

from oracle import ed_oracle as O

DESC4 = O.hubbard_descriptor(4, [[0, 1], [1, 2], [2, 3]], inter=2.0, mu=1.0, hop=1.0)


@pytest.mark.parametrize("beta", [5.0, np.inf])
@pytest.mark.parametrize("ij", [(0, 0), (0, 1), (1, 2)])
def test_draft_restatement_matches_reference(golden, beta, ij):
    d = golden["lehmann_full"]
    tag = f"chain4_U2_b{'inf' if not np.isfinite(beta) else int(beta)}_{ij[0]}{ij[1]}"
    g = O.greens_lehmann_draft(4, DESC4, d["z"], beta, *ij)
    assert np.array_equal(g, d[tag])


@pytest.mark.parametrize("beta", [5.0, 40.0])
@pytest.mark.parametrize("pos", [0, 2])
def test_gii_equals_reference_gf_lehmann(golden, beta, pos):
    e = golden["exactdiag"]
    z = e["chain4_z"]
    g = O.gf_offdiag_dense(4, DESC4, z, beta, pos, pos)
    assert np.max(np.abs(g - e[f"chain4_U2_b{int(beta)}_p{pos}_gf"])) < 1e-12


def test_gij_symmetric():
    z = np.linspace(-3, 3, 17) + 0.2j
    a = O.gf_offdiag_dense(4, DESC4, z, 7.0, 0, 2)
    b = O.gf_offdiag_dense(4, DESC4, z, 7.0, 2, 0)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14)
