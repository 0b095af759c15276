"""The allocation-free tridiagonal solver, called through the C ABI.

ed_tridiag_lowest_noalloc exists for callers that cannot allocate device memory where they
need the ground state of a Lanczos tridiagonal matrix (for example while a stream is being
captured into a CUDA graph, or when their device memory belongs to their own allocator). Its
scratch is a static array in the library, so it must give the same answer as the allocating
ed_tridiag_lowest, on consecutive calls that reuse that array.

This file is collected last on purpose: it must pass alone in a fresh process and after every
other test.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tridiagonal tolerance used by the other tests


def _call(fn, a, b, want_vec):
    m = a.numel()
    val = torch.empty(1, dtype=torch.float64, device="cuda")
    vec = torch.empty(m, dtype=torch.float64, device="cuda") if want_vec else None
    st = fn(a.data_ptr(), b.data_ptr(), m, val.data_ptr(), vec.data_ptr() if want_vec else None,
            torch.cuda.current_stream().cuda_stream)
    return st, val, vec


@pytest.mark.parametrize("m", [1, 7, 40, 300, 4096])
def test_noalloc_matches_allocating_twice(cuda, m):
    from cmpy_gb300 import _native as N

    L = N.lib()
    rng = np.random.default_rng(m)
    a = torch.as_tensor(rng.standard_normal(m)).cuda()
    b = torch.as_tensor(np.concatenate([[0.0], np.abs(rng.standard_normal(m - 1)) + 0.1])).cuda()
    st, v_ref, x_ref = _call(L.ed_tridiag_lowest, a, b, True)
    assert st == 0
    for _ in range(2):  # two calls in a row share the static scratch
        st, v, x = _call(L.ed_tridiag_lowest_noalloc, a, b, True)
        assert st == 0, L.ed_last_error().decode()
        torch.cuda.synchronize()
        assert abs(v.item() - v_ref.item()) <= TOL * max(1.0, abs(v_ref.item()))
        torch.testing.assert_close(x, x_ref, rtol=0, atol=TOL)
    # value-only calls skip the eigenvector
    st, v, _ = _call(L.ed_tridiag_lowest_noalloc, a, b, False)
    assert st == 0 and abs(v.item() - v_ref.item()) <= TOL * max(1.0, abs(v_ref.item()))


def test_noalloc_rejects_oversized(cuda):
    from cmpy_gb300 import _native as N

    L = N.lib()
    a = torch.zeros(4097, dtype=torch.float64, device="cuda")
    st, _, _ = _call(L.ed_tridiag_lowest_noalloc, a, a, True)
    assert st == N.ED_ERR_TOO_LARGE
    assert "4096" in L.ed_last_error().decode()
