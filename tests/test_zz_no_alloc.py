"""The allocation-free tridiagonal solver, called through the C ABI.

ed_tridiag_lowest_noalloc exists for callers that cannot allocate device memory where they
need the ground state of a Lanczos tridiagonal matrix (their device memory belongs to their
own allocator, or their host forbids library allocations). Its scratch is a static array in
the library, so it must give the same answer as the allocating ed_tridiag_lowest and as an
independent solver (scipy's eigh_tridiagonal), on consecutive calls that reuse that array —
including a large call followed by smaller ones with different data, so that stale scratch
from an earlier call would show.

This file is collected last on purpose; the last test re-runs the checks in a fresh Python
process, so the file passes both alone and after every other test.
"""

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tridiagonal tolerance used by the other tests
ROOT = Path(__file__).resolve().parent.parent


def _call(fn, a, b, want_vec):
    m = a.numel()
    val = torch.empty(1, dtype=torch.float64, device="cuda")
    vec = torch.empty(m, dtype=torch.float64, device="cuda") if want_vec else None
    st = fn(a.data_ptr(), b.data_ptr(), m, val.data_ptr(), vec.data_ptr() if want_vec else None,
            torch.cuda.current_stream().cuda_stream)
    return st, val, vec


def _problem(m, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(m)
    b = np.concatenate([[0.0], np.abs(rng.standard_normal(m - 1)) + 0.1])
    return a, b


def _scipy_lowest(a, b):
    w, v = sla.eigh_tridiagonal(a, b[1:], select="i", select_range=(0, 0))
    return float(w[0]), v[:, 0]


def _check(L, m, seed):
    """noalloc vs scipy and vs the allocating solver, twice in a row."""
    a_h, b_h = _problem(m, seed)
    a, b = torch.as_tensor(a_h).cuda(), torch.as_tensor(b_h).cuda()
    e_sp, v_sp = _scipy_lowest(a_h, b_h)
    st, v_ref, x_ref = _call(L.ed_tridiag_lowest, a, b, True)
    assert st == 0
    for _ in range(2):  # two calls in a row share the static scratch
        st, v, x = _call(L.ed_tridiag_lowest_noalloc, a, b, True)
        assert st == 0, L.ed_last_error().decode()
        torch.cuda.synchronize()
        assert abs(v.item() - v_ref.item()) <= TOL * max(1.0, abs(v_ref.item()))
        torch.testing.assert_close(x, x_ref, rtol=0, atol=TOL)
        assert abs(v.item() - e_sp) <= TOL * max(1.0, abs(e_sp))
        xh = x.cpu().numpy()
        assert abs(abs(float(xh @ v_sp)) - 1.0) <= 1e-10  # same eigenvector up to its sign
    # value-only calls skip the eigenvector
    st, v, _ = _call(L.ed_tridiag_lowest_noalloc, a, b, False)
    assert st == 0 and abs(v.item() - v_ref.item()) <= TOL * max(1.0, abs(v_ref.item()))


@pytest.mark.parametrize("m", [1, 7, 40, 300, 4096])
def test_noalloc_matches_allocating_and_scipy(cuda, m):
    from cmpy_gb300 import _native as N

    _check(N.lib(), m, m)


def test_noalloc_large_then_smaller_calls(cuda):
    """The static scratch is used for m > 512; a 4096 call followed by 1000 and 513 with
    fresh data must not read anything the earlier call left behind."""
    from cmpy_gb300 import _native as N

    L = N.lib()
    for m, seed in ((4096, 1), (1000, 2), (513, 3), (4096, 4), (600, 5)):
        _check(L, m, seed)


def test_noalloc_rejects_oversized(cuda):
    from cmpy_gb300 import _native as N

    L = N.lib()
    a = torch.zeros(4097, dtype=torch.float64, device="cuda")
    st, _, _ = _call(L.ed_tridiag_lowest_noalloc, a, a, True)
    # the same status as the allocating solver for the same limit
    assert st == N.ED_ERR_INVALID_ARG
    assert "4096" in L.ed_last_error().decode()
    st2, _, _ = _call(L.ed_tridiag_lowest, a, a, True)
    assert st2 == st


_FRESH = """
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import torch
from cmpy_gb300 import _native as N
import test_zz_no_alloc as T
L = N.lib()
for m, seed in ((4096, 7), (513, 8)):
    T._check(L, m, seed)
print("fresh-process no-alloc ok")
"""


def test_noalloc_in_fresh_process(cuda):
    """The first call of a process does the address set-up: run the checks in a new
    interpreter where nothing else has touched the library."""
    code = _FRESH.format(root=str(ROOT), tests=str(ROOT / "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh-process no-alloc ok" in r.stdout


def test_noalloc_in_cuda_graph(cuda):
    """After a warm-up call, a call captured into a CUDA graph replays correctly with its
    inputs changed in place between replays (the graph keeps the scratch address it was
    captured with)."""
    from cmpy_gb300 import _native as N

    L = N.lib()
    m = 1000  # above the shared-memory size: the kernel works in the static array
    a_h, b_h = _problem(m, 11)
    a, b = torch.as_tensor(a_h).cuda(), torch.as_tensor(b_h).cuda()
    val = torch.empty(1, dtype=torch.float64, device="cuda")
    vec = torch.empty(m, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        st = L.ed_tridiag_lowest_noalloc(a.data_ptr(), b.data_ptr(), m, val.data_ptr(), vec.data_ptr(),
                                         s.cuda_stream)
        assert st == 0, L.ed_last_error().decode()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    status = []
    with torch.cuda.graph(g):
        cs = torch.cuda.current_stream().cuda_stream
        status.append(L.ed_tridiag_lowest_noalloc(a.data_ptr(), b.data_ptr(), m, val.data_ptr(), vec.data_ptr(), cs))
    assert status == [0], L.ed_last_error().decode()
    for seed in (12, 13):
        a2, b2 = _problem(m, seed)
        a.copy_(torch.as_tensor(a2))
        b.copy_(torch.as_tensor(b2))
        g.replay()
        torch.cuda.synchronize()
        st, v_ref, x_ref = _call(L.ed_tridiag_lowest, a, b, True)
        assert st == 0
        torch.cuda.synchronize()
        assert abs(val.item() - v_ref.item()) <= TOL * max(1.0, abs(v_ref.item()))
        torch.testing.assert_close(vec, x_ref, rtol=0, atol=TOL)
        e_sp, _ = _scipy_lowest(a2, b2)
        assert abs(val.item() - e_sp) <= TOL * max(1.0, abs(e_sp))
