"""libcmpy_ed.so loads and exports every entry point include/cmpy_ed.h declares.

CPU-only: calls only the host functions (no kernel launches)."""

import re
from math import comb
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "cmpy_ed.h").read_text()
    return sorted(set(re.findall(r"ED_API\s+[\w\s\*]*?\b(ed_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from cmpy_gb300 import build, _native

    build.build()
    return _native.lib()


def test_every_header_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from cmpy_gb300 import _native

    assert sorted(_native.exported_symbols()) == header_functions()


def test_host_functions(lib):
    for n in range(0, 40):
        for k in range(0, n + 1):
            assert lib.ed_binomial(n, k) == comb(n, k)
    assert lib.ed_binomial(5, 7) == 0
    assert lib.ed_sector_size(14, 7) == 3432
    assert lib.ed_sector_size(20, 10) == 184756
    assert lib.ed_sector_size(6, -1) == 64
    assert lib.ed_sector_size(6, 7) == 0
    assert lib.ed_version() >= 100
    for st in range(9):
        assert lib.ed_status_string(st).decode() != "unknown status"
    assert lib.ed_status_string(99).decode() == "unknown status"
