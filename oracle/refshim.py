"""Import the unmodified reference package ``cmpy`` from a source checkout.

Test infrastructure only (used by tests/golden/make_golden.py). The reference imports
numba, matplotlib, colorcet, gftool and lattpy, none of which is installed here. This module
installs stand-ins into ``sys.modules`` before importing it:

* numba: ``njit`` returns the Python function unchanged and ``prange`` is ``range`` — the
  reference then runs interpreted, exactly like its own CI with NUMBA_DISABLE_JIT=1;
* matplotlib / colorcet: empty placeholders (plotting only);
* gftool: ``fourier.tt2z`` raises (only the time-evolution path uses it);
* lattpy: a ``Lattice`` base class plus chain/hypercubic helpers with ``num_sites``,
  ``neighbors(pos)`` and ``neighbor_pairs(unique)`` for open/periodic chains.

It also restores two names that newer numpy/scipy removed (``np.infty`` and
``scipy.sparse.linalg.interface.IdentityOperator``).
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

DEFAULT_REFERENCE = Path("/root/reference")


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything()


class _Anything:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()


def _njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


class StubLattice:
    """Chain lattice with the lattpy calls the reference makes."""

    def __init__(self, dim: int = 1):
        self.dim = dim
        self.num_sites = 0
        self.periodic = False
        self._nbrs: list[list[int]] = []

    def build(self, num_sites, primitive=True, periodic=None):
        n = int(np.prod(num_sites))
        self.num_sites = n
        if periodic is not None:
            self.periodic = bool(periodic)
        self._nbrs = chain_neighbors(n, self.periodic)
        return self

    def neighbors(self, pos):
        return np.asarray(self._nbrs[int(pos)], dtype=np.int64)

    def neighbor_pairs(self, unique=False):
        pairs = [[i, j] for i in range(self.num_sites) for j in self._nbrs[i] if (not unique or i < j)]
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        return pairs, np.zeros(len(pairs), dtype=np.int64)


def chain_neighbors(n: int, periodic: bool) -> list[list[int]]:
    out = []
    for i in range(n):
        nb = set()
        if i - 1 >= 0:
            nb.add(i - 1)
        elif periodic and n > 2:
            nb.add(n - 1)
        if i + 1 < n:
            nb.add(i + 1)
        elif periodic and n > 2:
            nb.add(0)
        if periodic and n == 2:
            nb.add(1 - i)
        nb.discard(i)
        out.append(sorted(nb))
    return out


def _install_stubs():
    numba = types.ModuleType("numba")
    numba.njit = _njit
    numba.jit = _njit
    numba.prange = range
    numba.int64 = _Anything()
    sys.modules.setdefault("numba", numba)

    mpl = _Stub("matplotlib")
    mpl.__path__ = []
    colors = _Stub("matplotlib.colors")

    class Normalize:
        def __init__(self, vmin=None, vmax=None, clip=False):
            self.vmin, self.vmax, self.clip = vmin, vmax, clip

    colors.Normalize = Normalize
    pyplot = _Stub("matplotlib.pyplot")
    mpl.colors = colors
    mpl.pyplot = pyplot
    for name, mod in (("matplotlib", mpl), ("matplotlib.colors", colors), ("matplotlib.pyplot", pyplot)):
        sys.modules.setdefault(name, mod)
    sys.modules.setdefault("colorcet", _Stub("colorcet"))

    gft = types.ModuleType("gftool")
    fourier = types.ModuleType("gftool.fourier")

    def tt2z(*a, **k):
        raise NotImplementedError("gftool is not installed")

    fourier.tt2z = tt2z
    gft.fourier = fourier
    sys.modules.setdefault("gftool", gft)
    sys.modules.setdefault("gftool.fourier", fourier)

    lp = types.ModuleType("lattpy")

    class Lattice(StubLattice):
        pass

    def simple_chain(a=1.0, neighbors=1):
        return Lattice(1)

    def finite_hypercubic(shape, a=1.0, periodic=False, neighbors=1):
        latt = Lattice(1)
        latt.periodic = bool(periodic)
        return latt.build(shape)

    lp.Lattice = Lattice
    lp.simple_chain = simple_chain
    lp.finite_hypercubic = finite_hypercubic
    sys.modules.setdefault("lattpy", lp)

    if not hasattr(np, "infty"):
        np.infty = np.inf
    import scipy.sparse.linalg as sla

    iface = getattr(sla, "interface", None)
    if iface is not None and not hasattr(iface, "IdentityOperator"):
        from scipy.sparse.linalg import _interface

        iface.IdentityOperator = _interface.IdentityOperator


def import_reference(path: Path | str = DEFAULT_REFERENCE):
    """Return the reference modules (cmpy, basis, operators, models, exactdiag)."""
    path = Path(path)
    if not (path / "cmpy" / "__init__.py").exists():
        raise FileNotFoundError(f"no cmpy checkout at {path}")
    _install_stubs()
    # the checkout is read-only input: never write bytecode caches next to its sources
    sys.dont_write_bytecode = True
    if str(path) not in sys.path:
        sys.path.insert(0, str(path))
    import cmpy  # noqa: F401
    from cmpy import basis, exactdiag, models, operators

    return types.SimpleNamespace(cmpy=cmpy, basis=basis, operators=operators, models=models, exactdiag=exactdiag,
                                 StubLattice=StubLattice)
