"""cmpy_gb300 — exact diagonalisation on NVIDIA GB300 (sm_103a).

A GPU engine for cmpy's hot path: Fock-sector bases, Hubbard / Anderson / Heisenberg
Hamiltonians, the Lanczos ground state and the Green's function. The module layout mirrors
cmpy (``basis``, ``operators``, ``models``, ``exactdiag``) so code written against cmpy can
switch by changing the import. All computation runs in libcmpy_ed.so (hand-written CUDA);
``engine`` exposes the device-level objects.
"""

from .basis import (  # noqa: F401
    DN,
    SPIN_CHARS,
    UP,
    Basis,
    Sector,
    SpinBasis,
    SpinState,
    State,
    annihilate,
    binarr,
    binidx,
    binstr,
    create,
    occupations,
    overlap,
    state_label,
)

__version__ = "0.1.0"


def __getattr__(name):
    # GPU-facing modules load lazily so that host-only helpers import without CUDA
    import importlib

    if name in ("operators", "models", "exactdiag", "engine", "batched", "adjoint"):
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
