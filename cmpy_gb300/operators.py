"""Linear operators on Fock sectors — drop-in for ``cmpy.operators`` (cmpy/operators.py).

* ``project_onsite_energy`` / ``project_hubbard_inter`` / ``project_hopping`` keep the
  reference generator signatures (cmpy/operators.py:306,360,464) and yield the same
  (row, col, value) triplets in the same order; the triplets are produced on the GPU by the
  ``ed_coo_*`` kernels. ``*_arrays`` variants return the device arrays directly.
* ``HamiltonOperator`` is a scipy ``LinearOperator`` (cmpy/operators.py:614-646). Built from
  a model it is matrix-free (``ed_matvec``); built from triplets, like the reference
  constructor, it applies them with a device CSR kernel that reproduces the reference loop
  ``y[col] += val * x[row]`` bit for bit.
* ``CreationOperator`` / ``AnnihilationOperator`` (cmpy/operators.py:706-791) apply c^dag / c
  on the GPU. ``jw_sign=False`` keeps the reference's convention (no Jordan-Wigner sign);
  the spin-down variants use the target sector's stride, which fixes the reference's
  IndexError (cmpy/operators.py:666-703 index the target with the source num_dn).
"""

from __future__ import annotations

import abc
from typing import Iterator, Tuple

import numpy as np
import scipy.sparse.linalg as sla
import torch

from . import engine as E
from .basis import SPIN_CHARS, UP

__all__ = [
    "LinearOperator",
    "HamiltonOperator",
    "CreationOperator",
    "AnnihilationOperator",
    "project_up",
    "project_dn",
    "project_elements_up",
    "project_elements_dn",
    "project_hubbard_inter",
    "project_onsite_energy",
    "project_hopping",
    "project_hubbard_inter_arrays",
    "project_onsite_energy_arrays",
    "project_hopping_arrays",
]


def project_up(up_idx, num_dn_states, dn_indices):
    """Many-body indices of an up state over the given dn indices (cmpy/operators.py:33-60)."""
    return np.atleast_1d(up_idx * num_dn_states + np.asarray(dn_indices))


def project_dn(dn_idx, num_dn_states, up_indices):
    """Many-body indices of a dn state over the given up indices (cmpy/operators.py:63-90)."""
    return np.atleast_1d(np.asarray(up_indices) * num_dn_states + dn_idx)


def project_elements_up(up_idx, num_dn_states, dn_indices, value, target=None):
    origins = np.atleast_1d(up_idx * num_dn_states + np.asarray(dn_indices))
    targets = origins if target is None else np.atleast_1d(target * num_dn_states + np.asarray(dn_indices))
    for row, col in zip(origins, targets):
        yield row, col, value


def project_elements_dn(dn_idx, num_dn_states, up_indices, value, target=None):
    origins = np.atleast_1d(np.asarray(up_indices) * num_dn_states + dn_idx)
    targets = origins if target is None else np.atleast_1d(np.asarray(up_indices) * num_dn_states + target)
    for row, col in zip(origins, targets):
        yield row, col, value


# -- projectors (GPU) ----------------------------------------------------------------------


def project_onsite_energy_arrays(up_states, dn_states, eps):
    """Device (rows, cols, vals) of project_onsite_energy (cmpy/operators.py:359-422)."""
    return E.coo_onsite(up_states, dn_states, eps)


def project_hubbard_inter_arrays(up_states, dn_states, u):
    """Device (rows, cols, vals) of project_hubbard_inter (cmpy/operators.py:305-356)."""
    return E.coo_inter(up_states, dn_states, u)


def project_hopping_arrays(up_states, dn_states, num_sites, site1, site2, hop):
    """Device (rows, cols, vals) of project_hopping (cmpy/operators.py:463-527)."""
    if not site1 < site2:
        raise AssertionError("site1 must be smaller than site2")
    return E.coo_hopping(up_states, dn_states, num_sites, site1, site2, hop)


def _yield(arrays) -> Iterator[Tuple[int, int, float]]:
    rows, cols, vals = (a.cpu().numpy() for a in arrays)
    yield from zip(rows.tolist(), cols.tolist(), vals.tolist())


def project_onsite_energy(up_states, dn_states, eps):
    yield from _yield(project_onsite_energy_arrays(up_states, dn_states, eps))


def project_hubbard_inter(up_states, dn_states, u):
    yield from _yield(project_hubbard_inter_arrays(up_states, dn_states, u))


def project_hopping(up_states, dn_states, num_sites, site1, site2, hop):
    yield from _yield(project_hopping_arrays(up_states, dn_states, num_sites, site1, site2, hop))


# -- linear operators ----------------------------------------------------------------------


class LinearOperator(sla.LinearOperator, abc.ABC):
    """scipy LinearOperator with ``toarray`` and ``trace`` (cmpy/operators.py:535-608)."""

    def __init__(self, shape, dtype=None):
        sla.LinearOperator.__init__(self, shape=shape, dtype=dtype)

    def __repr__(self):
        return f"{self.__class__.__name__}(shape: {self.shape}, dtype: {self.dtype})"

    def toarray(self) -> np.ndarray:
        return self.matmat(np.eye(self.shape[1], dtype=self.dtype))

    # torch tensors (on the GPU) pass straight to the device implementation; everything
    # else goes through scipy's checks like in the reference
    def matvec(self, x):
        if isinstance(x, torch.Tensor):
            return self._matvec(x)
        return super().matvec(x)

    def matmat(self, X):
        if isinstance(X, torch.Tensor):
            return self._matmat(X)
        return super().matmat(X)

    def _trace(self) -> float:
        return float(np.trace(self.toarray()))

    def trace(self) -> float:
        return self._trace()

    def __mul__(self, x):
        scaled = super().__mul__(x)
        try:
            scaled.trace = lambda: x * self.trace()
            scaled.toarray = lambda: x * self.toarray()
        except AttributeError:
            pass
        return scaled

    def __rmul__(self, x):
        scaled = super().__rmul__(x)
        try:
            scaled.trace = lambda: x * self.trace()
            scaled.toarray = lambda: x * self.toarray()
        except AttributeError:
            pass
        return scaled


def _apply_real(fn, x):
    """Apply a real linear map on the device to a numpy/torch vector or (D, k) matrix;
    numpy in -> numpy out, torch in -> torch (CUDA) out. Complex inputs are split."""
    is_np = not isinstance(x, torch.Tensor)
    t = torch.as_tensor(np.asarray(x)) if is_np else x
    if t.is_complex():
        re = fn(t.real.to(device=E.device(), dtype=torch.float64))
        im = fn(t.imag.to(device=E.device(), dtype=torch.float64))
        out = torch.complex(re, im)
    else:
        out = fn(t.to(device=E.device(), dtype=torch.float64))
    if is_np:
        out = out.cpu().numpy()
        if np.iscomplexobj(x):
            out = out.astype(np.result_type(np.asarray(x).dtype, np.complex128), copy=False)
    return out


class HamiltonOperator(LinearOperator):
    """Hamiltonian as a LinearOperator, applied on the GPU.

    ``HamiltonOperator(size, data, indices, dtype)`` keeps the reference constructor
    (cmpy/operators.py:617-624): ``indices`` is (2, nnz) rows/cols. ``from_plan`` builds
    the matrix-free operator of a model sector.
    """

    def __init__(self, size, data=None, indices=None, dtype=None, plan: "E.Plan" = None):
        if plan is None:
            data = np.asanyarray(data, dtype=np.float64)
            indices = np.asanyarray(indices, dtype=np.int64).reshape(2, -1)
            if dtype is None:
                dtype = data.dtype
        super().__init__((size, size), dtype=dtype if dtype is not None else np.float64)
        self.plan = plan
        self.data = data
        self.indices = None if indices is None else indices.T
        self._csr = None

    @classmethod
    def from_plan(cls, plan: "E.Plan", dtype=None) -> "HamiltonOperator":
        return cls(plan.dim, dtype=dtype, plan=plan)

    # device CSR of H^T, triplets kept in their original order within each row
    def _device_csr(self):
        if self._csr is None:
            dev = E.device()
            rows = torch.as_tensor(self.indices[:, 0].copy()).to(dev)
            cols = torch.as_tensor(self.indices[:, 1].copy()).to(dev)
            vals = torch.as_tensor(np.asarray(self.data, dtype=np.float64)).to(dev)
            cols_sorted, perm = torch.sort(cols, stable=True)
            counts = torch.bincount(cols_sorted, minlength=self.shape[0])
            rowptr = torch.zeros(self.shape[0] + 1, dtype=torch.int64, device=dev)
            rowptr[1:] = torch.cumsum(counts, 0)
            self._csr = (rowptr, rows[perm].contiguous(), vals[perm].contiguous())
        return self._csr

    def _apply_dev(self, x: torch.Tensor) -> torch.Tensor:
        if self.plan is not None:
            return self.plan.matvec(x) if x.ndim == 1 else self.plan.matmat(x)
        rowptr, cols, vals = self._device_csr()
        if x.ndim == 1:
            return E.csr_matvec(rowptr, cols, vals, x.contiguous())
        return torch.stack([E.csr_matvec(rowptr, cols, vals, x[:, k].contiguous()) for k in range(x.shape[1])], 1)

    def _matvec(self, x):
        shape = getattr(x, "shape", None)
        flat = x.reshape(-1) if shape is not None and len(shape) == 2 and shape[1] == 1 else x
        y = _apply_real(self._apply_dev, flat)
        return y.reshape(shape) if shape is not None and len(shape) == 2 else y

    def _matmat(self, X):
        return _apply_real(self._apply_dev, X)

    def toarray(self) -> np.ndarray:
        if self.plan is not None and self.plan.dim <= 32768:
            return self.plan.dense().cpu().numpy().astype(self.dtype, copy=False)
        dev = E.device()
        n = self.shape[0]
        flat = torch.zeros(n * n, dtype=torch.float64, device=dev)
        idx = torch.as_tensor(self.indices[:, 0] * n + self.indices[:, 1]).to(dev)
        flat.index_add_(0, idx, torch.as_tensor(np.asarray(self.data, dtype=np.float64)).to(dev))
        return flat.reshape(n, n).cpu().numpy().astype(self.dtype, copy=False)

    def _adjoint(self) -> "HamiltonOperator":
        return self

    def _trace(self) -> float:
        if self.plan is not None:
            return float(self.plan.diagonal().sum().item())
        sel = self.indices[:, 0] == self.indices[:, 1]
        return float(np.sum(np.asarray(self.data)[sel]))


def _basis_plan_of(sector):
    return E.basis_plan(sector.num_sites, sector.n_up, sector.n_dn)


class _FermionOperator(LinearOperator):
    _create = True

    def __init__(self, sector, sector_t, pos=0, sigma=UP, jw_sign: bool = False):
        dim_origin = sector.size
        if sigma == UP:
            dim_target = sector_t.num_up * sector.num_dn
        else:
            dim_target = sector_t.num_dn * sector.num_up
        super().__init__(shape=(dim_target, dim_origin), dtype=np.complex64)
        self.pos = pos
        self.sigma = sigma
        self.jw_sign = jw_sign
        self.sector = sector
        self._target = sector_t

    def __repr__(self):
        name = f"{self.__class__.__name__}_{self.pos}{SPIN_CHARS[self.sigma]}"
        return f"{name}(shape: {self.shape}, dtype: {self.dtype})"

    def _apply_dev(self, x: torch.Tensor) -> torch.Tensor:
        src, dst = _basis_plan_of(self.sector), _basis_plan_of(self._target)
        return src.apply_fermion(dst, self.pos, self.sigma, self._create, x, jw_sign=self.jw_sign)

    def _matvec(self, x):
        return _apply_real(self._apply_dev, np.asarray(x).reshape(-1) if not isinstance(x, torch.Tensor) else x.reshape(-1))

    def _matmat(self, X):
        return _apply_real(self._apply_dev, X)


class CreationOperator(_FermionOperator):
    """c^dag_{pos,sigma} from `sector` into `sector_p1` (cmpy/operators.py:706-747)."""

    _create = True

    def __init__(self, sector, sector_p1, pos=0, sigma=UP, jw_sign: bool = False):
        super().__init__(sector, sector_p1, pos, sigma, jw_sign)
        self.sector_p1 = sector_p1

    def _adjoint(self):
        return AnnihilationOperator(self.sector_p1, self.sector, self.pos, self.sigma, self.jw_sign)


class AnnihilationOperator(_FermionOperator):
    """c_{pos,sigma} from `sector` into `sector_m1` (cmpy/operators.py:750-791)."""

    _create = False

    def __init__(self, sector, sector_m1, pos=0, sigma=UP, jw_sign: bool = False):
        super().__init__(sector, sector_m1, pos, sigma, jw_sign)
        self.sector_m1 = sector_m1

    def _adjoint(self):
        return CreationOperator(self.sector_m1, self.sector, self.pos, self.sigma, self.jw_sign)
