"""Model classes — drop-in for ``cmpy.models`` (cmpy/models/abc.py, hubbard.py, anderson.py,
heisenberg.py).

The plugin surface is the reference's: a many-body model implements
``_hamiltonian_data(up_states, dn_states)`` yielding (row, col, value) triplets
(cmpy/models/abc.py:238-240). The built-in models additionally describe themselves to the
GPU engine (``fermion_descriptor`` / ``spin_descriptor``: on-site energies, U, bonds,
couplings), so ``hamilton_operator`` returns a matrix-free operator whose tables are built on
the device. A user model that only implements ``_hamiltonian_data`` still works: its triplets
are applied by the device CSR kernel.
"""

from __future__ import annotations

import json
from abc import ABC, abstractmethod
from collections import OrderedDict
from collections.abc import MutableMapping
from typing import Any, Dict, Iterator, List, Optional, Sequence, Union

import numpy as np
import torch

from . import engine as E
from .basis import UP, Basis, SpinBasis
from .operators import (
    HamiltonOperator,
    project_hopping,
    project_hopping_arrays,
    project_hubbard_inter,
    project_hubbard_inter_arrays,
    project_onsite_energy,
    project_onsite_energy_arrays,
)

__all__ = [
    "ModelParameters",
    "AbstractModel",
    "AbstractSpinModel",
    "AbstractManyBodyModel",
    "HubbardModel",
    "SingleImpurityAndersonModel",
    "HeisenbergModel",
    "ChainLattice",
]


class ModelParameters(MutableMapping):
    """A model's named parameters, reachable both as attributes (``model.u``) and as mapping
    items (``model["u"]``). The parameter names are the keyword arguments the constructor
    received plus later ``set_param`` calls; every other attribute is an ordinary instance
    attribute. Public surface as cmpy/models/abc.py:21-133.
    """

    def __init__(self, **params):
        object.__setattr__(self, "_values", dict(params))

    # ---- mapping over the parameters only ----------------------------------------------------
    def __getitem__(self, name: str) -> Any:
        return self._values[name]

    def __setitem__(self, name: str, value: Any) -> None:
        self._values[name] = value

    def __delitem__(self, name: str) -> None:
        self._values.pop(name)

    def __iter__(self) -> Iterator[str]:
        return iter(tuple(self._values))

    def __len__(self) -> int:
        return len(self._values)

    # ---- attribute access: ordinary lookup first, then the parameters --------------------------
    def __getattr__(self, name: str) -> Any:
        values = self.__dict__.get("_values", {})
        if name in values:
            return values[name]
        raise AttributeError(f"{type(self).__name__} has neither an attribute nor a parameter {name!r}")

    def __setattr__(self, name: str, value: Any) -> None:
        if name in self.__dict__.get("_values", {}):
            self._values[name] = value
        else:
            object.__setattr__(self, name, value)

    @property
    def params(self) -> Dict[str, Any]:
        return self._values

    def set_param(self, key: str, value: Any) -> None:
        """Add (or overwrite) a parameter; it becomes an attribute of the model."""
        self._values[key] = value

    def delete_param(self, key: str) -> None:
        self._values.pop(key)

    def rename_param(self, key: str, new_key: str) -> None:
        """Rename a parameter in place (its position in the parameter order is kept)."""
        self._values = {(new_key if k == key else k): v for k, v in self._values.items()}

    @staticmethod
    def _fmt(value, decimals=None) -> str:
        if decimals is not None and isinstance(value, (float, np.floating)):
            return f"{float(value):.{decimals}f}"
        return str(value)

    def key(self, decimals=None, delim="; "):
        """One-line identifier of the parameter set, e.g. for cache keys or file names."""
        return delim.join(f"{k}={self._fmt(v, decimals)}" for k, v in self._values.items())

    def json(self):
        def plain(v):
            if isinstance(v, np.ndarray):
                return v.tolist()
            if isinstance(v, np.generic):
                return v.item()
            return v

        return json.dumps({k: plain(v) for k, v in self._values.items()})

    def pformat(self):
        return ", ".join(f"{k}={self._fmt(v)}" for k, v in self._values.items())

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.pformat()})"

    def __str__(self) -> str:
        return self.pformat()


class AbstractModel(ModelParameters, ABC):
    """Base of every model: a parameter set plus a Hamiltonian."""

    def __str__(self) -> str:
        return f"{type(self).__name__}({self.pformat()})"

    def hamiltonian(self, *args, **kwargs):
        raise NotImplementedError


class _PlanCache:
    """Per-model cache of device plans keyed by the model description and sector."""

    def __init__(self, size: int = 8):
        self.size = size
        self._d: "OrderedDict[Any, E.Plan]" = OrderedDict()

    def get(self, key, build):
        key = (torch.cuda.current_device(), key)
        p = self._d.get(key)
        if p is None:
            p = build()
            self._d[key] = p
            while len(self._d) > self.size:
                self._d.popitem(last=False)
        else:
            self._d.move_to_end(key)
        return p


def _is_full_sector(states, num_sites: int, n) -> bool:
    if n is None:
        return False
    return len(states) == E.sector_size(num_sites, n)


class AbstractManyBodyModel(AbstractModel):
    """Fermionic many-body model on a Fock basis (cmpy/models/abc.py:206-260)."""

    def __init__(self, num_sites: Optional[int] = 0, **params):
        ModelParameters.__init__(self, **params)
        self.basis: Basis = Basis()
        self.init_basis(num_sites)
        object.__setattr__(self, "_plans", _PlanCache())

    @property
    def num_sites(self) -> int:
        return self.basis.num_sites

    @property
    def fillings(self) -> List[int]:
        return self.basis.fillings

    def init_basis(self, num_sites, init_sectors=None):
        self.basis.init(num_sites, init_sectors)

    def iter_fillings(self):
        return self.basis.iter_fillings()

    def iter_sectors(self):
        return self.basis.iter_sectors()

    def get_sector(self, n_up=None, n_dn=None):
        return self.basis.get_sector(n_up, n_dn)

    # -- engine description ----------------------------------------------------------------
    def fermion_descriptor(self):
        """(eps[N], u[N], bonds[(i, j, hop)], sign_width) or None for triplet-only models."""
        return None

    def plan(self, n_up: int, n_dn: int) -> "E.Plan":
        return self.plans([(n_up, n_dn)])[0]

    def plans(self, sectors) -> list:
        """Plans of several (n_up, n_dn) sectors of the current parameters (one descriptor for
        all of them); a None entry gives None."""
        desc = self.fermion_descriptor()
        if desc is None:
            raise NotImplementedError(f"{type(self).__name__} has no engine descriptor")
        eps, u, bonds, width = desc
        base = (tuple(np.asarray(eps, float).tolist()), tuple(np.asarray(u, float).tolist()),
                tuple(tuple(b) for b in bonds), int(width))
        out = []
        for sec in sectors:
            if sec is None:
                out.append(None)
                continue
            nu, nd = int(sec[0]), int(sec[1])
            out.append(self._plans.get(base + (nu, nd),
                                       lambda nu=nu, nd=nd: E.Plan.fermion(self.num_sites, eps, u, bonds, nu, nd, width)))
        return out

    # -- reference surface -----------------------------------------------------------------
    @abstractmethod
    def _hamiltonian_data(self, up_states, dn_states):
        pass

    def hamiltonian_data_arrays(self, up_states, dn_states):
        """Device (rows, cols, vals) in the reference's emission order."""
        desc = self.fermion_descriptor()
        if desc is None:
            rows, cols, vals = [], [], []
            for r, c, v in self._hamiltonian_data(up_states, dn_states):
                rows.append(r)
                cols.append(c)
                vals.append(v)
            dev = E.device()
            return (torch.as_tensor(np.asarray(rows, np.int64)).to(dev), torch.as_tensor(np.asarray(cols, np.int64)).to(dev),
                    torch.as_tensor(np.asarray(vals, np.float64)).to(dev))
        eps, u, bonds, width = desc
        parts = [project_onsite_energy_arrays(up_states, dn_states, eps),
                 project_hubbard_inter_arrays(up_states, dn_states, u)]
        for i, j, t in bonds:
            parts.append(E.coo_hopping(up_states, dn_states, width, i, j, t))
        return tuple(torch.cat([p[k] for p in parts]) for k in range(3))

    def hamiltonian_data(self, up_states, dn_states):
        """(data, int64[2, nnz]) like cmpy/models/abc.py:242-248."""
        rows, cols, vals = (a.cpu().numpy() for a in self.hamiltonian_data_arrays(up_states, dn_states))
        return vals, np.array([rows, cols], dtype=np.int64)

    def hamilton_operator(self, n_up=None, n_dn=None, sector=None, dtype=None) -> HamiltonOperator:
        if sector is None:
            sector = self.basis.get_sector(n_up, n_dn)
        up_states, dn_states = sector.up_states, sector.dn_states
        if (self.fermion_descriptor() is not None and _is_full_sector(up_states, self.num_sites, sector.n_up)
                and _is_full_sector(dn_states, self.num_sites, sector.n_dn)):
            return HamiltonOperator.from_plan(self.plan(sector.n_up, sector.n_dn), dtype=dtype)
        size = len(up_states) * len(dn_states)
        data, indices = self.hamiltonian_data(up_states, dn_states)
        return HamiltonOperator(size, data, indices, dtype=dtype)

    def hamiltonian(self, n_up=None, n_dn=None, sector=None, dtype=None) -> np.ndarray:
        return self.hamilton_operator(n_up, n_dn, sector, dtype).toarray()


class HubbardModel(AbstractManyBodyModel):
    """Hubbard model (cmpy/models/hubbard.py:37-81):
    H = U sum_i n_iu n_id + sum_is (eps_i - mu) n_is + t sum_<ij>s c^dag_is c_js.

    ``HubbardModel(latt, ...)`` or ``HubbardModel(num_sites, neighbors, ...)``; only pairs
    with i < j of ``neighbors`` become bonds (hubbard.py:19-21). ``eps`` and ``inter`` may be
    scalars or per-site arrays.
    """

    def __init__(self, *args, inter=0.0, eps=0.0, hop=1.0, mu=0.0):
        if len(args) == 1:
            latt = args[0]
            num_sites = latt.num_sites
            neighbors = latt.neighbor_pairs(True)[0]
        else:
            num_sites, neighbors = args
        super().__init__(num_sites, inter=inter, eps=eps, hop=hop, mu=mu)
        self.neighbors = neighbors

    def pformat(self):
        return f"U={self.inter}, ε={self.eps}, t={self.hop}, μ={self.mu}"

    def fermion_descriptor(self):
        n = self.num_sites
        energy = np.full(n, self.eps - self.mu, dtype=np.float64)
        interaction = np.full(n, self.inter, dtype=np.float64)
        bonds = [(int(i), int(j), float(self.hop)) for i, j in self.neighbors if i < j]
        return energy, interaction, bonds, n

    def _hamiltonian_data(self, up_states, dn_states):
        energy, interaction, bonds, n = self.fermion_descriptor()
        yield from project_onsite_energy(up_states, dn_states, energy)
        yield from project_hubbard_inter(up_states, dn_states, interaction)
        for i, j, t in bonds:
            yield from project_hopping(up_states, dn_states, n, i, j, t)


class SingleImpurityAndersonModel(AbstractManyBodyModel):
    """Single-impurity Anderson model in star geometry (cmpy/models/anderson.py:24-164).

    Site 0 is the impurity, sites 1..N_b the bath. ``physical_signs=False`` keeps the
    reference's hopping without fermionic sign (anderson.py:149 passes width 0)."""

    def __init__(self, u=2.0, eps_imp=0.0, eps_bath=0.0, v=1.0, mu=None, temp=0.0, physical_signs: bool = False):
        mu = u / 2 if mu is None else mu
        eps_bath = np.atleast_1d(np.asarray(eps_bath, dtype=np.float64))
        v = np.atleast_1d(np.asarray(v, dtype=np.float64))
        num_bath = len(eps_bath)
        if num_bath > 1 and len(v) == 1:
            v = np.ones(len(eps_bath)) * v[0]
        if num_bath == 1 and len(v) > 1:
            eps_bath = np.ones(len(v)) * eps_bath[0]
        assert len(eps_bath) == len(v), (
            f"Shape of bath on-site energy {num_bath} doesn't match hybridization {len(v)}!")
        super().__init__(len(eps_bath) + 1, u=u, eps_imp=eps_imp, eps_bath=eps_bath, v=v, mu=mu, temp=temp)
        object.__setattr__(self, "physical_signs", bool(physical_signs))

    @property
    def num_bath(self) -> int:
        return len(self.eps_bath)

    @property
    def num_sites(self) -> int:
        return self.num_bath + 1

    @property
    def beta(self) -> float:
        return 1 / self.temp

    def update_bath_energy(self, eps_bath) -> None:
        eps_bath = np.atleast_1d(eps_bath).astype(np.float64)
        if eps_bath.shape[0] != self.num_bath:
            raise ValueError(f"Dimension of the new bath energy {eps_bath.shape} does not match number of baths "
                             f"{self.num_bath}")
        self.eps_bath = eps_bath

    def update_hybridization(self, v) -> None:
        v = np.atleast_1d(v).astype(np.float64)
        if v.shape[0] != self.num_bath:
            raise ValueError(f"Dimension of the new hybridization {v.shape} does not match number of baths "
                             f"{self.num_bath}")
        self.v = v

    def hybridization_func(self, z):
        """Delta(z) = sum_i |V_i|^2 / (z - eps_i) (anderson.py:127-145); torch in -> torch out."""
        if isinstance(z, torch.Tensor):
            v = torch.as_tensor(self.v, dtype=torch.float64, device=z.device)
            eb = torch.as_tensor(self.eps_bath, dtype=torch.float64, device=z.device)
            return torch.sum(v.abs() ** 2 / (z[..., None] - eb), dim=-1)
        x = np.asarray(z)[..., np.newaxis]
        return np.sum(np.square(np.abs(self.v)) / (x - self.eps_bath), axis=-1)

    def impurity_gf0(self, z):
        return 1 / (z + self.mu + self.eps_imp - self.hybridization_func(z))

    def fermion_descriptor(self):
        u = np.append(self.u, np.zeros(self.num_bath)).astype(np.float64)
        eps = np.append(self.eps_imp - self.mu, self.eps_bath).astype(np.float64)
        bonds = [(0, j + 1, float(self.v[j])) for j in range(self.num_bath)]
        width = self.num_sites if self.physical_signs else 0
        return eps, u, bonds, width

    def _hamiltonian_data(self, up_states, dn_states):
        eps, u, bonds, width = self.fermion_descriptor()
        yield from project_onsite_energy(up_states, dn_states, eps)
        yield from project_hubbard_inter(up_states, dn_states, u)
        for i, j, t in bonds:
            yield from project_hopping(up_states, dn_states, width, i, j, t)

    def impurity_gf(self, z, sigma=UP):
        from .exactdiag import gf_lehmann

        return gf_lehmann(self, z, beta=1 / self.temp, pos=0, sigma=sigma).gf

    def pformat(self):
        return (f"U={self.u}, ε_i={self.eps_imp}, ε_b={self.eps_bath}, v={self.v}, "
                f"μ={self.mu}, T={self.temp}")


class ChainLattice:
    """Minimal lattice for chains/rings (stands in for the lattpy objects the reference takes):
    ``num_sites``, ``neighbors(pos)`` and ``neighbor_pairs(unique)``."""

    def __init__(self, num_sites: int, periodic: bool = False):
        self.num_sites = int(num_sites)
        self.periodic = bool(periodic)

    def neighbors(self, pos: int) -> List[int]:
        n = self.num_sites
        out = []
        if pos - 1 >= 0:
            out.append(pos - 1)
        elif self.periodic and n > 2:
            out.append(n - 1)
        if pos + 1 < n:
            out.append(pos + 1)
        elif self.periodic and n > 2:
            out.append(0)
        if self.periodic and n == 2 and not out:
            out.append(1 - pos)
        return sorted(set(out))

    def neighbor_pairs(self, unique: bool = False):
        pairs = []
        for i in range(self.num_sites):
            for j in self.neighbors(i):
                if not unique or i < j:
                    pairs.append([i, j])
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        return pairs, np.ones(len(pairs), dtype=np.int64)


class AbstractSpinModel(AbstractModel):
    """Spin model on Sz sectors (cmpy/models/abc.py:160-203)."""

    def __init__(self, num_sites: Optional[int] = 0, **params):
        ModelParameters.__init__(self, **params)
        self.basis: SpinBasis = SpinBasis()
        self.init_basis(num_sites)
        object.__setattr__(self, "_plans", _PlanCache())

    @property
    def num_sites(self) -> int:
        return self.basis.num_sites

    @property
    def spins(self) -> List[int]:
        return self.basis.spins

    def init_basis(self, num_sites: int, init_sectors: bool = None):
        self.basis.init(num_sites, init_sectors)

    def get_states(self, s: float = None):
        return self.basis.get_states(s)

    def spin_descriptor(self):
        """Directed pairs [(pos1, pos2, j, jz)] in emission order, or None."""
        return None

    def plan(self, s: float = None) -> "E.Plan":
        pairs = self.spin_descriptor()
        if pairs is None:
            raise NotImplementedError(f"{type(self).__name__} has no engine descriptor")
        n_up = -1 if s is None else self.basis.n_up(s)
        key = (tuple(tuple(p) for p in pairs), n_up)
        return self._plans.get(key, lambda: E.Plan.spin(self.num_sites, pairs, n_up))

    @abstractmethod
    def _hamiltonian_data(self, states):
        pass

    def hamiltonian_data(self, states):
        rows, cols, data = list(), list(), list()
        for row, col, val in self._hamiltonian_data(states):
            rows.append(row)
            cols.append(col)
            data.append(val)
        return data, (rows, cols)

    def hamilton_operator(self, s=None, states=None, dtype=None) -> HamiltonOperator:
        if states is None and self.spin_descriptor() is not None:
            return HamiltonOperator.from_plan(self.plan(s), dtype=dtype)
        if states is None:
            states = self.get_states(s)
        data, indices = self.hamiltonian_data(states)
        return HamiltonOperator(len(states), data, indices, dtype=dtype)

    def hamiltonian(self, s=None, states=None, dtype=None):
        return self.hamilton_operator(s, states, dtype).toarray()


def _coupling(c, i: int, k: int) -> float:
    if np.ndim(c) == 0:
        return float(c)
    return float(np.asarray(c)[i, k])


class HeisenbergModel(AbstractSpinModel):
    """Spin-1/2 XXZ model (cmpy/models/heisenberg.py). ``latt`` needs ``num_sites`` and
    ``neighbors(pos)``. ``j``/``jz`` are scalars like the reference or symmetric (N, N)
    arrays of per-bond couplings. Each directed neighbour pair contributes sign*0.25*jz to
    the diagonal and (0.25*j)/2 to a spin flip (heisenberg.py:19-40)."""

    def __init__(self, latt, j=1.0, jz=None):
        super().__init__(latt.num_sites)
        self.latt = latt
        self.j = j
        self.jz = j if jz is None else jz

    def spin_descriptor(self):
        pairs = []
        for p1 in range(self.num_sites):
            for p2 in self.latt.neighbors(p1):
                p2 = int(p2)
                pairs.append((p1, p2, _coupling(self.j, p1, p2), _coupling(self.jz, p1, p2)))
        return pairs

    def _hamiltonian_data(self, states):
        plan = E.Plan.spin(self.num_sites, self.spin_descriptor(), -1)
        rows, cols, vals = (a.cpu().numpy() for a in plan.coo())
        states = np.asarray(states, dtype=np.int64)
        # the full-space plan indexes by state value; map to positions in `states`
        pos = np.full(1 << self.num_sites, -1, dtype=np.int64)
        pos[states] = np.arange(len(states))
        keep = (pos[rows] >= 0) & (pos[cols] >= 0)
        yield from zip(pos[rows[keep]].tolist(), pos[cols[keep]].tolist(), vals[keep].tolist())
