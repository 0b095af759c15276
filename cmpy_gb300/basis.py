"""Fock basis and spin sectors — drop-in for ``cmpy.basis`` (cmpy/basis.py).

The string/bit helpers are host-side formatting. Sector enumeration (Basis.generate_states,
SpinBasis.generate_states) runs on the GPU through ``ed_enumerate``: the ascending integers
with popcount n are produced by unranking the combinatorial number system, so the order is
exactly the reference's sorted-permutation order (cmpy/basis.py:655-666).
"""

from __future__ import annotations

from collections import defaultdict
from itertools import product
from typing import Iterable, List, Tuple, Union

import numpy as np

__all__ = [
    "UP",
    "DN",
    "SPIN_CHARS",
    "state_label",
    "bit_count",
    "binstr",
    "binarr",
    "binidx",
    "get_ibit",
    "set_ibit",
    "overlap",
    "occupations",
    "create",
    "annihilate",
    "SpinState",
    "State",
    "upper_sector",
    "lower_sector",
    "Sector",
    "Basis",
    "SpinBasis",
    "spinstate_label",
]

UP, DN = 1, 2  # spin channels (cmpy/basis.py:39)

EMPTY_CHAR = "."
UP_CHAR = "↑"
DN_CHAR = "↓"
UD_CHAR = "⇅"
SPIN_CHARS = {0: EMPTY_CHAR, UP: UP_CHAR, DN: DN_CHAR, 3: UD_CHAR}


def state_label(up_num: int, dn_num: int, digits: int = None) -> str:
    """Label of an (up, dn) pair, one character per site, site 0 first (cmpy/basis.py:48-73)."""
    width = max(int(up_num).bit_length() or 1, int(dn_num).bit_length() or 1, digits or 0)
    chars = [SPIN_CHARS[((int(up_num) >> i) & 1) | (((int(dn_num) >> i) & 1) << 1)] for i in range(width)]
    return "".join(chars)


def bit_count(num: int) -> int:
    """Number of set bits."""
    return bin(int(num)).count("1")


def binstr(num: int, width: int = 0) -> str:
    """Binary string, most significant bit first, zero-padded to `width`."""
    return format(int(num), f"0{width or 0}b")


def binarr(num: int, width: int = None, dtype=None) -> np.ndarray:
    """Bits as an array, index 0 = bit 0 (cmpy/basis.py:123-157)."""
    s = format(int(num), f"0{width or 0}b")[::-1]
    return np.fromiter((int(c) for c in s), dtype=dtype or np.int64, count=len(s))


def binidx(num, width: int = None) -> List[int]:
    """Indices of the set bits, ascending."""
    n = int(num)
    return [i for i in range(max(n.bit_length(), width or 0)) if (n >> i) & 1]


def get_ibit(num: int, index: int, length: int = 1) -> int:
    return (int(num) >> index) & ((1 << length) - 1)


def set_ibit(num: int, index: int, value: int, length: int = 1) -> int:
    mask = ((1 << length) - 1) << index
    return (int(num) & ~mask) | ((int(value) << index) & mask)


def overlap(num1: int, num2: int, width: int = None, dtype=None) -> np.ndarray:
    """Bits of num1 & num2 as an array."""
    return binarr(int(num1) & int(num2), width, dtype)


def occupations(num: int, width: int = None, dtype=None) -> np.ndarray:
    return binarr(num, width, dtype)


def create(num: int, pos: int) -> Union[int, None]:
    """State with a particle created at pos, or None if occupied (cmpy/basis.py:345-380)."""
    op = 1 << pos
    return None if int(num) & op else int(num) ^ op


def annihilate(num: int, pos: int) -> Union[int, None]:
    """State with the particle at pos removed, or None if empty (cmpy/basis.py:383-416)."""
    op = 1 << pos
    return int(num) ^ op if int(num) & op else None


class SpinState(int):
    """Integer bitstring of one spin species (cmpy/basis.py:422-468)."""

    @property
    def n(self) -> int:
        return bit_count(self)

    def binstr(self, width: int = None) -> str:
        return binstr(self, width)

    def binarr(self, width: int = None, dtype=None) -> np.ndarray:
        return binarr(self, width, dtype)

    def occ(self, pos: int) -> int:
        return self & (1 << pos)

    def occupations(self, dtype=None) -> np.ndarray:
        return binarr(self, dtype=dtype)

    def overlap(self, other, dtype=None) -> np.ndarray:
        return overlap(self, other, dtype=dtype)

    def create(self, pos: int):
        num = create(self, pos)
        return None if num is None else self.__class__(num)

    def annihilate(self, pos: int):
        num = annihilate(self, pos)
        return None if num is None else self.__class__(num)

    def __repr__(self) -> str:
        return f"{self.__class__.__name__}({self.binstr()})"

    def __str__(self) -> str:
        return self.binstr()


class State:
    """An (up, dn) pair of spin states (cmpy/basis.py:471-499)."""

    __slots__ = ["up", "dn", "num_sites"]

    def __init__(self, up, dn, num_sites: int = None):
        self.up = SpinState(up)
        self.dn = SpinState(dn)
        self.num_sites = num_sites

    def label(self, width: int = None) -> str:
        return state_label(self.up, self.dn, width if width is not None else self.num_sites)

    def __repr__(self) -> str:
        return f"{self.__class__.__name__}({self.up}, {self.dn})"

    def __str__(self) -> str:
        return f"{self.__class__.__name__}: {self.label()}"

    def __eq__(self, other) -> bool:
        return self.up == other.up and self.dn == other.dn


def upper_sector(n_up: int, n_dn: int, sigma: int, num_sites: int) -> Union[Tuple[int, int], None]:
    """(n_up+1, n_dn) or (n_up, n_dn+1), None at the top (cmpy/basis.py:504-528)."""
    if sigma == UP and n_up < num_sites:
        return n_up + 1, n_dn
    if sigma == DN and n_dn < num_sites:
        return n_up, n_dn + 1
    return None


def lower_sector(n_up: int, n_dn: int, sigma: int) -> Union[Tuple[int, int], None]:
    """(n_up-1, n_dn) or (n_up, n_dn-1), None at the bottom (cmpy/basis.py:531-553)."""
    if sigma == UP and n_up > 0:
        return n_up - 1, n_dn
    if sigma == DN and n_dn > 0:
        return n_up, n_dn - 1
    return None


class Sector:
    """Up- and dn-state lists of one (n_up, n_dn) sector; many-body index is up-major
    (idx = up_idx * num_dn + dn_idx, cmpy/basis.py:556-603)."""

    __slots__ = ["num_sites", "n_up", "n_dn", "up_states", "dn_states"]

    def __init__(self, up_states, dn_states, n_up=None, n_dn=None, num_sites=0):
        self.num_sites = num_sites
        self.n_up = n_up
        self.n_dn = n_dn
        self.up_states = up_states
        self.dn_states = dn_states

    @property
    def states(self):
        for up, dn in product(self.up_states, self.dn_states):
            yield State(up, dn, num_sites=self.num_sites)

    @property
    def size(self) -> int:
        return len(self.up_states) * len(self.dn_states)

    @property
    def num_up(self) -> int:
        return len(self.up_states)

    @property
    def num_dn(self) -> int:
        return len(self.dn_states)

    @property
    def filling(self):
        return self.n_up, self.n_dn

    def state_labels(self):
        return [s.label(self.num_sites) for s in self.states]

    def __repr__(self):
        return (f"{self.__class__.__name__}(size: {self.size}, num_sites: {self.num_sites}, "
                f"filling: [{self.n_up}, {self.n_dn}])")

    def __str__(self):
        return f"{self.__class__.__name__}({self.n_up}, {self.n_dn}, size: {self.size})"

    def __iter__(self):
        return iter(self.states)


def _gpu_states(num_sites: int, n) -> np.ndarray:
    from .engine import enumerate_states

    return enumerate_states(num_sites, n).cpu().numpy()


class Basis:
    """All basis states of the Hilbert space, grouped by filling (cmpy/basis.py:606-718).

    States of a filling are generated on the GPU on first use and cached as int64 arrays.
    """

    __slots__ = ["size", "num_sites", "num_spinstates", "sectors", "fillings"]

    def __init__(self, num_sites: int = 0, init_sectors: bool = False):
        self.size = 0
        self.num_sites = 0
        self.num_spinstates = 0
        self.sectors = defaultdict(list)
        self.fillings = []
        self.init(num_sites, init_sectors)

    def init(self, num_sites: int, init_sectors: bool = False):
        self.num_sites = num_sites
        self.num_spinstates = 2**num_sites
        self.size = self.num_spinstates**2
        self.sectors = defaultdict(list)
        self.fillings = list(range(self.num_sites + 1))
        if init_sectors:
            for n in range(num_sites + 1):
                self.sectors[n] = _gpu_states(num_sites, n)

    def generate_states(self, n: int = None) -> np.ndarray:
        return _gpu_states(self.num_sites, n)

    def get_states(self, n: int = None) -> np.ndarray:
        if n in self.sectors:
            return self.sectors[n]
        states = self.generate_states(n)
        self.sectors[n] = states
        return states

    def get_sector(self, n_up: int = None, n_dn: int = None) -> Sector:
        return Sector(self.get_states(n_up), self.get_states(n_dn), n_up, n_dn, self.num_sites)

    def iter_fillings(self):
        return product(self.fillings, repeat=2)

    def iter_sectors(self):
        for n_up, n_dn in product(self.fillings, repeat=2):
            yield self.get_sector(n_up, n_dn)

    def keys(self):
        return self.fillings

    def check(self, n_up, n_dn):
        return n_up in self.fillings and n_dn in self.fillings

    def upper_sector(self, n_up, n_dn, sigma):
        f = upper_sector(n_up, n_dn, sigma, self.num_sites)
        return None if f is None else self.get_sector(*f)

    def lower_sector(self, n_up, n_dn, sigma):
        f = lower_sector(n_up, n_dn, sigma)
        return None if f is None else self.get_sector(*f)

    def __getitem__(self, item):
        if hasattr(item, "__len__"):
            return self.get_sector(*item)
        return self.get_states(item)

    def __repr__(self):
        return (f"{self.__class__.__name__}(size: {self.size}, num_sites: {self.num_sites}, "
                f"fillings: {self.fillings})")


def spinstate_label(state: int, digits: int = None) -> str:
    chars = {"0": DN_CHAR, "1": UP_CHAR}
    return "".join(chars[c] for c in binstr(state, digits))


class SpinBasis:
    """Sz sectors of a spin-1/2 chain (cmpy/basis.py:726-787): the states with
    N/2 + s up-spins (bit = 1), ascending."""

    __slots__ = ["size", "num_sites", "num_spinstates", "sectors", "spins"]

    def __init__(self, num_sites: int = 0):
        self.size = 0
        self.num_sites = 0
        self.num_spinstates = 0
        self.sectors = defaultdict(list)
        self.spins = list()
        self.init(num_sites)

    def init(self, num_sites: int, init_sectors: bool = False):
        self.num_sites = num_sites
        self.num_spinstates = 2**num_sites
        self.size = self.num_sites**2
        self.spins = list(np.arange(-0.5 * num_sites, +0.5 * num_sites + 0.1, 1))
        if init_sectors:
            for s in self.spins:
                self.sectors[s] = list(self.generate_states(s))

    def n_up(self, s: float) -> int:
        n_up = self.num_sites / 2 + s
        n_dn = self.num_sites / 2 - s
        if (n_up % 1 != 0.0) or (n_dn % 1 != 0.0) or n_up < 0 or n_dn < 0:
            raise ValueError(f"Total spin of {s} not realizable with {self.num_sites} sites")
        return int(n_up)

    def generate_states(self, s: float = None) -> List[int]:
        if s is None:
            return list(range(2**self.num_sites))
        return _gpu_states(self.num_sites, self.n_up(s)).tolist()

    def get_states(self, s: float = None) -> List[int]:
        if s in self.sectors:
            return self.sectors[s]
        states = self.generate_states(s)
        self.sectors[s] = list(states)
        return self.sectors[s]

    def state_labels(self, s: float = None):
        return [spinstate_label(state, self.num_sites) for state in self.get_states(s)]

    def __getitem__(self, item) -> List[int]:
        return self.get_states(item)

    def __repr__(self):
        return (f"{self.__class__.__name__}(size: {self.size}, num_sites: {self.num_sites}, "
                f"spins: {self.spins})")
