"""Local operator terms (same names, fields and bucketing as src/vmc/operators/local_terms.py).

Terms are plain frozen dataclasses holding NumPy arrays; the engine lowers a
``LocalHamiltonian`` into a compact device table (see ``vmc_gb300.plan``).
The local-energy convention is the reference's: an off-diagonal term at
sites with current local index ``s`` contributes ``sum_p op[p, s] psi(p) / psi``
(the column ``op[:, s]``; src/vmc/peps/common/energy.py:176-200).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "LocalTerm",
    "OneSiteTerm",
    "DiagonalTerm",
    "HorizontalTwoSiteTerm",
    "VerticalTwoSiteTerm",
    "PlaquetteTerm",
    "LocalHamiltonian",
    "bucket_terms",
    "heisenberg",
    "transverse_field_ising",
]


class LocalTerm:
    """local_terms.py:22-23."""


@dataclass(frozen=True)
class OneSiteTerm(LocalTerm):
    """local_terms.py:26-49: d x d operator at (row, col)."""

    row: int
    col: int
    op: np.ndarray

    def __post_init__(self):
        object.__setattr__(self, "op", np.asarray(self.op))

    @property
    def sites(self):
        return ((self.row, self.col),)


@dataclass(frozen=True)
class DiagonalTerm(LocalTerm):
    """local_terms.py:52-70: diagonal table indexed by sum s_k d^(n-1-k) over ``sites``."""

    sites: tuple
    diag: np.ndarray

    def __post_init__(self):
        object.__setattr__(self, "sites", tuple(tuple(int(v) for v in s) for s in self.sites))
        object.__setattr__(self, "diag", np.asarray(self.diag))


@dataclass(frozen=True)
class HorizontalTwoSiteTerm(LocalTerm):
    """local_terms.py:73-96: d^2 x d^2 operator on (row, col), (row, col+1)."""

    row: int
    col: int
    op: np.ndarray

    def __post_init__(self):
        object.__setattr__(self, "op", np.asarray(self.op))

    @property
    def sites(self):
        return ((self.row, self.col), (self.row, self.col + 1))


@dataclass(frozen=True)
class VerticalTwoSiteTerm(LocalTerm):
    """local_terms.py:99-122: d^2 x d^2 operator on (row, col), (row+1, col)."""

    row: int
    col: int
    op: np.ndarray

    def __post_init__(self):
        object.__setattr__(self, "op", np.asarray(self.op))

    @property
    def sites(self):
        return ((self.row, self.col), (self.row + 1, self.col))


@dataclass(frozen=True)
class PlaquetteTerm(LocalTerm):
    """local_terms.py:125-144 (used by the gauge-invariant model only)."""

    row: int
    col: int
    coeff: complex


@dataclass(frozen=True)
class LocalHamiltonian:
    """local_terms.py:147-162."""

    shape: tuple
    terms: tuple = field(default=())


def bucket_terms(terms, shape):
    """local_terms.py:165-200: group terms by type and lattice location."""
    n_rows, n_cols = shape
    one_site = [[[] for _ in range(n_cols)] for _ in range(n_rows)]
    horizontal = [[[] for _ in range(max(n_cols - 1, 0))] for _ in range(n_rows)]
    vertical = [[[] for _ in range(n_cols)] for _ in range(max(n_rows - 1, 0))]
    plaquette = [[[] for _ in range(max(n_cols - 1, 0))] for _ in range(max(n_rows - 1, 0))]
    diagonal = []
    for term in terms:
        if isinstance(term, OneSiteTerm):
            one_site[term.row][term.col].append(term)
        elif isinstance(term, HorizontalTwoSiteTerm):
            horizontal[term.row][term.col].append(term)
        elif isinstance(term, VerticalTwoSiteTerm):
            vertical[term.row][term.col].append(term)
        elif isinstance(term, DiagonalTerm):
            diagonal.append(term)
        elif isinstance(term, PlaquetteTerm):
            plaquette[term.row][term.col].append(term)
        else:
            raise TypeError(f"Unsupported term type: {type(term)!r}")
    return diagonal, one_site, horizontal, vertical, plaquette


def heisenberg(shape, bond_op=None, J: float = 1.0) -> LocalHamiltonian:
    """Nearest-neighbour Heisenberg model H = J sum <ij> S_i . S_j (S = sigma/2) in the Sz basis.

    The default bond operator is 1/4 [[1,0,0,0],[0,-1,2,0],[0,2,-1,0],[0,0,0,1]]
    on every horizontal and vertical bond of the open lattice.
    """
    if bond_op is None:
        bond_op = 0.25 * J * np.array([[1, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]],
                                      dtype=np.float64)
    n_rows, n_cols = shape
    terms = []
    for r in range(n_rows):
        for c in range(n_cols):
            if c + 1 < n_cols:
                terms.append(HorizontalTwoSiteTerm(r, c, bond_op))
            if r + 1 < n_rows:
                terms.append(VerticalTwoSiteTerm(r, c, bond_op))
    return LocalHamiltonian(shape=tuple(shape), terms=tuple(terms))


def transverse_field_ising(shape, J: float = 1.0, h: float = 3.0) -> LocalHamiltonian:
    """H = -J sum <ij> z_i z_j - h sum x_i, built as examples/ground_states/ising.py:36-53 does."""
    n_rows, n_cols = shape
    diag_zz = -J * np.array([1.0, -1.0, -1.0, 1.0])
    op_x = -h * np.array([[0.0, 1.0], [1.0, 0.0]])
    terms = []
    for r in range(n_rows):
        for c in range(n_cols):
            terms.append(OneSiteTerm(r, c, op_x))
            if c + 1 < n_cols:
                terms.append(DiagonalTerm(((r, c), (r, c + 1)), diag_zz))
            if r + 1 < n_rows:
                terms.append(DiagonalTerm(((r, c), (r + 1, c)), diag_zz))
    return LocalHamiltonian(shape=tuple(shape), terms=tuple(terms))
