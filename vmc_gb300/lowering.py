"""Host-side lowering of model parameters and operators into the C-ABI formats.

* ``pack_tensors``: site tensors -> one flat FP32 vector, site-major, each
  site (d, up, down, left, right) C-order -- the parameter order of the
  reference's ``ravel_pytree(model.tensors)``.
* ``lower_operator``: ``LocalHamiltonian`` -> the dense per-location tables of
  ``vmc_peps_plan_set_operator``.  Terms of one kind at one location are
  summed (their local-energy contributions are linear in the operator);
  bucketing follows src/vmc/operators/local_terms.py:165-200.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .operators import bucket_terms

__all__ = ["LoweredOperator", "lower_operator", "pack_tensors", "site_dims", "params_per_site"]


def site_dims(row: int, col: int, n_rows: int, n_cols: int, bond_dim: int):
    """src/vmc/peps/standard/model.py:27-35."""
    up = 1 if row == 0 else bond_dim
    down = 1 if row == n_rows - 1 else bond_dim
    left = 1 if col == 0 else bond_dim
    right = 1 if col == n_cols - 1 else bond_dim
    return up, down, left, right


def params_per_site(shape, bond_dim):
    """src/vmc/utils/smallo.py:23-35."""
    n_rows, n_cols = shape
    return [int(np.prod(site_dims(r, c, n_rows, n_cols, bond_dim)))
            for r in range(n_rows) for c in range(n_cols)]


def pack_tensors(tensors, complex_elements: bool | None = None) -> np.ndarray:
    """ravel_pytree order of tensors[r][c].  Complex tensors (or complex_elements=True) pack as
    complex64; real ones as float32."""
    if complex_elements is None:
        complex_elements = any(np.iscomplexobj(t) for row in tensors for t in row)
    dt = np.complex64 if complex_elements else np.float32
    return np.concatenate([np.asarray(t).astype(dt).reshape(-1) for row in tensors for t in row])


@dataclass
class LoweredOperator:
    onesite: np.ndarray
    onesite_mask: np.ndarray
    horiz: np.ndarray
    horiz_mask: np.ndarray
    vert: np.ndarray
    vert_mask: np.ndarray
    diag_nsites: np.ndarray
    diag_site_off: np.ndarray
    diag_sites: np.ndarray
    diag_value_off: np.ndarray
    diag_values: np.ndarray

    @property
    def n_diag(self) -> int:
        return int(self.diag_nsites.shape[0])


def _as_complex(op, what):
    return np.asarray(op, dtype=np.complex128)


def _real(op, what):
    op = np.asarray(op)
    if np.iscomplexobj(op):
        if np.max(np.abs(op.imag)) > 0:
            raise NotImplementedError(f"complex {what} operators need the complex engine")
        op = op.real
    return np.asarray(op, dtype=np.float64)


def lower_operator(operator, shape, phys_dim: int, complex_elements: bool = False) -> LoweredOperator:
    """Dense per-location tables of the operator's terms.  For a complex engine
    (complex_elements=True) the one-site, horizontal and vertical tables are
    complex128, handed to the C ABI as interleaved (re, im) doubles; diagonal
    tables stay real."""
    n_rows, n_cols = shape
    d, d2 = phys_dim, phys_dim * phys_dim
    _mat = _as_complex if complex_elements else _real
    mdt = np.complex128 if complex_elements else np.float64
    diagonal, one_site, horizontal, vertical, plaquette = bucket_terms(operator.terms, shape)
    if any(t for row in plaquette for t in row):
        raise NotImplementedError("PlaquetteTerm belongs to the gauge-invariant PEPS model")
    n_sites = n_rows * n_cols
    onesite = np.zeros((n_sites, d, d), dtype=mdt)
    onesite_mask = np.zeros(n_sites, dtype=np.int32)
    for r in range(n_rows):
        for c in range(n_cols):
            for term in one_site[r][c]:
                onesite[r * n_cols + c] += _mat(term.op, "one-site").reshape(d, d)
                onesite_mask[r * n_cols + c] = 1
    nh = max(n_rows * (n_cols - 1), 1)
    horiz = np.zeros((nh, d2, d2), dtype=mdt)
    horiz_mask = np.zeros(nh, dtype=np.int32)
    for r in range(n_rows):
        for c in range(n_cols - 1):
            for term in horizontal[r][c]:
                horiz[r * (n_cols - 1) + c] += _mat(term.op, "horizontal").reshape(d2, d2)
                horiz_mask[r * (n_cols - 1) + c] = 1
    nv = max((n_rows - 1) * n_cols, 1)
    vert = np.zeros((nv, d2, d2), dtype=mdt)
    vert_mask = np.zeros(nv, dtype=np.int32)
    for r in range(n_rows - 1):
        for c in range(n_cols):
            for term in vertical[r][c]:
                vert[r * n_cols + c] += _mat(term.op, "vertical").reshape(d2, d2)
                vert_mask[r * n_cols + c] = 1
    nsites, site_off, sites, value_off, values = [], [], [], [], []
    for term in diagonal:
        ids = [int(r) * n_cols + int(c) for r, c in term.sites]
        table = _real(term.diag, "diagonal").reshape(-1)
        if table.shape[0] != d ** len(ids):
            raise ValueError("diagonal table must have d**n_sites entries")
        nsites.append(len(ids))
        site_off.append(len(sites))
        sites.extend(ids)
        value_off.append(len(values))
        values.extend(table.tolist())
    return LoweredOperator(
        onesite=onesite, onesite_mask=onesite_mask, horiz=horiz, horiz_mask=horiz_mask,
        vert=vert, vert_mask=vert_mask,
        diag_nsites=np.asarray(nsites, dtype=np.int32),
        diag_site_off=np.asarray(site_off, dtype=np.int32),
        diag_sites=np.asarray(sites, dtype=np.int32),
        diag_value_off=np.asarray(value_off, dtype=np.int32),
        diag_values=np.asarray(values, dtype=np.float64),
    )
