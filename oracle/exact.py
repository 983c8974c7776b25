"""Exact (no boundary-MPS) answers used to pin the oracle -- test infrastructure only.

* ``brute_amplitudes``: contracts the PEPS row by row keeping the FULL vector
  over the open vertical bonds -- a code path independent of the boundary-MPS
  machinery in ``oracle.peps``;
* ``apply_local_hamiltonian``: matrix-free action of a LocalHamiltonian on a
  dense wavefunction tensor, with the reference's local-energy convention
  (an off-diagonal term contributes ``op[p, s] * psi(s -> p)``, i.e. the
  column ``op[:, s]``; src/vmc/peps/common/energy.py:176-200);
* ``full_sum_energy_and_grad``: E = sum |psi|^2 E_loc / sum |psi|^2 and
  grad = sum w (E_loc - E) conj(O) as in tests/test_mc_energy_grad_evaluator.py:58-73.
"""
from __future__ import annotations

import itertools
import string

import numpy as np


def all_configs(n_sites: int, d: int = 2) -> np.ndarray:
    """All d^n occupancy configurations, site 0 most significant (row-major sites)."""
    return np.array(list(itertools.product(range(d), repeat=n_sites)), dtype=np.int64)


def brute_amplitudes(tensors, configs, shape) -> np.ndarray:
    """Exact amplitudes of configs[z, n_sites] by full row-transfer contraction."""
    n_rows, n_cols = shape
    z = configs.shape[0]
    spins = configs.reshape(z, n_rows, n_cols)
    dtype = np.result_type(*[np.asarray(t).dtype for row in tensors for t in row])
    letters = string.ascii_letters
    # state axes: z, then one leg per column (down legs of the previous row).
    state = np.ones((z,) + (1,) * n_cols, dtype=dtype)
    for r in range(n_rows):
        # Carry a horizontal bond h while sweeping the row left to right.
        state = state[..., None]  # trailing horizontal bond of dim 1
        for c in range(n_cols):
            a = np.asarray(tensors[r][c])[spins[:, r, c]]  # (z, up, down, left, right)
            legs = list(letters[:n_cols])
            h, u, dn, rt = "H", legs[c], "D", "R"
            src = "z" + "".join(legs) + h
            out_legs = legs.copy()
            out_legs[c] = dn
            dst = "z" + "".join(out_legs) + rt
            state = np.einsum(f"{src},z{u}{dn}{h}{rt}->{dst}", state, a)
        state = state[..., 0]
    return state.reshape(z)


def apply_local_hamiltonian(psi: np.ndarray, terms, shape, d: int) -> np.ndarray:
    """(M psi)(s) = sum_terms sum_p op[p, s_local] psi(s with the term's sites set to p)."""
    n_rows, n_cols = shape
    n = n_rows * n_cols
    psi = psi.reshape((d,) * n)
    out = np.zeros(psi.shape, dtype=np.result_type(psi.dtype, np.complex128
                                                    if any(np.iscomplexobj(getattr(t, "op", getattr(t, "diag", 0)))
                                                           for t in terms) else psi.dtype))
    letters = string.ascii_letters[:n]

    def site(rc):
        return rc[0] * n_cols + rc[1]

    for term in terms:
        kind = type(term).__name__
        if kind == "DiagonalTerm":
            idx = [site(rc) for rc in term.sites]
            diag = np.asarray(term.diag).reshape((d,) * len(idx))
            # broadcast the diagonal over the other sites
            sub_in = "".join(letters[i] for i in idx)
            out = out + np.einsum(f"{sub_in},{letters}->{letters}", diag, psi)
        elif kind in ("OneSiteTerm", "HorizontalTwoSiteTerm", "VerticalTwoSiteTerm"):
            idx = [site(rc) for rc in term.sites]
            k = len(idx)
            op = np.asarray(term.op).reshape((d,) * (2 * k))  # op[p..., s...]
            p_letters = string.ascii_uppercase[:k]
            src = list(letters)
            for j, i in enumerate(idx):
                src[i] = p_letters[j]
            s_letters = "".join(letters[i] for i in idx)
            out = out + np.einsum(f"{''.join(p_letters)}{s_letters},{''.join(src)}->{letters}", op, psi)
        else:
            raise TypeError(f"unsupported term {kind}")
    return out.reshape(-1)


def full_sum_energy_and_grad(amps, o_full, e_loc, rel_mask=1e-12):
    """tests/test_mc_energy_grad_evaluator.py:58-73 (mask relative to the largest weight)."""
    weights = np.abs(amps) ** 2
    mask = weights > rel_mask * weights.max()
    w = weights[mask] / weights[mask].sum()
    energy = np.sum(w * e_loc[mask])
    grad = np.sum(w[:, None] * (e_loc[mask] - energy)[:, None] * o_full[mask].conj(), axis=0)
    return energy, grad
