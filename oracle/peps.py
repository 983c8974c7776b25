"""FP64 NumPy restatement of the reference PEPS evaluation path (oracle; test infrastructure only).

Everything is batched over a leading sample/chain axis ``z`` -- the reference
``jax.vmap``s its per-chain kernels over chains (src/vmc/core/sampling.py:38);
here the same per-chain algebra runs on stacked arrays.  Site tensors are
shared (unbatched) ``tensors[r][c]`` of shape (d, up, down, left, right)
(src/vmc/peps/standard/model.py:27-74); boundary-MPS tensors are
(z, left, phys, right); row-MPO tensors are (z, wl, wr, pin, pout)
(src/vmc/peps/common/contraction.py:22-27).

Randomness is explicit: the transition consumes one uniform per site per
sweep (and, for d>2, one flip offset in [1, d) per site) in the order the
reference draws them (src/vmc/peps/standard/kernels.py:166-190).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, NamedTuple

import numpy as np

__all__ = [
    "NoTruncation", "ZipUp", "DensityMatrix", "Variational",
    "PEPS", "LocalHamiltonianView", "bucket_terms",
    "build_row_mpo", "contract_bottom", "forward_with_cache", "apply_mpo_from_below",
    "compute_right_envs", "metropolis_ratio",
    "compute_all_env_grads_and_energy", "compute_all_gradients",
    "build_mc_kernels", "make_mc_sampler", "sample_counts", "trim_samples",
    "value", "value_and_grad", "local_estimate", "spin_to_occupancy",
    "params_per_site", "sliced_dims",
]


def _ein(subscripts: str, *operands, path=None):
    if path is None:
        return np.einsum(subscripts, *operands, optimize=True)
    return np.einsum(subscripts, *operands, optimize=["einsum_path", *path])


def _ones(batch: int, ndim: int, dtype) -> np.ndarray:
    return np.ones((batch,) + (1,) * ndim, dtype=dtype)


# --------------------------------------------------------------------------- #
# Strategies  (src/vmc/peps/common/strategy.py)
# --------------------------------------------------------------------------- #


class ContractionStrategy:
    """strategy.py:25-41."""

    def __init__(self, truncate_bond_dimension: int):
        self.truncate_bond_dimension = int(truncate_bond_dimension)

    def apply(self, mps, mpo):  # pragma: no cover - abstract
        raise NotImplementedError


class NoTruncation(ContractionStrategy):
    """strategy.py:44-51."""

    def __init__(self):
        super().__init__(1)

    def apply(self, mps, mpo):
        return apply_mpo_exact(mps, mpo)


class ZipUp(ContractionStrategy):
    """strategy.py:54-61."""

    def apply(self, mps, mpo):
        return apply_mpo_zip_up(mps, mpo, self.truncate_bond_dimension)


class DensityMatrix(ContractionStrategy):
    """strategy.py:64-71."""

    def apply(self, mps, mpo):
        return apply_mpo_density_matrix(mps, mpo, self.truncate_bond_dimension)


class Variational(ContractionStrategy):
    """strategy.py:74-92."""

    def __init__(self, truncate_bond_dimension: int, n_sweeps: int = 2):
        super().__init__(truncate_bond_dimension)
        self.n_sweeps = int(n_sweeps)

    def apply(self, mps, mpo):
        return apply_mpo_variational(mps, mpo, self.truncate_bond_dimension, self.n_sweeps)


def contract_theta(m, w, carry):
    """strategy.py:95-115: theta = carry . m . w -> (z, left, phys, Dr, wr)."""
    if carry is not None:
        theta = _ein("zkdl,zdpr,zlwpq->zkqrw", carry, m, w, path=[(0, 1), (0, 1)])
        return theta, theta.shape[1], theta.shape[2], theta.shape[3], theta.shape[4]
    theta = _ein("zdpr,zlwpq->zdlqrw", m, w)
    z, dl, wl, q, dr, wr = theta.shape
    return theta.reshape(z, dl * wl, q, dr, wr), dl * wl, q, dr, wr


def apply_mpo_exact(mps, mpo):
    """strategy.py:118-125 (bonds multiply, no truncation)."""
    out = []
    for m, w in zip(mps, mpo):
        t = _ein("zdpr,zlwpq->zdlqrw", m, w)
        z, dl, wl, q, dr, wr = t.shape
        out.append(t.reshape(z, dl * wl, q, dr * wr))
    return tuple(out)


def apply_mpo_zip_up(mps, mpo, chi: int):
    """strategy.py:128-150: SVD-truncated zip-up; the last site is untruncated."""
    new, carry = [], None
    n = len(mps)
    for i, (m, w) in enumerate(zip(mps, mpo)):
        theta, left, phys, dr, wr = contract_theta(m, w, carry)
        z = theta.shape[0]
        if i == n - 1:
            new.append(theta.reshape(z, left, phys, dr * wr))
            break
        mat = theta.reshape(z, left * phys, dr * wr)
        u, s, vh = np.linalg.svd(mat, full_matrices=False)
        k = min(chi, s.shape[-1])
        new.append(u[..., :k].reshape(z, left, phys, k))
        carry = (s[..., :k, None].astype(vh.dtype) * vh[..., :k, :]).reshape(z, k, dr, wr)
    return tuple(new)


def apply_mpo_density_matrix(mps, mpo, chi: int):
    """strategy.py:153-176: rho = theta^H theta, keep the top-k eigenvectors."""
    new, carry = [], None
    n = len(mps)
    for i, (m, w) in enumerate(zip(mps, mpo)):
        theta, left, phys, dr, wr = contract_theta(m, w, carry)
        z = theta.shape[0]
        mat = theta.reshape(z, left * phys, dr * wr)
        if i == n - 1:
            new.append(mat.reshape(z, left, phys, dr * wr))
            break
        rho = np.swapaxes(mat.conj(), -1, -2) @ mat
        evals, evecs = np.linalg.eigh(rho)
        k = min(chi, rho.shape[-1])
        order = np.argsort(evals, axis=-1, kind="stable")[..., ::-1][..., :k]
        vecs_k = np.take_along_axis(evecs, order[:, None, :], axis=-1)
        new.append((mat @ vecs_k).reshape(z, left, phys, k))
        carry = np.swapaxes(vecs_k.conj(), -1, -2).reshape(z, k, dr, wr)
    return tuple(new)


def _qr(a):
    """src/vmc/utils/factorizations.py:9-16: reduced Householder QR (geqrf)."""
    return np.linalg.qr(a, mode="reduced")


def _init_compressed_mps(mps, mpo, dc: int):
    """strategy.py:222-254: left-canonical QR initialisation capped at Dc."""
    result, carry = [], None
    n = len(mps)
    for i, (m, w) in enumerate(zip(mps, mpo)):
        theta, left, phys, dr, wr = contract_theta(m, w, carry)
        z = theta.shape[0]
        if i == n - 1:
            result.append(theta.reshape(z, left, phys, dr * wr))
            break
        q, r = _qr(theta.reshape(z, left * phys, dr * wr))
        k = min(dc, q.shape[-1])
        result.append(q[..., :k].reshape(z, left, phys, k))
        carry = r[..., :k, :].reshape(z, k, dr, wr)
    return result


_ENV_PATH = [(1, 0), (2, 0), (1, 0)]


def _build_right_envs(mps, mpo, result, dtype):
    """strategy.py:257-289."""
    n = len(mps)
    z = mps[0].shape[0]
    envs = [None] * n
    r_env = _ones(z, 3, dtype)
    envs[n - 1] = r_env
    for i in range(n - 2, -1, -1):
        r_env = _ein("zaqb,zrwb,zlwpq,zdpr->zdla", result[i + 1].conj(), r_env,
                     mpo[i + 1], mps[i + 1], path=_ENV_PATH)
        envs[i] = r_env
    return envs


def _variational_sweep_lr(mps, mpo, result, right_envs, dtype):
    """strategy.py:292-356."""
    n = len(mps)
    z = mps[0].shape[0]
    new = list(result)
    left_envs = [None] * n
    l_env = _ones(z, 3, dtype)
    for i in range(n):
        left_envs[i] = l_env
        m, w, r_env = mps[i], mpo[i], right_envs[i]
        optimal = _ein("zdpr,zdla,zlwpq,zrwb->zaqb", m, l_env, w, r_env, path=_ENV_PATH)
        if i == n - 1:
            new[i] = optimal
            break
        _, left, phys, right = optimal.shape
        a, c = _qr(optimal.reshape(z, left * phys, right))
        tensor = a.reshape(z, left, phys, a.shape[-1])
        new[i] = tensor
        new[i + 1] = _ein("zab,zbpr->zapr", c, new[i + 1])
        l_env = _ein("zdpr,zdla,zlwpq,zaqb->zrwb", m, l_env, w, tensor.conj(), path=_ENV_PATH)
    return new, left_envs


def _variational_sweep_rl(mps, mpo, result, left_envs, dtype):
    """strategy.py:359-427 (LQ through QR of the transpose)."""
    n = len(mps)
    z = mps[0].shape[0]
    new = list(result)
    right_envs = [None] * n
    r_env = _ones(z, 3, dtype)
    for i in range(n - 1, -1, -1):
        right_envs[i] = r_env
        m, w, l_env = mps[i], mpo[i], left_envs[i]
        optimal = _ein("zdpr,zdla,zlwpq,zrwb->zaqb", m, l_env, w, r_env, path=_ENV_PATH)
        if i == 0:
            new[i] = optimal
            break
        _, left, phys, right = optimal.shape
        q_t, r_t = _qr(np.swapaxes(optimal.reshape(z, left, phys * right), -1, -2))
        b = np.swapaxes(q_t, -1, -2)
        c = np.swapaxes(r_t, -1, -2)
        tensor = b.reshape(z, b.shape[1], phys, right)
        new[i] = tensor
        new[i - 1] = _ein("zlpr,zrb->zlpb", new[i - 1], c)
        r_env = _ein("zaqb,zrwb,zlwpq,zdpr->zdla", tensor.conj(), r_env, w, m, path=_ENV_PATH)
    return new, right_envs


def apply_mpo_variational(mps, mpo, dc: int, n_sweeps: int = 2):
    """strategy.py:179-219."""
    dtype = mps[0].dtype
    result = _init_compressed_mps(mps, mpo, dc)
    right_envs = _build_right_envs(mps, mpo, result, dtype)
    for _ in range(n_sweeps):
        result, left_envs = _variational_sweep_lr(mps, mpo, result, right_envs, dtype)
        result, right_envs = _variational_sweep_rl(mps, mpo, result, left_envs, dtype)
    return tuple(result)


# --------------------------------------------------------------------------- #
# Model container and operator bucketing
# --------------------------------------------------------------------------- #


class PEPS:
    """Parameter container mirroring src/vmc/peps/standard/model.py:22-98.

    Tensors are supplied by the caller (seeded synthetic inputs), not drawn
    from the reference's uniform initialiser.
    """

    def __init__(self, tensors, shape, bond_dim, phys_dim=2, strategy=None):
        self.tensors = [[np.asarray(t) for t in row] for row in tensors]
        self.shape = (int(shape[0]), int(shape[1]))
        self.bond_dim = int(bond_dim)
        self.phys_dim = int(phys_dim)
        self.strategy = strategy if strategy is not None else Variational(bond_dim * bond_dim)

    @staticmethod
    def site_dims(row, col, n_rows, n_cols, bond_dim):
        """model.py:27-35."""
        up = 1 if row == 0 else bond_dim
        down = 1 if row == n_rows - 1 else bond_dim
        left = 1 if col == 0 else bond_dim
        right = 1 if col == n_cols - 1 else bond_dim
        return up, down, left, right


def params_per_site(model) -> list[int]:
    """src/vmc/utils/smallo.py:23-35."""
    n_rows, n_cols = model.shape
    out = []
    for r in range(n_rows):
        for c in range(n_cols):
            u, d, l, rr = PEPS.site_dims(r, c, n_rows, n_cols, model.bond_dim)
            out.append(u * d * l * rr)
    return out


def sliced_dims(model) -> tuple[int, ...]:
    """src/vmc/utils/smallo.py:38-42."""
    return (model.phys_dim,) * (model.shape[0] * model.shape[1])


@dataclass
class LocalHamiltonianView:
    shape: tuple
    terms: tuple = ()


def bucket_terms(terms, shape):
    """src/vmc/operators/local_terms.py:165-200 (dispatch on the term class name)."""
    n_rows, n_cols = shape
    one_site = [[[] for _ in range(n_cols)] for _ in range(n_rows)]
    horizontal = [[[] for _ in range(max(n_cols - 1, 0))] for _ in range(n_rows)]
    vertical = [[[] for _ in range(n_cols)] for _ in range(max(n_rows - 1, 0))]
    plaquette = [[[] for _ in range(max(n_cols - 1, 0))] for _ in range(max(n_rows - 1, 0))]
    diagonal = []
    for term in terms:
        kind = type(term).__name__
        if kind == "OneSiteTerm":
            one_site[term.row][term.col].append(term)
        elif kind == "HorizontalTwoSiteTerm":
            horizontal[term.row][term.col].append(term)
        elif kind == "VerticalTwoSiteTerm":
            vertical[term.row][term.col].append(term)
        elif kind == "DiagonalTerm":
            diagonal.append(term)
        elif kind == "PlaquetteTerm":
            plaquette[term.row][term.col].append(term)
        else:
            raise TypeError(f"Unsupported term type: {type(term)!r}")
    return diagonal, one_site, horizontal, vertical, plaquette


# --------------------------------------------------------------------------- #
# Contraction primitives  (src/vmc/peps/common/contraction.py)
# --------------------------------------------------------------------------- #


def build_row_mpo(tensors, spins_row, row):
    """contraction.py:22-27: gather A[s] and transpose (u,d,l,r)->(l,r,u,d)."""
    return tuple(
        np.transpose(np.asarray(tensors[row][c])[spins_row[:, c]], (0, 3, 4, 1, 2))
        for c in range(spins_row.shape[1])
    )


def contract_bottom(mps):
    """contraction.py:30-35."""
    z = mps[0].shape[0]
    state = np.ones((z, 1), dtype=mps[0].dtype)
    for site in mps:
        state = np.einsum("za,zab->zb", state, site[:, :, 0, :])
    return state[:, 0]


def forward_with_cache(tensors, spins, shape, strategy):
    """contraction.py:38-56."""
    n_rows, n_cols = shape
    dtype = np.asarray(tensors[0][0]).dtype
    z = spins.shape[0]
    top_envs = [None] * n_rows
    boundary = tuple(_ones(z, 3, dtype) for _ in range(n_cols))
    for row in range(n_rows):
        top_envs[row] = boundary
        boundary = strategy.apply(boundary, build_row_mpo(tensors, spins[:, row], row))
    return contract_bottom(boundary), top_envs


def apply_mpo_from_below(bottom_mps, mpo, strategy):
    """contraction.py:59-65: swap pin/pout and apply from below."""
    return strategy.apply(bottom_mps, tuple(np.swapaxes(w, 3, 4) for w in mpo))


def compute_right_envs(top_env, mpo_row, bottom_env, dtype):
    """contraction.py:68-86."""
    n = len(mpo_row)
    z = mpo_row[0].shape[0]
    envs = [None] * n
    envs[n - 1] = _ones(z, 3, dtype)
    for c in range(n - 2, -1, -1):
        envs[c] = _ein("zaub,zcduv,zevf,zbdf->zace", top_env[c + 1], mpo_row[c + 1],
                       bottom_env[c + 1], envs[c + 1], path=[(0, 3), (0, 2), (0, 1)])
    return envs


def metropolis_ratio(prob_cur, prob_flip):
    """contraction.py:88-94."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(prob_cur > 0.0, prob_flip / np.where(prob_cur > 0.0, prob_cur, 1.0),
                        np.where(prob_flip > 0.0, np.inf, 0.0))


# --------------------------------------------------------------------------- #
# Energy and gradients  (src/vmc/peps/common/energy.py)
# --------------------------------------------------------------------------- #


def compute_right_envs_2row(top_env, mpo0, mpo1, bottom_env, dtype):
    """energy.py:24-44."""
    n = len(mpo0)
    z = mpo0[0].shape[0]
    envs = [None] * n
    envs[n - 1] = _ones(z, 4, dtype)
    for c in range(n - 2, -1, -1):
        envs[c] = _ein("zaub,zlruv,zxyvw,zewf,zbryf->zalxe", top_env[c + 1], mpo0[c + 1],
                       mpo1[c + 1], bottom_env[c + 1], envs[c + 1],
                       path=[(0, 4), (0, 3), (0, 2), (0, 1)])
    return envs


def _apply_op_column(op, col_idx, amps_flat, amp):
    """sum_j op[j, col_idx] * amps[j] / amp -- the reference's jnp.dot(op[:, idx], amps) / amp."""
    op = np.asarray(op)
    return np.sum(op[:, col_idx].T * amps_flat, axis=1) / amp


def compute_row_pair_vertical_energy(top_mps, bottom_mps, mpo0, mpo1, tensors0, tensors1,
                                     spins0, spins1, terms_row, amp, phys_dim):
    """energy.py:47-95."""
    z = amp.shape[0]
    if not any(terms_row):
        return np.zeros(z, dtype=amp.dtype)
    n = len(mpo0)
    dtype = mpo0[0].dtype
    right = compute_right_envs_2row(top_mps, mpo0, mpo1, bottom_mps, dtype)
    left = _ones(z, 4, dtype)
    energy = np.zeros(z, dtype=amp.dtype)
    for c in range(n):
        if terms_row[c]:
            amps_edge = _ein("zalmg,zaub,puvlr,qvwmn,zgwf,zbrnf->zpq", left, top_mps[c],
                             tensors0[c], tensors1[c], bottom_mps[c], right[c],
                             path=[(0, 1), (2, 3), (0, 2), (1, 2), (0, 1)])
            col_idx = spins0[:, c] * phys_dim + spins1[:, c]
            flat = amps_edge.reshape(z, -1)
            for term in terms_row[c]:
                energy = energy + _apply_op_column(term.op, col_idx, flat, amp)
        left = _ein("zalxe,zaub,zlruv,zxyvw,zewf->zbryf", left, top_mps[c], mpo0[c], mpo1[c],
                    bottom_mps[c], path=[(0, 1), (0, 3), (0, 2), (0, 1)])
    return energy


def compute_single_gradient(left_env, right_env, top_tensor, bot_tensor):
    """energy.py:259-273: dpsi/dA[s] as (z, up, down, left, right)."""
    g = _ein("zace,zaub,zevf,zbdf->zcuvd", left_env, top_tensor, bot_tensor, right_env,
             path=[(0, 1), (0, 1), (0, 1)])
    return np.transpose(g, (0, 2, 3, 1, 4))


def _left_update(left_env, top, mpo, bot):
    return _ein("zace,zaub,zcduv,zevf->zbdf", left_env, top, mpo, bot,
                path=[(0, 1), (0, 2), (0, 1)])


def compute_all_row_gradients(top_mps, bottom_mps, mpo):
    """energy.py:98-120."""
    dtype = mpo[0].dtype
    z = mpo[0].shape[0]
    right = compute_right_envs(top_mps, mpo, bottom_mps, dtype)
    grads = []
    left = _ones(z, 3, dtype)
    for c in range(len(mpo)):
        grads.append(compute_single_gradient(left, right[c], top_mps[c], bottom_mps[c]))
        left = _left_update(left, top_mps[c], mpo[c], bottom_mps[c])
    return grads


def compute_all_env_grads_and_energy(tensors, spins, amp, shape, strategy, top_envs, *,
                                     diagonal_terms, one_site_terms, horizontal_terms,
                                     vertical_terms, collect_grads=True):
    """energy.py:123-224: bottom->top pass reusing the transition's top envs."""
    n_rows, n_cols = shape
    dtype = np.asarray(tensors[0][0]).dtype
    phys_dim = int(np.asarray(tensors[0][0]).shape[0])
    z = spins.shape[0]
    env_grads = [[None] * n_cols for _ in range(n_rows)] if collect_grads else []
    bottom_cache = [None] * n_rows
    energy = np.zeros(z, dtype=np.result_type(amp.dtype, dtype))

    for term in diagonal_terms:
        idx = np.zeros(z, dtype=np.int64)
        for r, c in term.sites:
            idx = idx * phys_dim + spins[:, r, c]
        energy = energy + np.asarray(term.diag)[idx]

    bottom_env = tuple(_ones(z, 3, dtype) for _ in range(n_cols))
    next_row_mpo = None
    for row in range(n_rows - 1, -1, -1):
        bottom_cache[row] = bottom_env
        top_env = top_envs[row]
        mpo = build_row_mpo(tensors, spins[:, row], row)
        right = compute_right_envs(top_env, mpo, bottom_env, dtype)
        left = _ones(z, 3, dtype)
        for c in range(n_cols):
            site_terms = one_site_terms[row][c]
            if collect_grads or site_terms:
                env_grad = compute_single_gradient(left, right[c], top_env[c], bottom_env[c])
                if collect_grads:
                    env_grads[row][c] = env_grad
                if site_terms:
                    amps_site = _ein("pudlr,zudlr->zp", tensors[row][c], env_grad)
                    for term in site_terms:
                        energy = energy + _apply_op_column(term.op, spins[:, row, c], amps_site, amp)
            if c < n_cols - 1 and horizontal_terms[row][c]:
                amps_edge = _ein(
                    "zace,zaub,zedf,pudcr,qvwrx,zbvg,zfwi,zgxi->zpq",
                    left, top_env[c], bottom_env[c], tensors[row][c], tensors[row][c + 1],
                    top_env[c + 1], bottom_env[c + 1], right[c + 1],
                    path=[(0, 1), (1, 6), (0, 5), (1, 3), (1, 2), (1, 2), (0, 1)],
                )
                col_idx = spins[:, row, c] * phys_dim + spins[:, row, c + 1]
                flat = amps_edge.reshape(z, -1)
                for term in horizontal_terms[row][c]:
                    energy = energy + _apply_op_column(term.op, col_idx, flat, amp)
            left = _left_update(left, top_env[c], mpo[c], bottom_env[c])
        if row < n_rows - 1:
            energy = energy + compute_row_pair_vertical_energy(
                top_env, bottom_cache[row + 1], mpo, next_row_mpo, tensors[row],
                tensors[row + 1], spins[:, row], spins[:, row + 1], vertical_terms[row],
                amp, phys_dim)
        bottom_env = apply_mpo_from_below(bottom_env, mpo, strategy)
        next_row_mpo = mpo
    return env_grads, energy, bottom_cache


def compute_all_gradients(tensors, spins, shape, strategy, top_envs):
    """energy.py:276-301."""
    n_rows, n_cols = shape
    dtype = np.asarray(tensors[0][0]).dtype
    z = spins.shape[0]
    grads = [None] * n_rows
    bottom_env = tuple(_ones(z, 3, dtype) for _ in range(n_cols))
    for row in range(n_rows - 1, -1, -1):
        mpo = build_row_mpo(tensors, spins[:, row], row)
        grads[row] = compute_all_row_gradients(top_envs[row], bottom_env, mpo)
        bottom_env = apply_mpo_from_below(bottom_env, mpo, strategy)
    return grads


# --------------------------------------------------------------------------- #
# MC kernels  (src/vmc/peps/standard/kernels.py)
# --------------------------------------------------------------------------- #


class Cache(NamedTuple):
    """kernels.py:32-35."""
    bottom_envs: Any


class Context(NamedTuple):
    """kernels.py:38-42 (plus the per-site acceptance margins used for flagging)."""
    amp: np.ndarray
    top_envs: Any
    margins: np.ndarray | None = None


class LocalEstimates(NamedTuple):
    """kernels.py:45-51."""
    local_log_derivatives: np.ndarray
    local_estimate: np.ndarray
    active_slice_indices: np.ndarray | None
    amp: np.ndarray | None = None


def assemble_log_derivatives(tensors, pps, shape, env_grads, config, amp, *, full_gradient):
    """kernels.py:54-88."""
    n_rows, n_cols = shape
    z = config.shape[0]
    cfg = config.reshape(z, n_rows, n_cols)
    if full_gradient:
        parts = []
        for r in range(n_rows):
            for c in range(n_cols):
                full = np.zeros((z,) + np.asarray(tensors[r][c]).shape,
                                dtype=np.result_type(env_grads[r][c].dtype, tensors[r][c].dtype))
                full[np.arange(z), cfg[:, r, c]] = env_grads[r][c]
                parts.append(full.reshape(z, -1))
        return np.concatenate(parts, axis=1) / amp[:, None], None
    parts = [env_grads[r][c].reshape(z, -1) for r in range(n_rows) for c in range(n_cols)]
    p = np.repeat(config.astype(np.int8), pps, axis=1)
    return np.concatenate(parts, axis=1) / amp[:, None], p


def build_mc_kernels(model, operator, *, full_gradient=False):
    """kernels.py:91-247, batched over chains.

    Returns ``(init_cache, transition, estimate)`` where
    ``transition(tensors, configs[z, n_sites], uniforms[z, n_sites], cache, deltas=None)``
    replaces the reference's per-chain key with explicit per-site draws.
    """
    shape = model.shape
    n_rows, n_cols = shape
    n_sites = n_rows * n_cols
    strategy = model.strategy
    pps = params_per_site(model)
    diagonal, one_site, horizontal, vertical, _ = bucket_terms(operator.terms, shape)

    def init_cache(tensors, config_states):
        """kernels.py:115-129."""
        z = config_states.shape[0]
        idx = config_states.reshape(z, n_rows, n_cols)
        dtype = np.asarray(tensors[0][0]).dtype
        envs = [None] * n_rows
        env = tuple(_ones(z, 3, dtype) for _ in range(n_cols))
        for row in range(n_rows - 1, -1, -1):
            envs[row] = env
            env = apply_mpo_from_below(env, build_row_mpo(tensors, idx[:, row], row), strategy)
        return Cache(bottom_envs=tuple(envs))

    def transition(tensors, config_state, uniforms, cache, deltas=None):
        """kernels.py:131-209 with the per-site uniform U[site] and flip offset explicit."""
        z = config_state.shape[0]
        idx = np.array(config_state, dtype=np.int64).reshape(z, n_rows, n_cols)
        dtype = np.asarray(tensors[0][0]).dtype
        top_env = tuple(_ones(z, 3, dtype) for _ in range(n_cols))
        top_cache = [None] * n_rows
        margins = np.zeros((z, n_sites))
        for row in range(n_rows):
            top_cache[row] = top_env
            bottom_env = cache.bottom_envs[row]
            mpo_row = build_row_mpo(tensors, idx[:, row], row)
            right = compute_right_envs(top_env, mpo_row, bottom_env, dtype)
            left = _ones(z, 3, dtype)
            amp_cur = _ein("zace,zaub,zcduv,zevf,zbdf->z", left, top_env[0], mpo_row[0],
                           bottom_env[0], right[0], path=[(0, 1), (1, 2), (1, 2), (0, 1)])
            updated = []
            for col in range(n_cols):
                site = np.asarray(tensors[row][col])
                d = site.shape[0]
                cur = idx[:, row, col]
                if d == 1:
                    flip = cur
                elif d == 2:
                    flip = 1 - cur
                else:
                    flip = (cur + deltas[:, row * n_cols + col]) % d
                mpo_cur = mpo_row[col]
                mpo_flip = np.transpose(site[flip], (0, 3, 4, 1, 2))
                amp_flip = _ein("zace,zaub,zcduv,zevf,zbdf->z", left, top_env[col], mpo_flip,
                                bottom_env[col], right[col], path=[(0, 1), (1, 2), (1, 2), (0, 1)])
                ratio = metropolis_ratio(np.abs(amp_cur) ** 2, np.abs(amp_flip) ** 2)
                u = uniforms[:, row * n_cols + col]
                threshold = np.minimum(1.0, ratio)
                margins[:, row * n_cols + col] = np.abs(threshold - u)
                accept = u < threshold
                idx[:, row, col] = np.where(accept, flip, cur)
                amp_cur = np.where(accept, amp_flip, amp_cur)
                mpo_sel = np.where(accept[:, None, None, None, None], mpo_flip, mpo_cur)
                updated.append(mpo_sel)
                left = _left_update(left, top_env[col], mpo_sel, bottom_env[col])
            top_env = strategy.apply(top_env, tuple(updated))
        amp = contract_bottom(top_env)
        return idx.reshape(z, -1), Context(amp=amp, top_envs=tuple(top_cache), margins=margins)

    def estimate(tensors, config_state_next, context):
        """kernels.py:211-245."""
        z = config_state_next.shape[0]
        idx = config_state_next.reshape(z, n_rows, n_cols)
        env_grads, e_loc, bottom_next = compute_all_env_grads_and_energy(
            tensors, idx, context.amp, shape, strategy, context.top_envs,
            diagonal_terms=diagonal, one_site_terms=one_site, horizontal_terms=horizontal,
            vertical_terms=vertical, collect_grads=True)
        o, p = assemble_log_derivatives(tensors, pps, shape, env_grads, config_state_next,
                                        context.amp, full_gradient=full_gradient)
        return Cache(bottom_envs=tuple(bottom_next)), LocalEstimates(
            local_log_derivatives=o, local_estimate=e_loc, active_slice_indices=p,
            amp=context.amp)

    return init_cache, transition, estimate


def make_mc_sampler(transition, estimate):
    """src/vmc/core/sampling.py:22-64 with explicit draws: uniforms[n_steps, z, n_sites]."""

    def mc_sampler(tensors, config_states, uniforms, cache, *, n_steps, deltas=None):
        configs = config_states
        hist_cfg, hist_est, hist_margin = [], [], []
        for step in range(n_steps):
            configs, ctx = transition(tensors, configs, uniforms[step], cache,
                                      None if deltas is None else deltas[step])
            cache, est = estimate(tensors, configs, ctx)
            hist_cfg.append(configs)
            hist_est.append(est)
            hist_margin.append(ctx.margins)
        stacked = LocalEstimates(
            local_log_derivatives=np.stack([e.local_log_derivatives for e in hist_est]),
            local_estimate=np.stack([e.local_estimate for e in hist_est]),
            active_slice_indices=(None if hist_est[0].active_slice_indices is None
                                  else np.stack([e.active_slice_indices for e in hist_est])),
            amp=np.stack([e.amp for e in hist_est]),
        )
        return (configs, cache), (np.stack(hist_cfg), stacked, np.stack(hist_margin))

    return mc_sampler


def sample_counts(n_samples, n_chains):
    """src/vmc/core/sampling.py:76-78."""
    chain_length = -(-n_samples // n_chains)
    return n_samples, n_chains, chain_length, chain_length * n_chains


def trim_samples(samples, total_samples, num_samples):
    """src/vmc/core/sampling.py:81-82."""
    return samples.reshape((total_samples,) + samples.shape[2:])[:num_samples]


# --------------------------------------------------------------------------- #
# Compatibility evaluators  (src/vmc/peps/standard/compat.py)
# --------------------------------------------------------------------------- #


def spin_to_occupancy(spins):
    """src/vmc/utils/utils.py:55-57."""
    return ((np.asarray(spins) + 1) // 2).astype(np.int64)


def peps_apply(tensors, samples, shape, strategy):
    """compat.py:31-40 (batched)."""
    z = samples.shape[0]
    spins = spin_to_occupancy(samples).reshape(z, *shape)
    amp, _ = forward_with_cache(tensors, spins, shape, strategy)
    return amp


def value(model, samples):
    """compat.py:67-78."""
    return peps_apply(model.tensors, np.atleast_2d(samples), model.shape, model.strategy)


def value_and_grad(model, samples, *, full_gradient=False):
    """compat.py:94-133 (full_gradient scatters the same hand-written adjoint).  Samples pass through
    spin_to_occupancy as in compat.py:119, which maps +-1 spins to 0/1 and, for d > 2, occupancy 2 to 1."""
    samples = np.atleast_2d(samples)
    return value_and_grad_occupancy(model, spin_to_occupancy(samples), full_gradient=full_gradient)


def value_and_grad_occupancy(model, occupancies, *, full_gradient=False):
    """The amplitudes and dpsi/dA of configurations given as occupancies 0..d-1, the convention of the
    sampler kernels (kernels.py:54-88 index the site tensors with the configuration as given)."""
    occupancies = np.atleast_2d(occupancies)
    z = occupancies.shape[0]
    n_rows, n_cols = model.shape
    spins = np.asarray(occupancies, dtype=np.int64).reshape(z, n_rows, n_cols)
    amp, top_envs = forward_with_cache(model.tensors, spins, model.shape, model.strategy)
    env_grads = compute_all_gradients(model.tensors, spins, model.shape, model.strategy, top_envs)
    if full_gradient:
        parts = []
        for r in range(n_rows):
            for c in range(n_cols):
                t = model.tensors[r][c]
                full = np.zeros((z,) + t.shape, dtype=np.result_type(t.dtype, env_grads[r][c].dtype))
                full[np.arange(z), spins[:, r, c]] = env_grads[r][c]
                parts.append(full.reshape(z, -1))
        return amp, np.concatenate(parts, axis=1), None
    grads = np.concatenate([env_grads[r][c].reshape(z, -1)
                            for r in range(n_rows) for c in range(n_cols)], axis=1)
    p = np.repeat(spins.reshape(z, -1).astype(np.int8), params_per_site(model), axis=1)
    return amp, grads, p


def local_estimate(model, samples, operator, amps):
    """compat.py:136-194 (samples through spin_to_occupancy, as compat.py:162)."""
    return local_estimate_occupancy(model, spin_to_occupancy(np.atleast_2d(samples)), operator, amps)


def local_estimate_occupancy(model, occupancies, operator, amps):
    """E_loc of configurations given as occupancies 0..d-1 (the sampler kernels' convention)."""
    samples = np.atleast_2d(occupancies)
    z = samples.shape[0]
    shape = model.shape
    diagonal, one_site, horizontal, vertical, _ = bucket_terms(operator.terms, shape)
    spins = np.asarray(samples, dtype=np.int64).reshape(z, *shape)
    _, top_envs = forward_with_cache(model.tensors, spins, shape, model.strategy)
    _, energy, _ = compute_all_env_grads_and_energy(
        model.tensors, spins, np.asarray(amps), shape, model.strategy, top_envs,
        diagonal_terms=diagonal, one_site_terms=one_site, horizontal_terms=horizontal,
        vertical_terms=vertical, collect_grads=False)
    return energy
