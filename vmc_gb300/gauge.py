"""Gauge removal for the SR solve (API of src/vmc/gauge/gauge.py:16-37 and weight.py:13-26).

A PEPS is unchanged when an invertible matrix X is inserted on an internal bond, A_a -> A_a X on one
leg and A_b -> X^-1 A_b on the other.  To first order, X = 1 + eps T with T = E_ij (i, j < D) moves the
parameters along

    dA_a = A_a E_ij  (the bond leg of A_a: its slice i moves to position j)
    dA_b = -E_ij A_b (the bond leg of A_b: its slice j moves to position i, negated),

D^2 directions per internal bond, along which log psi does not change; with
``include_global_scale`` the direction theta itself (psi scales by (1 + eps)^n_sites, so the centred
log-derivative does not change either) joins them.  These directions are null (or, under boundary-MPS
truncation, nearly null) directions of the quantum geometric tensor S.  Gauge removal solves the SR
system in their orthogonal complement: with Q an orthonormal basis of that complement, the reference's
SR step (src/vmc/preconditioners/preconditioners.py:288-309) solves with O Q and returns Q y.

The reference ships only the configuration and raises NotImplementedError; this is built from the
mathematics above (parity against the reference is therefore unpinned).  Q is never formed: with U an
orthonormal basis of the gauge span (an SVD of the generators, rank by ``rcond``), Q Q^H = 1 - U U^H, so

    SampleSpace:    T_Q = (O_c Q)(O_c Q)^H / n = (O_c O_c^H - W W^H) / n,  W = O_c U
    ParameterSpace: Q (Q^H S Q + shift)^-1 Q^H F = the solution of (P S P + shift) x = P F, P = 1 - U U^H

(O_c = O - mean, in the full parameter layout).  ``compute_gauge_projection`` returns Q as an operator
(``GaugeProjection``: ``Q @ y``, ``O @ Q``, ``.dense()``).
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from .lowering import site_dims

__all__ = ["GaugeConfig", "GaugeProjection", "compute_gauge_projection", "gauge_generators", "WeightConfig",
           "compute_weight_projection"]


@dataclass(frozen=True)
class GaugeConfig:
    """gauge.py:16-21."""

    rcond: float | None = None
    include_global_scale: bool = True


def _site_tensors(model, params):
    if params is None:
        return model.tensors
    if isinstance(params, torch.Tensor) and params.ndim == 1:
        return model.unpack(params)
    return params


def gauge_generators(model, params=None, include_global_scale: bool = True) -> torch.Tensor:
    """(n_params_full, m) FP64 (complex128 for complex parameters) tangent vectors of the bond gauges,
    ravel order of tensors[r][c] with each site (d, up, down, left, right) C-order."""
    tensors = _site_tensors(model, params)
    R, C = model.shape
    D = model.bond_dim
    dt = torch.complex128 if tensors[0][0].is_complex() else torch.float64
    dev = tensors[0][0].device
    offs, off = {}, 0
    for r in range(R):
        for c in range(C):
            offs[(r, c)] = off
            off += tensors[r][c].numel()
    n = off
    n_bonds = R * (C - 1) + (R - 1) * C
    cols = []

    def one(a, leg_a, b, leg_b):
        # leg index in (d, up, down, left, right): a's leg carries E_ij on the right, b's on the left
        A = tensors[a[0]][a[1]].to(dt)
        B = tensors[b[0]][b[1]].to(dt)
        g = torch.zeros((n, D * D), dtype=dt, device=dev)
        for i in range(D):
            for j in range(D):
                da = torch.zeros_like(A)
                da.select(leg_a, j).copy_(A.select(leg_a, i))
                db = torch.zeros_like(B)
                db.select(leg_b, i).copy_(-B.select(leg_b, j))
                k = i * D + j
                g[offs[a]:offs[a] + A.numel(), k] = da.reshape(-1)
                g[offs[b]:offs[b] + B.numel(), k] = db.reshape(-1)
        cols.append(g)

    for r in range(R):
        for c in range(C - 1):
            one((r, c), 4, (r, c + 1), 3)      # right leg of (r, c), left leg of (r, c+1)
    for r in range(R - 1):
        for c in range(C):
            one((r, c), 2, (r + 1, c), 1)      # down leg of (r, c), up leg of (r+1, c)
    if include_global_scale:
        cols.append(torch.cat([tensors[r][c].to(dt).reshape(-1) for r in range(R) for c in range(C)])[:, None])
    G = torch.cat(cols, dim=1) if cols else torch.zeros((n, 0), dtype=dt, device=dev)
    assert n_bonds * D * D + int(include_global_scale) == G.shape[1]
    return G


class GaugeProjection:
    """Q, an orthonormal basis of the complement of the gauge span, held as U (a basis of the span):
    ``Q @ y`` projects a full-layout vector, ``O @ Q`` the rows of a full-layout Jacobian, onto the
    complement (in the parameter basis, i.e. Q Q^H applied); ``dense()`` forms Q itself."""

    def __init__(self, U: torch.Tensor, n_params: int):
        self.U = U
        self.n_params = n_params
        self.rank = U.shape[1]

    def project(self, x: torch.Tensor) -> torch.Tensor:
        """(1 - U U^H) x for x (n_params,) or (n_params, k)."""
        return x - self.U @ (self.U.conj().T @ x)

    def project_rows(self, O: torch.Tensor) -> torch.Tensor:
        """O (1 - U U^H) for O (n, n_params)."""
        return O - (O @ self.U) @ self.U.conj().T

    def __matmul__(self, y):
        return self.project(y)

    def __rmatmul__(self, O):
        return self.project_rows(O)

    def dense(self) -> torch.Tensor:
        """Q (n_params, n_params - rank): the last columns of a complete QR of U."""
        q, _ = torch.linalg.qr(self.U, mode="complete")
        return q[:, self.rank:]


def compute_gauge_projection(cfg: GaugeConfig, model, params=None, *, return_info: bool = False):
    """gauge.py:24-37: the projection onto the complement of the gauge directions of `model` at
    `params` (site tensors, a flat vector, or None for the model's own)."""
    G = gauge_generators(model, params, cfg.include_global_scale)
    u, s, _ = torch.linalg.svd(G, full_matrices=False)
    rcond = cfg.rcond if cfg.rcond is not None else max(G.shape) * torch.finfo(torch.float64).eps
    keep = s > rcond * (s[0] if s.numel() else 0.0)
    proj = GaugeProjection(u[:, keep], G.shape[0])
    if return_info:
        return proj, {"n_generators": int(G.shape[1]), "rank": int(keep.sum()),
                      "singular_values": s.detach()}
    return proj


@dataclass(frozen=True)
class WeightConfig:
    """weight.py:13-16."""


def compute_weight_projection(cfg, samples, sampler=None):
    """weight.py:19-26: all-ones null vector for the sample-space QGT."""
    return torch.ones(samples.shape[0], dtype=torch.complex128, device=samples.device)
