"""Quantum geometric tensor and sliced Jacobian on the GPU in FP64
(API of src/vmc/qgt/jacobian.py:21-139, qgt.py:36-223, solvers.py:16-37).

The log-derivatives O come from the engine as FP32 (n_samples, n_params);
every contraction here promotes to FP64 on the device.  The sliced ("small-o")
Jacobian stores, per sample, only the active slice of each site; slice k of
the expanded Jacobian is where(p == k, o, 0) (jacobian.py:56-93).

The dense builds accumulate over column blocks (``n_blocks`` slices of the
parameter axis) so the FP64 working set stays bounded.  The SampleSpace Gram of
a real sliced Jacobian on the GPU is the engine's ``vmc_sliced_gram`` kernel
(the masked product of the sliced rows, without the expanded blocks' zero half).
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

__all__ = [
    "SliceOrdering", "SiteOrdering", "Jacobian", "SlicedJacobian", "ParameterSpace", "SampleSpace", "QGT",
    "jacobian_mean", "solve_cholesky", "solve_svd", "solve_cg",
]


@dataclass(frozen=True)
class SliceOrdering:
    """jacobian.py:21-33: columns [k=0 all sites][k=1 all sites]..."""


@dataclass(frozen=True)
class SiteOrdering:
    """jacobian.py:36-46: columns [site0 all k][site1 all k]..."""

    params_per_site: tuple


@dataclass
class Jacobian:
    """jacobian.py:49-53."""

    O: torch.Tensor


@dataclass
class SlicedJacobian:
    """jacobian.py:56-93."""

    o: torch.Tensor
    p: torch.Tensor
    sliced_dims: tuple
    ordering: object = SliceOrdering()

    @property
    def phys_dim(self) -> int:
        return max(self.sliced_dims) if self.sliced_dims else 2


@dataclass(frozen=True)
class ParameterSpace:
    """qgt.py:36-40: S = O^H O / N - mean^H mean."""


@dataclass(frozen=True)
class SampleSpace:
    """qgt.py:43-47: T = O O^H / N with centring terms."""


def _f64(x):
    return x.to(torch.complex128 if x.is_complex() else torch.float64)


def iter_sliced_blocks(jac: SlicedJacobian, n_blocks: int = 1):
    """qgt.py:62-87, yielding FP64 blocks of the expanded Jacobian (optionally split column-wise)."""
    o, p = jac.o, jac.p
    if isinstance(jac.ordering, SliceOrdering):
        for k in range(max(jac.sliced_dims)):
            n = o.shape[1]
            step = -(-n // max(1, n_blocks))
            for c0 in range(0, n, step):
                ob = o[:, c0:c0 + step]
                yield torch.where(p[:, c0:c0 + step] == k, _f64(ob), torch.zeros((), dtype=torch.float64,
                                                                                   device=o.device))
    else:
        i = 0
        for site, n in enumerate(jac.ordering.params_per_site):
            for k in range(jac.sliced_dims[site]):
                yield torch.where(p[:, i:i + n] == k, _f64(o[:, i:i + n]),
                                  torch.zeros((), dtype=torch.float64, device=o.device))
            i += n


def sliced_dense_blocks(jac: SlicedJacobian) -> torch.Tensor:
    """qgt.py:106-108."""
    return torch.cat(list(iter_sliced_blocks(jac)), dim=1)


def _dense_O(jac):
    return _f64(jac.O) if isinstance(jac, Jacobian) else sliced_dense_blocks(jac)


def jacobian_mean(jac) -> torch.Tensor:
    """jacobian.py:96-139."""
    if isinstance(jac, Jacobian):
        return _f64(jac.O).mean(dim=0)
    return torch.cat([b.mean(dim=0) for b in iter_sliced_blocks(jac)])


def sliced_centring(jac: SlicedJacobian):
    """(w, |mean|^2) of a real sliced Jacobian without the expanded blocks: the mean of expanded
    column (k, c) is sum_i o_ic [p_ic == k] / n, and row i of the expanded O meets it only in its own
    slice, so w_i = (O_exp mean)_i = sum_c o_ic mean[p_ic, c]."""
    o64 = _f64(jac.o)
    n = o64.shape[0]
    pl = jac.p.long()
    mean = torch.zeros((jac.phys_dim, o64.shape[1]), dtype=torch.float64, device=o64.device)
    mean.scatter_add_(0, pl, o64)
    mean /= n
    return (o64 * mean.gather(0, pl)).sum(dim=1), (mean * mean).sum()


def _site_from_slice_order(jac):
    """For a site-ordered sliced Jacobian (jacobian.py:36-46): the slice-order index (k * ncols + c) of
    every site-order column of the expanded Jacobian ([site 0: slice 0 columns, slice 1 columns, ...]
    [site 1: ...]); None for another ordering or when the parameter counts do not cover the columns."""
    if not isinstance(jac, SlicedJacobian) or not isinstance(jac.ordering, SiteOrdering):
        return None
    ncols = jac.o.shape[1]
    pps = jac.ordering.params_per_site
    if sum(pps) != ncols or len(jac.sliced_dims) != len(pps):
        return None
    idx, off = [], 0
    for site, n_s in enumerate(pps):
        for k in range(jac.sliced_dims[site]):
            idx.extend(k * ncols + off + j for j in range(n_s))
        off += n_s
    return torch.tensor(idx, dtype=torch.long)


def _kernel_gram(jac) -> bool:
    return (isinstance(jac, SlicedJacobian) and jac.o.device.type == "cuda" and jac.o.dtype == torch.float32
            and jac.p.dtype == torch.int8)


def _sample_space_dense(jac, n_blocks):
    src = jac.O if isinstance(jac, Jacobian) else jac.o
    n, dev = src.shape[0], src.device
    dt = torch.complex128 if src.is_complex() else torch.float64
    if _kernel_gram(jac):
        from .linalg import sliced_gram

        G = sliced_gram(jac.o, jac.p)
        w, msq = sliced_centring(jac)
    else:
        G = torch.zeros((n, n), dtype=dt, device=dev)
        w = torch.zeros(n, dtype=dt, device=dev)
        msq = torch.zeros((), dtype=torch.float64, device=dev)
        blocks = [_f64(jac.O)] if isinstance(jac, Jacobian) else iter_sliced_blocks(jac, n_blocks)
        for ob in blocks:
            G += ob @ ob.conj().T
            mb = ob.mean(dim=0)
            w += ob @ mb.conj()
            msq += torch.vdot(mb, mb).real
    G /= n
    ones = torch.ones(n, dtype=dt, device=dev)
    G -= (w[:, None] * ones[None, :]) / n
    G -= (ones[:, None] * w.conj()[None, :]) / n
    G += (msq / n) * torch.ones((n, n), dtype=dt, device=dev)
    return G


@dataclass
class QGT:
    """qgt.py:36-49: lazy QGT with S @ v and to_dense()."""

    jac: object
    space: object = ParameterSpace()
    n_blocks: int = 16

    def to_dense(self) -> torch.Tensor:
        """qgt.py:173-223."""
        if isinstance(self.space, SampleSpace):
            return _sample_space_dense(self.jac, self.n_blocks)
        perm = _site_from_slice_order(self.jac)
        if _kernel_gram(self.jac) and self.jac.phys_dim == 2 and all(k == 2 for k in self.jac.sliced_dims) and \
                (isinstance(self.jac.ordering, SliceOrdering) or perm is not None):
            # O_exp^T O_exp from the sliced rows (vmc_sliced_gram_params, slice order), less the centring
            # term; a site-ordered Jacobian takes the same matrix with rows and columns permuted
            from .linalg import sliced_gram_params

            n = self.jac.o.shape[0]
            S = sliced_gram_params(self.jac.o, self.jac.p, 2)
            S /= n
            o64 = _f64(self.jac.o)
            mean = torch.zeros((2, o64.shape[1]), dtype=torch.float64, device=o64.device)
            mean.scatter_add_(0, self.jac.p.long(), o64)
            m = (mean / n).reshape(-1)
            S -= m[:, None] * m[None, :]
            if not isinstance(self.jac.ordering, SliceOrdering):
                idx = perm.to(S.device)
                S = S.index_select(0, idx).index_select(1, idx)
            return S
        O = _dense_O(self.jac)
        m = O.mean(dim=0)
        return (O.conj().T @ O) / O.shape[0] - m.conj()[:, None] * m[None, :]

    def __matmul__(self, v):
        """qgt.py:116-165."""
        O = _dense_O(self.jac)
        n = O.shape[0]
        m = O.mean(dim=0)
        v = _f64(v)
        if isinstance(self.space, ParameterSpace):
            return (O.conj().T @ (O @ v)) / n - m.conj() * torch.dot(m, v)
        res = (O @ (O.conj().T @ v)) / n
        vs = v.sum()
        w = O @ m.conj()
        res = res - w * (vs / n)
        res = res - torch.vdot(w, v) / n
        return res + torch.vdot(m, m) * vs / n


def adjoint_matvec(jac, v) -> torch.Tensor:
    """preconditioners.py:100-114: O^H v - mean^H sum(v), block by block."""
    if isinstance(jac, Jacobian):
        O = _f64(jac.O)
        return O.conj().T @ v - O.mean(dim=0).conj() * v.sum()
    parts = [ob.conj().T @ v - ob.mean(dim=0).conj() * v.sum() for ob in iter_sliced_blocks(jac)]
    return torch.cat(parts)


def solve_cholesky(mat, rhs):
    """solvers.py:25-28 (cuSOLVER potrf/potrs in FP64).  Like jax.scipy's cho_factor, a matrix that
    is not positive definite yields NaNs rather than an exception; nothing here reads the host, so
    the solve can run inside a captured CUDA graph."""
    L, _ = torch.linalg.cholesky_ex(mat)
    return torch.cholesky_solve(rhs[:, None], L)[:, 0]


def solve_svd(mat, rhs, rcond: float = 1e-12):
    """solvers.py:31-37."""
    U, S, Vh = torch.linalg.svd(mat, full_matrices=False)
    s_inv = torch.where(S > rcond * S.max(), 1.0 / S, torch.zeros_like(S))
    return Vh.conj().T @ (s_inv * (U.conj().T @ rhs))


def solve_cg(mat, rhs, maxiter: int = 1000, tol: float = 1e-5):
    """solvers.py:16-22 (stop when |r| <= tol |b|)."""
    x = torch.zeros_like(rhs)
    r = rhs - mat @ x
    p = r.clone()
    rs = torch.vdot(r, r).real
    stop = (tol * torch.linalg.norm(rhs)) ** 2
    for _ in range(maxiter):
        if rs <= stop:
            break
        ap = mat @ p
        alpha = rs / torch.vdot(p, ap)
        x = x + alpha * p
        r = r - alpha * ap
        rs_new = torch.vdot(r, r).real
        p = r + (rs_new / rs) * p
        rs = rs_new
    return x
