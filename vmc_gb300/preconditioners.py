"""SR / TDVP preconditioner on the GPU in FP64
(API of src/vmc/preconditioners/preconditioners.py:41-330)."""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable

import torch

from .lowering import params_per_site
from .qgt import (
    QGT,
    Jacobian,
    ParameterSpace,
    SampleSpace,
    SiteOrdering,
    SliceOrdering,
    SlicedJacobian,
    adjoint_matvec,
    jacobian_mean,
    solve_cg,
    solve_cholesky,
    solve_svd,
)

__all__ = ["DirectSolve", "QRSolve", "SRPreconditioner", "reorder_updates", "solve_cholesky", "solve_svd",
           "solve_cg"]


@dataclass(frozen=True)
class DirectSolve:
    """preconditioners.py:41-45."""

    solver: Callable = solve_cholesky


@dataclass(frozen=True)
class QRSolve:
    """preconditioners.py:48-53 (ParameterSpace and full Jacobian only, like the reference)."""

    rcond: float | None = None
    min_norm: bool = True


_REORDER_INDEX = {}


def _reorder_index(pps, sliced_dims, device):
    key = (tuple(pps), tuple(sliced_dims), str(device))
    idx = _REORDER_INDEX.get(key)
    if idx is None:
        total = sum(pps)
        perm = []
        off = 0
        for site, n in enumerate(pps):
            for k in range(sliced_dims[site]):
                base = k * total + off
                perm.extend(range(base, base + n))
            off += n
        idx = torch.as_tensor(perm, device=device)
        _REORDER_INDEX[key] = idx
    return idx


def reorder_updates(ordering, updates, pps, sliced_dims):
    """preconditioners.py:61-97: slice-major -> site-major parameter order.  The index is built once
    per (sizes, device), so the call reads nothing from the host after the first."""
    if isinstance(ordering, SiteOrdering):
        return updates
    return updates[_reorder_index(pps, sliced_dims, updates.device)]


def _direct_solve(space, jac, dv, diag_shift, solver):
    """preconditioners.py:117-152."""
    qgt = QGT(jac, space)
    S = qgt.to_dense()
    mat = S + diag_shift * torch.eye(S.shape[0], dtype=S.dtype, device=S.device)
    if isinstance(space, ParameterSpace):
        rhs = adjoint_matvec(jac, dv)
        x = solver(mat, rhs)
        res = torch.linalg.norm(S @ x - rhs) ** 2 / torch.linalg.norm(rhs) ** 2
        return x, {"residual_error": res}
    y = solver(mat, dv)
    x = adjoint_matvec(jac, y)
    res = torch.linalg.norm(S @ y - dv) ** 2 / torch.linalg.norm(dv) ** 2
    return x, {"residual_error": res}


def _full_layout(o, p, model):
    """The sliced O (n, n_params_sliced) scattered into the full layout (n, d * n_params_sliced): a
    sample's columns of site s go to the block of its own slice p (ravel order of (d, u, v, l, r))."""
    pps = params_per_site(model.shape, model.bond_dim)
    d = model.phys_dim
    base, sz = [], []
    off = 0
    for n_s in pps:
        base.append(torch.arange(n_s, device=o.device) + d * off)
        sz.append(torch.full((n_s,), n_s, device=o.device))
        off += n_s
    base = torch.cat(base)
    sz = torch.cat(sz)
    idx = base[None, :] + p.to(torch.int64) * sz[None, :]
    full = torch.zeros((o.shape[0], d * off), dtype=o.dtype, device=o.device)
    return full.scatter_(1, idx, o)


def _gauge_direct_solve(space, O, dv, diag_shift, solver, proj):
    """The SR solve in the complement of the gauge directions (preconditioners.py:288-309 with
    O_eff = O Q and updates Q y), through U (proj.U, a basis of the gauge span): Q Q^H = 1 - U U^H."""
    O = O.to(torch.complex128 if O.is_complex() else torch.float64)
    n = O.shape[0]
    Oc = O - O.mean(dim=0)
    U = proj.U.to(O.dtype)
    eye = lambda k: torch.eye(k, dtype=O.dtype, device=O.device)  # noqa: E731
    if isinstance(space, SampleSpace):
        W = Oc @ U
        T = (Oc @ Oc.conj().T - W @ W.conj().T) / n
        y = solver(T + diag_shift * eye(n), dv)
        x = proj.project(Oc.conj().T @ y)
        res = torch.linalg.norm(T @ y - dv) ** 2 / torch.linalg.norm(dv) ** 2
        return x, {"residual_error": res, "gauge_rank": proj.rank}
    S = (Oc.conj().T @ Oc) / n
    SU = S @ U
    PSP = S - U @ SU.conj().T - SU @ U.conj().T + U @ (U.conj().T @ SU) @ U.conj().T
    F = proj.project(Oc.conj().T @ dv)
    x = solver(PSP + diag_shift * eye(S.shape[0]), F)
    res = torch.linalg.norm(PSP @ x - F) ** 2 / torch.linalg.norm(F) ** 2
    return x, {"residual_error": res, "gauge_rank": proj.rank}


def _qr_solve(jac: Jacobian, dv, rcond, min_norm, lib=None):
    """preconditioners.py:166-214: column-pivoted QR of the centred full Jacobian (diag shift
    unused), all in FP64 (complex128) on the Jacobian's device: the factorisation is the
    engine's vmc_qr_pivoted kernel, the rank and triangular solves are torch linear algebra."""
    from .linalg import qr_pivoted

    O = jac.O
    cplx = O.is_complex() or dv.is_complex()
    dt = torch.complex128 if cplx else torch.float64
    o = O.to(dt)
    oc = o - o.mean(dim=0, keepdim=True)
    dvd = dv.to(device=o.device, dtype=dt)
    r, piv, y = qr_pivoted(oc, dvd, lib=lib)
    y = y[:, 0]
    k, n_red = r.shape
    # One Householder QR of R^H (n x k), R^H = Q T, serves both the rank and the solve: R = T^H Q^H has
    # T's singular values (an SVD of the k x k triangle instead of the k x n trapezoid, with no squaring
    # as R R^H would), and the minimum-norm solution of R[:rank] z = y1 is z = Q [T11^-H y1; 0] with
    # T11 = T[:rank, :rank], since R[:rank]^H = Q[:, :rank] T11
    qa = tau = None
    if n_red > k:
        qa, tau = torch.geqrf(r.mH)
        rt = qa[:k].triu()
    else:
        rt = r
    eps = torch.finfo(torch.float64).eps
    rtol = max(r.shape) * eps if rcond is None else rcond
    if rt.is_cuda and rt.numel():
        # singular values only, by cuSOLVER's QR-iteration SVD (gesvd): robust on the rank-deficient
        # triangles that repeated samples produce (the approximate gesvda does not converge on them)
        sv = torch.linalg.svdvals(rt, driver="gesvd")
    else:
        sv = torch.linalg.svdvals(rt)
    smax = sv.max() if sv.numel() else torch.zeros((), dtype=torch.float64, device=o.device)
    tol = rtol * smax
    rank = int((sv > tol).sum())  # the reference's int(matrix_rank(r)) also reads it on the host
    n2 = n_red - rank
    x = torch.zeros(n_red, dtype=dt, device=o.device)
    if rank:
        y1 = y[:rank, None]
        if min_norm and n2 > 0:
            # the reference's z1 + B z2 = a, a = R11^-1 y1, B = R11^-1 R12, minimising |z|, is the
            # minimum-norm solution of [R11 R12] z = y1
            if qa is None:
                qa, tau = torch.geqrf(r.mH)
            w = torch.zeros((n_red, 1), dtype=dt, device=o.device)
            w[:rank] = torch.linalg.solve_triangular(qa[:rank, :rank].triu().mH, y1, upper=False)
            z = torch.ormqr(qa, tau, w, left=True, transpose=False)
        else:
            z = torch.zeros((n_red, 1), dtype=dt, device=o.device)
            z[:rank] = torch.linalg.solve_triangular(r[:rank, :rank], y1, upper=True)
        x[piv] = z[:, 0]
    rhs = oc.mH @ dvd
    resid = oc.mH @ (oc @ x) - rhs
    err = (torch.linalg.norm(resid) ** 2 / torch.linalg.norm(rhs) ** 2).item()
    return x, {"residual_error": err, "rank": rank}


class SRPreconditioner:
    """preconditioners.py:244-330."""

    def __init__(self, space=ParameterSpace(), strategy=DirectSolve(), diag_shift: float = 1e-2,
                 gauge_config=None, ordering=SliceOrdering()):
        self.space = space
        self.strategy = strategy
        self.diag_shift = float(diag_shift)
        self.gauge_config = gauge_config
        self.ordering = ordering
        self.uses_local_energies = True
        self._metrics = {}

    @property
    def residual_error(self):
        return self._metrics.get("residual_error")

    def apply(self, model, params, samples, o, p, local_energies, *, grad_factor=1.0):
        """Returns (updates as a list of per-site tensors shaped like model.tensors, metrics)."""
        e = local_energies.reshape(-1)
        e = e.to(torch.complex128 if e.is_complex() else torch.float64)
        n_samples = samples.shape[0]
        dv = (e - e.mean()) / n_samples
        complex_factor = isinstance(grad_factor, complex) and grad_factor.imag != 0
        if complex_factor:
            dv = dv.to(torch.complex128) * grad_factor
        else:
            dv = dv * float(getattr(grad_factor, "real", grad_factor))
        pps = tuple(params_per_site(model.shape, model.bond_dim))
        # slices per site: phys_dim, or a GI model's phys_dim * nc per site (src/vmc/peps/gi/model.py:1066-1080)
        sd = model.sliced_dims() if hasattr(model, "sliced_dims") else (model.phys_dim,) * (
            model.shape[0] * model.shape[1])
        if self.gauge_config is not None:
            # gauge removal (preconditioners.py:288-309): the solve in the complement of the gauge span,
            # the update returned in the full parameter layout
            from .gauge import compute_gauge_projection

            if hasattr(model, "sliced_dims"):
                raise NotImplementedError("gauge removal: standard PEPS")
            proj = compute_gauge_projection(self.gauge_config, model, params)
            O_full = o if p is None else _full_layout(o, p, model)
            if isinstance(self.strategy, DirectSolve):
                x, metrics = _gauge_direct_solve(self.space, O_full, dv, self.diag_shift, self.strategy.solver,
                                                 proj)
            else:
                if isinstance(self.space, SampleSpace):
                    raise NotImplementedError("QRSolve not supported for SampleSpace")
                # the minimum-norm solution of (O P) x = dv lies in range(P) and equals Q (O Q)^+ dv
                o_p = proj.project_rows(O_full.to(proj.U.dtype))
                x, metrics = _qr_solve(Jacobian(o_p), dv, self.strategy.rcond, self.strategy.min_norm)
                metrics = dict(metrics, gauge_rank=proj.rank)
            param_dtype = getattr(model, "dtype", torch.float32)
            if not complex_factor and not param_dtype.is_complex:
                x = 2.0 * x.real
            self._metrics = metrics
            return model.unpack(x.to(param_dtype)), metrics
        jac = Jacobian(o) if p is None else SlicedJacobian(o, p, sd, self.ordering)
        if isinstance(self.strategy, DirectSolve):
            x, metrics = _direct_solve(self.space, jac, dv, self.diag_shift, self.strategy.solver)
        else:
            if p is not None:
                raise NotImplementedError("QRSolve not supported for SlicedJacobian")
            if isinstance(self.space, SampleSpace):
                raise NotImplementedError("QRSolve not supported for SampleSpace")
            x, metrics = _qr_solve(jac, dv, self.strategy.rcond, self.strategy.min_norm)
        if p is not None:
            x = reorder_updates(self.ordering, x, pps, sd)
        param_dtype = getattr(model, "dtype", torch.float32)
        if not complex_factor and not param_dtype.is_complex:
            x = 2.0 * x.real  # real parameters: preconditioners.py:322-329
        self._metrics = metrics
        return model.unpack(x.to(param_dtype)), metrics
