"""FP64 restatement of the sliced QGT, SR solve, linear solvers and integrators (oracle).

Follows src/vmc/qgt/jacobian.py:21-139, src/vmc/qgt/qgt.py:62-223,
src/vmc/qgt/solvers.py:16-37, src/vmc/preconditioners/preconditioners.py:41-330
and src/vmc/drivers/integrators.py:45-144.  Test infrastructure only.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg as sla


@dataclass(frozen=True)
class SliceOrdering:
    """jacobian.py:21-33."""


@dataclass(frozen=True)
class SiteOrdering:
    """jacobian.py:36-46."""
    params_per_site: tuple


@dataclass
class Jacobian:
    """jacobian.py:49-53."""
    O: np.ndarray


@dataclass
class SlicedJacobian:
    """jacobian.py:56-93."""
    o: np.ndarray
    p: np.ndarray
    sliced_dims: tuple
    ordering: object = SliceOrdering()


@dataclass(frozen=True)
class ParameterSpace:
    """qgt.py:36-40."""


@dataclass(frozen=True)
class SampleSpace:
    """qgt.py:43-47."""


def iter_sliced_blocks(o, p, sliced_dims, ordering):
    """qgt.py:62-87."""
    if isinstance(ordering, SliceOrdering):
        for k in range(max(sliced_dims)):
            yield np.where(p == k, o, 0), o.shape[1]
    else:
        i = 0
        for site_idx, n in enumerate(ordering.params_per_site):
            for k in range(sliced_dims[site_idx]):
                yield np.where(p[:, i:i + n] == k, o[:, i:i + n], 0), n
            i += n


def sliced_dense_blocks(jac: SlicedJacobian):
    """qgt.py:106-108."""
    return np.concatenate([b for b, _ in iter_sliced_blocks(jac.o, jac.p, jac.sliced_dims,
                                                            jac.ordering)], axis=1)


def jacobian_mean(jac):
    """jacobian.py:96-139."""
    if isinstance(jac, Jacobian):
        return jac.O.mean(axis=0)
    return np.concatenate([b.mean(axis=0) for b, _ in
                           iter_sliced_blocks(jac.o, jac.p, jac.sliced_dims, jac.ordering)])


def _dense_O(jac):
    return jac.O if isinstance(jac, Jacobian) else sliced_dense_blocks(jac)


def to_dense(jac, space):
    """qgt.py:173-223."""
    O = _dense_O(jac)
    n = O.shape[0]
    mean = jacobian_mean(jac)
    if isinstance(space, ParameterSpace):
        return (O.conj().T @ O) / n - mean.conj()[:, None] * mean[None, :]
    G = (O @ O.conj().T) / n
    ones = np.ones(n)
    w = O @ mean.conj()
    G = G - (w[:, None] * ones[None, :]) / n
    G = G - (ones[:, None] * w.conj()[None, :]) / n
    G = G + (np.vdot(mean, mean) / n) * np.ones((n, n))
    return G


def matvec(jac, space, v):
    """qgt.py:116-165."""
    O = _dense_O(jac)
    n = O.shape[0]
    mean = jacobian_mean(jac)
    if isinstance(space, ParameterSpace):
        return (O.conj().T @ (O @ v)) / n - mean.conj() * np.dot(mean, v)
    res = (O @ (O.conj().T @ v)) / n
    v_sum = np.sum(v)
    w = O @ mean.conj()
    res = res - w * (v_sum / n)
    res = res - np.ones(n) * (np.vdot(w, v) / n)
    res = res + np.ones(n) * (np.vdot(mean, mean) * v_sum / n)
    return res


def adjoint_matvec(jac, v):
    """preconditioners.py:100-114."""
    O = _dense_O(jac)
    return O.conj().T @ v - jacobian_mean(jac).conj() * np.sum(v)


def reorder_updates(ordering, updates, pps, sliced_dims):
    """preconditioners.py:61-97: slice-major -> site-major."""
    if isinstance(ordering, SiteOrdering):
        return updates
    total = sum(pps)
    perm = []
    off = 0
    for site_idx, n in enumerate(pps):
        for k in range(sliced_dims[site_idx]):
            base = k * total + off
            perm.extend(range(base, base + n))
        off += n
    return updates[np.asarray(perm)]


def solve_cholesky(mat, rhs):
    """solvers.py:25-28."""
    return sla.cho_solve(sla.cho_factor(mat), rhs)


def solve_svd(mat, rhs, rcond=1e-12):
    """solvers.py:31-37."""
    u, s, vh = np.linalg.svd(mat, full_matrices=False)
    s_inv = np.where(s > rcond * s.max(), 1.0 / s, 0.0)
    return vh.conj().T @ (s_inv * (u.conj().T @ rhs))


def solve_cg(mat, rhs, maxiter=1000, tol=1e-5):
    """solvers.py:16-22 (jax.scipy.sparse.linalg.cg: stop when |r| <= tol |b|)."""
    x = np.zeros_like(rhs)
    r = rhs - mat @ x
    p = r.copy()
    rs = np.vdot(r, r).real
    stop = (tol * np.linalg.norm(rhs)) ** 2
    for _ in range(maxiter):
        if rs <= stop:
            break
        ap = mat @ p
        alpha = rs / np.vdot(p, ap)
        x = x + alpha * p
        r = r - alpha * ap
        rs_new = np.vdot(r, r).real
        p = r + (rs_new / rs) * p
        rs = rs_new
    return x


@dataclass(frozen=True)
class DirectSolve:
    """preconditioners.py:41-45."""
    solver: object = solve_cholesky


@dataclass(frozen=True)
class QRSolve:
    """preconditioners.py:48-53."""
    rcond: float | None = None
    min_norm: bool = True


def direct_solve(space, jac, dv, diag_shift, solver):
    """preconditioners.py:117-152."""
    S = to_dense(jac, space)
    mat = S + diag_shift * np.eye(S.shape[0])
    if isinstance(space, ParameterSpace):
        rhs = adjoint_matvec(jac, dv)
        x = solver(mat, rhs)
        return x, {"residual_error": np.linalg.norm(S @ x - rhs) ** 2 / np.linalg.norm(rhs) ** 2}
    y = solver(mat, dv)
    x = adjoint_matvec(jac, y)
    return x, {"residual_error": np.linalg.norm(S @ y - dv) ** 2 / np.linalg.norm(dv) ** 2}


def qr_solve(jac: Jacobian, dv, rcond=None, min_norm=True):
    """preconditioners.py:166-214 (pivoted QR; diag_shift unused as in the reference)."""
    mean = jacobian_mean(jac)
    oc = jac.O - mean[None, :]
    q, r, piv = sla.qr(oc, mode="economic", pivoting=True)
    y = q.conj().T @ dv
    sv = np.linalg.svd(r, compute_uv=False)
    tol = (max(r.shape) * np.finfo(r.dtype).eps if rcond is None else rcond) * (sv.max() if sv.size else 0)
    rank = int(np.sum(sv > tol))
    n_red = r.shape[1]
    n2 = n_red - rank
    if rank == 0:
        x = np.zeros(n_red, dtype=oc.dtype)
    else:
        r11, r12, y1 = r[:rank, :rank], r[:rank, rank:], y[:rank]
        if min_norm and n2 > 0:
            a = sla.solve_triangular(r11, y1, lower=False)
            b = sla.solve_triangular(r11, r12, lower=False)
            lhs = b.conj().T @ b + np.eye(n2)
            x2 = sla.solve(lhs, b.conj().T @ a, assume_a="pos")
            x1 = a - b @ x2
        else:
            x1 = sla.solve_triangular(r11, y1, lower=False)
            x2 = np.zeros(n2, dtype=oc.dtype)
        x = np.zeros(n_red, dtype=np.result_type(x1.dtype, oc.dtype))
        x[piv] = np.concatenate([x1, x2])
    rhs = oc.conj().T @ dv
    resid = oc.conj().T @ (oc @ x) - rhs
    return x, {"residual_error": np.linalg.norm(resid) ** 2 / np.linalg.norm(rhs) ** 2, "rank": rank}


def sr_apply(o, p, local_energies, *, pps, sliced_dims, n_samples, space=ParameterSpace(),
             strategy=DirectSolve(), diag_shift=1e-2, ordering=SliceOrdering(), grad_factor=1.0,
             real_params=True):
    """preconditioners.py:268-330 -> flat site-major update vector and metrics."""
    e = local_energies.reshape(-1)
    dv = grad_factor * (e - e.mean()) / n_samples
    jac = Jacobian(o) if p is None else SlicedJacobian(o, p, tuple(sliced_dims), ordering)
    if isinstance(strategy, DirectSolve):
        x, metrics = direct_solve(space, jac, dv, diag_shift, strategy.solver)
    else:
        if p is not None:
            raise NotImplementedError("QRSolve not supported for SlicedJacobian")
        if isinstance(space, SampleSpace):
            raise NotImplementedError("QRSolve not supported for SampleSpace")
        x, metrics = qr_solve(jac, dv, strategy.rcond, strategy.min_norm)
    if p is not None:
        x = reorder_updates(ordering, x, tuple(pps), tuple(sliced_dims))
    if np.isrealobj(np.asarray(grad_factor)) and real_params:
        x = 2.0 * x.real
    return x, metrics


def euler_step(f, state, t, dt, carry):
    """integrators.py:45-63."""
    k, carry_next, aux = f(state, t, carry)
    return state + dt * k, t + dt, carry_next, aux


def rk4_step(f, state, t, dt, carry):
    """integrators.py:66-109."""
    k1, c1, _ = f(state, t, carry)
    k2, c2, _ = f(state + 0.5 * dt * k1, t + 0.5 * dt, c1)
    k3, c3, _ = f(state + 0.5 * dt * k2, t + 0.5 * dt, c2)
    k4, c4, aux = f(state + dt * k3, t + dt, c3)
    return state + dt * (k1 + 2.0 * k2 + 2.0 * k3 + k4) / 6.0, t + dt, c4, aux
