"""Pins the oracle's QGT / SR solve / solvers / integrators.

Restates tests/test_qgt.py:84-160 (slice-ordering reorder, slice vs site
solve), tests/test_qgt_solvers.py:15-46 and tests/test_integrators.py:25-69
of the reference.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from oracle import peps as oracle
from oracle import sr
from tests.helpers import uniform_init_tensors
from vmc_gb300.operators import LocalHamiltonian


def _samples_o_p(n=64, seed=0):
    shape, D = (2, 3), 2
    T = uniform_init_tensors(shape, D, seed=seed)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    init, trans, est = oracle.build_mc_kernels(model, LocalHamiltonian(shape, ()))
    rng = np.random.default_rng(seed)
    cfg = rng.integers(0, 2, size=(n, 6))
    cache = init(T, cfg)
    cfg, ctx = trans(T, cfg, rng.random((n, 6)), cache)
    amps, grads_full, _ = oracle.value_and_grad(model, cfg, full_gradient=True)
    amps, grads, p = oracle.value_and_grad(model, cfg)
    return model, grads_full / amps[:, None], grads / amps[:, None], p


def test_slice_ordering_reorders_to_full_jacobian():
    """tests/test_qgt.py:84-119."""
    model, o_full, o, p = _samples_o_p(32)
    sd = oracle.sliced_dims(model)
    pps = tuple(oracle.params_per_site(model))
    o_slice = sr.sliced_dense_blocks(sr.SlicedJacobian(o, p, sd, sr.SliceOrdering()))
    perm = sr.reorder_updates(sr.SliceOrdering(), np.arange(o_slice.shape[1]), pps, sd)
    assert np.allclose(o_slice[:, perm], o_full, rtol=1e-10)


def test_slice_ordering_solve_matches_site_ordering():
    """tests/test_qgt.py:121-160 (diag_shift 1e-4, rel err < 1e-6)."""
    model, _, o, p = _samples_o_p(64)
    sd = oracle.sliced_dims(model)
    pps = tuple(oracle.params_per_site(model))
    shift = 1e-4
    s_slice = sr.to_dense(sr.SlicedJacobian(o, p, sd, sr.SliceOrdering()), sr.ParameterSpace())
    rhs = np.random.default_rng(1).standard_normal(s_slice.shape[0])
    x_slice = sr.solve_cholesky(s_slice + shift * np.eye(s_slice.shape[0]), rhs)
    x_slice = sr.reorder_updates(sr.SliceOrdering(), x_slice, pps, sd)
    s_site = sr.to_dense(sr.SlicedJacobian(o, p, sd, sr.SiteOrdering(pps)), sr.ParameterSpace())
    rhs_site = sr.reorder_updates(sr.SliceOrdering(), rhs, pps, sd)
    x_site = sr.solve_cholesky(s_site + shift * np.eye(s_site.shape[0]), rhs_site)
    assert np.linalg.norm(x_slice - x_site) / np.linalg.norm(x_site) < 1e-6


def test_sample_and_parameter_space_updates_agree():
    """Push-through identity (O^T O + l I)^-1 O^T = O^T (O O^T + l I)^-1 for the centred O."""
    model, _, o, p = _samples_o_p(48)
    sd = oracle.sliced_dims(model)
    pps = oracle.params_per_site(model)
    e = np.random.default_rng(3).standard_normal(o.shape[0])
    kw = dict(pps=pps, sliced_dims=sd, n_samples=o.shape[0], diag_shift=1e-3, grad_factor=-1.0)
    x_p, _ = sr.sr_apply(o, p, e, space=sr.ParameterSpace(), **kw)
    x_s, _ = sr.sr_apply(o, p, e, space=sr.SampleSpace(), **kw)
    assert np.linalg.norm(x_p - x_s) / np.linalg.norm(x_p) < 1e-6


def test_matvec_matches_dense():
    model, _, o, p = _samples_o_p(40)
    jac = sr.SlicedJacobian(o, p, oracle.sliced_dims(model), sr.SliceOrdering())
    rng = np.random.default_rng(2)
    for space in (sr.ParameterSpace(), sr.SampleSpace()):
        S = sr.to_dense(jac, space)
        v = rng.standard_normal(S.shape[0])
        assert np.allclose(sr.matvec(jac, space, v), S @ v, rtol=1e-10, atol=1e-12)


def test_qr_solve_matches_min_norm_least_squares():
    """preconditioners.py:166-214: pivoted-QR minimum-norm solve of the centred full Jacobian."""
    rng = np.random.default_rng(7)
    O = rng.standard_normal((30, 12)) @ rng.standard_normal((12, 40))  # rank 12 < 40 params
    dv = rng.standard_normal(30)
    x, metrics = sr.qr_solve(sr.Jacobian(O), dv)
    oc = O - O.mean(axis=0)
    x_ref = np.linalg.lstsq(oc, dv, rcond=None)[0]
    assert metrics["rank"] == np.linalg.matrix_rank(oc)
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8


def test_solvers_match_dense_solve():
    """tests/test_qgt_solvers.py:15-46."""
    rng = np.random.default_rng(0)
    a = rng.standard_normal((24, 24))
    a = a.T @ a + 0.1 * np.eye(24)
    b = rng.standard_normal(24)
    x = np.linalg.solve(a, b)
    assert np.linalg.norm(sr.solve_cg(a, b, tol=1e-10, maxiter=2000) - x) / np.linalg.norm(x) < 1e-6
    c = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    c = c @ c.conj().T + 0.2 * np.eye(16)
    bc = rng.standard_normal(16) + 1j * rng.standard_normal(16)
    xc = np.linalg.solve(c, bc)
    assert np.linalg.norm(sr.solve_svd(c, bc) - xc) / np.linalg.norm(xc) < 1e-8
    s = rng.standard_normal((12, 12))
    s = s.T @ s + 0.5 * np.eye(12)
    bs = rng.standard_normal(12)
    xs = np.linalg.solve(s, bs)
    assert np.linalg.norm(sr.solve_cholesky(s, bs) - xs) / np.linalg.norm(xs) < 1e-10


def _lin(mat):
    return lambda y, t, carry: (mat @ y, carry, None)


def test_rk4_matches_expm():
    """tests/test_integrators.py:25-47: 4x4 Hermitian generator, dt=0.1, rel err < 1e-7."""
    rng = np.random.default_rng(0)
    m = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    m = 0.1 * (m + m.conj().T)
    y0 = rng.standard_normal(4) + 1j * rng.standard_normal(4)
    y1, t1, _, _ = sr.rk4_step(_lin(m), y0, 0.0, 0.1, None)
    ref = sla.expm(m * 0.1) @ y0
    assert np.linalg.norm(y1 - ref) / np.linalg.norm(ref) < 1e-7
    assert t1 == 0.1


def test_euler_is_first_order():
    """tests/test_integrators.py:49-69."""
    rng = np.random.default_rng(2)
    m = rng.standard_normal((3, 3))
    m = 0.05 * (m + m.T)
    y0 = rng.standard_normal(3)
    y1, _, _, _ = sr.euler_step(_lin(m), y0, 0.0, 0.1, None)
    ref = sla.expm(m * 0.1) @ y0
    assert np.linalg.norm(y1 - ref) / np.linalg.norm(ref) < 1e-3
