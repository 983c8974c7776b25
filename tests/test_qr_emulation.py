"""The FP64 / complex128 pivoted QR kernels (vmc_qr_pivoted) in the host-emulation build against
LAPACK xGEQP3 through SciPy.  Up to min(m, n) = 128 LAPACK's xGEQP3 runs the unblocked xLAQP2 that
the kernels restate, so pivots agree exactly and R, Q^H b agree to rounding."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from vmc_gb300.linalg import qr_pivoted


def _rand(rng, shape, cplx):
    a = rng.standard_normal(shape)
    return a + 1j * rng.standard_normal(shape) if cplx else a


def _check(emu_lib, a, b):
    r, piv, qhb = qr_pivoted(torch.as_tensor(a), torch.as_tensor(b), lib=emu_lib)
    q_ref, r_ref, piv_ref = sla.qr(a, mode="economic", pivoting=True)
    assert np.array_equal(piv.numpy(), piv_ref)
    scale = np.abs(r_ref).max()
    assert np.abs(r.numpy() - r_ref).max() <= 1e-12 * scale
    qhb_ref = q_ref.conj().T @ b.reshape(a.shape[0], -1)
    assert np.abs(qhb.numpy() - qhb_ref).max() <= 1e-12 * max(1.0, np.abs(qhb_ref).max())
    # A P = Q R through the reconstruction as well
    assert np.allclose(q_ref @ r.numpy(), a[:, piv.numpy()], atol=1e-11 * scale)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(7, 5), (5, 9), (12, 30), (30, 12), (1, 4), (4, 1), (40, 40), (300, 60), (229, 100)])
def test_matches_lapack_geqp3(emu_lib, m, n, cplx):
    rng = np.random.default_rng(m * 100 + n + cplx)
    a = _rand(rng, (m, n), cplx) * rng.uniform(0.1, 10.0, n)  # distinct column scales
    b = _rand(rng, (m, 2), cplx)
    _check(emu_lib, a, b)


@pytest.mark.parametrize("cplx", [False, True])
def test_rank_deficient_columns_trigger_norm_recomputation(emu_lib, cplx):
    """Repeated and nearly parallel columns drive partial norms to the recompute threshold;
    the factorisation must still reveal the rank like xGEQP3 does."""
    rng = np.random.default_rng(3)
    base = _rand(rng, (25, 6), cplx)
    a = np.concatenate([base, base[:, :3] * 2.0, base[:, 3:] + 1e-9 * _rand(rng, (25, 3), cplx)], axis=1)
    b = _rand(rng, (25,), cplx)
    r, piv, _ = qr_pivoted(torch.as_tensor(a), torch.as_tensor(b), lib=emu_lib)
    _, r_ref, piv_ref = sla.qr(a, mode="economic", pivoting=True)
    d, d_ref = np.abs(np.diag(r.numpy())), np.abs(np.diag(r_ref))
    # the leading, well-separated part of the factorisation is LAPACK's
    assert np.array_equal(piv.numpy()[:6], piv_ref[:6])
    assert np.allclose(d[:6], d_ref[:6], rtol=1e-10)
    # exact duplicates leave nothing; nearly parallel columns leave ~1e-9
    assert d[6:9].max() < 1e-7 * d[0] and d[9:].max() < 1e-12 * d[0]


def test_zero_sizes_and_bad_arguments(emu_lib):
    import ctypes as ct

    from vmc_gb300 import _abi

    r, piv, qhb = qr_pivoted(torch.zeros((0, 3), dtype=torch.float64), lib=emu_lib)
    assert r.shape == (0, 3) and qhb is None
    assert emu_lib.vmc_qr_pivoted(None, 0, None, 1, 2, 2, 0, None, None, None, 0) == _abi.VMC_ERR_INVALID
    buf = torch.zeros(16, dtype=torch.float64)
    p = ct.c_void_p(buf.data_ptr())
    assert emu_lib.vmc_qr_pivoted(None, 0, p, 1, 2, 2, 0, p, p, p, 64) == _abi.VMC_ERR_INVALID  # lda < m
    assert emu_lib.vmc_qr_pivoted(None, 0, p, 2, 2, 2, 0, p, p, p, 8) == _abi.VMC_ERR_WORKSPACE


def test_no_cpu_fallback():
    from vmc_gb300._lib import EngineUnavailable

    with pytest.raises(EngineUnavailable):
        qr_pivoted(torch.zeros((3, 3), dtype=torch.float64))


@pytest.mark.parametrize("m,n,rank", [(30, 100, 12), (60, 40, 25), (50, 50, 50)],
                         ids=["wide-rank-deficient", "tall-rank-deficient", "square-full"])
@pytest.mark.parametrize("cplx", [False, True])
def test_qr_solve_both_min_norm_branches_match_oracle(emu_lib, m, n, rank, cplx):
    """preconditioners.py:166-214 through the device factorisation: the minimum-norm solve picks the
    smaller of its two equivalent systems (rank x rank or n2 x n2); both give the oracle's x."""
    from oracle import sr as osr
    from vmc_gb300 import qgt as gq
    from vmc_gb300.preconditioners import _qr_solve

    rng = np.random.default_rng(m + n + rank)
    O = _rand(rng, (m, rank), cplx) @ _rand(rng, (rank, n), cplx)
    dv = _rand(rng, (m,), cplx)
    x, met = _qr_solve(gq.Jacobian(torch.as_tensor(O)), torch.as_tensor(dv), None, True, lib=emu_lib)
    xr, mr = osr.qr_solve(osr.Jacobian(O), dv)
    assert met["rank"] == mr["rank"]
    assert np.linalg.norm(x.numpy() - xr) <= 1e-9 * np.linalg.norm(xr)


@pytest.mark.parametrize("m,n", [(40, 90), (90, 40)], ids=["wide", "tall"])
@pytest.mark.parametrize("cplx", [False, True])
def test_qr_solve_graded_spectrum(emu_lib, m, n, cplx):
    """Singular values spread over eight decades (rank 30, kept whole by the default rcond): the
    minimum-norm x from the QR of R^H matches the oracle and the pseudo-inverse solution."""
    from oracle import sr as osr
    from vmc_gb300 import qgt as gq
    from vmc_gb300.preconditioners import _qr_solve

    rng = np.random.default_rng(m * n + cplx)
    rank = 30
    u = np.linalg.qr(_rand(rng, (m, rank), cplx))[0]
    v = np.linalg.qr(_rand(rng, (n, rank), cplx))[0]
    O = (u * np.logspace(0, -8, rank)) @ v.conj().T
    dv = _rand(rng, (m,), cplx)
    x, met = _qr_solve(gq.Jacobian(torch.as_tensor(O)), torch.as_tensor(dv), None, True, lib=emu_lib)
    xr, mr = osr.qr_solve(osr.Jacobian(O), dv)
    assert met["rank"] == mr["rank"]
    oc = O - O.mean(axis=0, keepdims=True)
    xp = np.linalg.pinv(oc, rcond=1e-12) @ dv
    assert np.linalg.norm(x.numpy() - xr) <= 1e-6 * np.linalg.norm(xr)
    assert np.linalg.norm(x.numpy() - xp) <= 1e-6 * np.linalg.norm(xp)


@pytest.mark.parametrize("seed", range(12))
def test_random_shapes_and_scales_match_lapack(emu_lib, seed):
    """Random m, n (min(m, n) <= 128, where xGEQP3 runs the unblocked xLAQP2), real or complex, column
    scales over four decades and 1-3 right-hand sides."""
    rng = np.random.default_rng(700 + seed)
    m, n = int(rng.integers(1, 200)), int(rng.integers(1, 129))
    cplx = bool(rng.random() < 0.5)
    a = _rand(rng, (m, n), cplx) * 10.0 ** rng.uniform(-2, 2, n)
    b = _rand(rng, (m, int(rng.integers(1, 4))), cplx)
    _check(emu_lib, a, b)
