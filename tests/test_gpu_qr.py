"""The FP64 / complex128 pivoted QR (vmc_qr_pivoted) and the SR QR solve on the GPU: against
LAPACK xGEQP3 where it runs the same unblocked algorithm (min(m, n) <= 128), through exact
invariants above that, and the solve at the 8x8 D=4 workload's full-Jacobian size (4096 samples x
21,632 parameters) against the minimum-norm solution computed another way."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from oracle import sr as osr
from vmc_gb300 import qgt as gq
from vmc_gb300.linalg import qr_pivoted
from vmc_gb300.preconditioners import _qr_solve

pytestmark = pytest.mark.gpu


def _rand(rng, shape, cplx):
    a = rng.standard_normal(shape)
    return a + 1j * rng.standard_normal(shape) if cplx else a


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(100, 60), (60, 128), (128, 128)])
def test_matches_lapack_geqp3(cuda_device, m, n, cplx):
    rng = np.random.default_rng(m + n + cplx)
    a = _rand(rng, (m, n), cplx) * rng.uniform(0.1, 10.0, n)
    b = _rand(rng, (m,), cplx)
    r, piv, qhb = qr_pivoted(torch.as_tensor(a, device=cuda_device), torch.as_tensor(b, device=cuda_device))
    q_ref, r_ref, piv_ref = sla.qr(a, mode="economic", pivoting=True)
    assert np.array_equal(piv.cpu().numpy(), piv_ref)
    assert np.abs(r.cpu().numpy() - r_ref).max() <= 1e-12 * np.abs(r_ref).max()
    assert np.allclose(qhb.cpu().numpy()[:, 0], q_ref.conj().T @ b, rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("cplx", [False, True])
def test_invariants_beyond_the_unblocked_size(cuda_device, cplx):
    """R^H R = (A P)^H (A P); |R_jj| never increases; least squares from (R, Q^H b) = lstsq."""
    m, n = 700, 400
    rng = np.random.default_rng(11)
    a = _rand(rng, (m, n), cplx)
    b = _rand(rng, (m,), cplx)
    r, piv, qhb = qr_pivoted(torch.as_tensor(a, device=cuda_device), torch.as_tensor(b, device=cuda_device))
    r, piv, qhb = r.cpu().numpy(), piv.cpu().numpy(), qhb.cpu().numpy()[:, 0]
    assert np.array_equal(np.sort(piv), np.arange(n))
    ap = a[:, piv]
    g = ap.conj().T @ ap
    assert np.abs(r.conj().T @ r - g).max() <= 1e-11 * np.abs(g).max()
    d = np.abs(np.diag(r))
    assert np.all(d[1:] <= d[:-1] * (1 + 1e-12))
    x = np.zeros(n, dtype=a.dtype)
    x[piv] = sla.solve_triangular(r, qhb, lower=False)
    assert np.allclose(x, np.linalg.lstsq(a, b, rcond=None)[0], rtol=1e-9, atol=1e-10)


def test_qr_solve_matches_oracle(cuda_device):
    rng = np.random.default_rng(5)
    O = rng.standard_normal((300, 40)) @ rng.standard_normal((40, 900))  # rank 40 < 300 samples
    dv = rng.standard_normal(300)
    x, met = _qr_solve(gq.Jacobian(torch.as_tensor(O, device=cuda_device)), torch.as_tensor(dv, device=cuda_device),
                       None, True)
    xr, mr = osr.qr_solve(osr.Jacobian(O), dv)
    assert met["rank"] == mr["rank"] == 40
    assert np.linalg.norm(x.cpu().numpy() - xr) <= 1e-8 * np.linalg.norm(xr)


def test_qr_solve_at_the_full_jacobian_size(cuda_device):
    """4096 x 21,632 (the 8x8 D=4 full Jacobian): full row rank, so x is the minimum-norm
    solution oc^H (oc oc^H)^-1 dv whatever the pivots."""
    m, n = 4096, 21632
    g = torch.Generator(device=cuda_device).manual_seed(0)
    O = torch.randn((m, n), generator=g, dtype=torch.float64, device=cuda_device)
    dv = torch.randn(m, generator=g, dtype=torch.float64, device=cuda_device)
    x, met = _qr_solve(gq.Jacobian(O), dv, None, True)
    assert met["rank"] == m - 1  # centring removes one direction
    oc = O - O.mean(dim=0, keepdim=True)
    # centred columns sum to zero, so oc oc^T has the all-ones null vector: pseudo-inverse
    ref = oc.T @ (torch.linalg.pinv(oc @ oc.T, hermitian=True) @ dv)
    assert float(torch.linalg.norm(x - ref) / torch.linalg.norm(ref)) < 1e-8
    assert met["residual_error"] < 1e-12
