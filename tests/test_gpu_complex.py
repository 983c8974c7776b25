"""Complex64 PEPS on the GPU at larger sizes: the 10x10 TFIM quench workload (complex64, D=4, chi=16)
through exact properties, a 6x6 subset against the complex128 oracle, and a real-time RK4 step."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, assert_parity, complex_tensors, hamiltonian
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors, params_per_site
from vmc_gb300.synthetic import WORKLOADS

pytestmark = pytest.mark.gpu


def test_config3_10x10_complex_exact_properties(cuda_device):
    w = WORKLOADS["tfim10x10_D4_chi16_c64"]
    R, C = w.shape
    n = 512
    T = w.tensors(seed=0)
    eng = PEPSEngine(w.shape, w.bond_dim, w.chi, 2, "ZipUp", operator=w.operator(), device=cuda_device,
                     dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    cfg = torch.from_numpy(np.random.default_rng(2).integers(0, 2, (n, R * C)).astype(np.int32)).to(cuda_device)
    c = cfg.clone()
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.zeros((n, R * C), dtype=torch.float64, device=cuda_device), cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    assert torch.equal(res.configs, 1 - cfg)
    assert torch.isfinite(res.O.real).all() and torch.isfinite(res.O.imag).all()
    assert torch.isfinite(res.E.real).all() and torch.isfinite(res.logamp).all()
    pps = params_per_site(w.shape, w.bond_dim)
    off, vals = 0, []
    for site in range(R * C):
        r, col = divmod(site, C)
        A = torch.from_numpy(np.asarray(T[r][col], dtype=np.complex64)).to(cuda_device).reshape(2, -1)
        vals.append((A[res.configs[:, site].long()] * res.O[:, off:off + pps[site]]).sum(1).to(torch.complex128))
        off += pps[site]
    v = torch.stack(vals, 1).reshape(n, R, C)
    # sum_k A_k O_k = psi_row(r) / psi: 1 on the last row, one value along every row
    assert float((v[:, R - 1, :] - 1).abs().max()) < 1e-3
    mean = v.mean(dim=2, keepdim=True)
    spread = (v - mean).abs().amax(dim=2) / mean.abs().squeeze(2).clamp_min(1e-2)
    assert float(spread.median()) < 1e-4


def test_complex_6x6_subset_matches_oracle(cuda_device):
    shape, D, chi = (6, 6), 4, 16
    H = hamiltonian("tfim", shape)
    T = complex_tensors(shape, D, seed=8)
    cfg = np.random.default_rng(9).integers(0, 2, (6, 36)).astype(np.int32)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device, dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, ph, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, ph)
    torch.cuda.synchronize()
    eng.raise_on_status()
    model = oracle.PEPS(T, shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    assert_parity(np.abs(np.exp(la.cpu().numpy() + 1j * ph.cpu().numpy()) / amp - 1), True, **tol)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True, **tol)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(E.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True, **tol)


def test_real_time_rk4_on_the_gpu(cuda_device):
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.drivers import RK4, RealTimeUnit, TDVPDriver
    from vmc_gb300.operators import transverse_field_ising
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import SampleSpace

    shape, D = (3, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), device=cuda_device,
                 dtype=torch.complex64, tensors=complex_tensors(shape, D, seed=3))
    drv = TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=RealTimeUnit(), integrator=RK4(),
                     preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=1e-2), n_samples=128,
                     n_chains=64)
    drv.run(0.02)
    assert drv.step_count == 2 and abs(drv.t - 0.02) < 1e-12
    assert drv._tensors[0][0].dtype == torch.complex64
    assert np.isfinite(drv.energy["mean"].real) and np.isfinite(drv.energy["variance"])


def test_complex_density_matrix_matches_oracle(cuda_device):
    """DensityMatrix on complex64 tensors (strategy.py:153-176), chi <= D so every kept eigenvector of
    rho = theta^H theta has a nonzero eigenvalue: one transition + estimate against the complex128 oracle."""
    from tests.helpers import oracle_sweep

    shape, D, chi, n = (4, 4), 3, 3, 16
    H = hamiltonian("tfim", shape)
    T = complex_tensors(shape, D, seed=7)
    rng = np.random.default_rng(7)
    cfg = rng.integers(0, 2, (n, 16)).astype(np.int32)
    u = rng.random((n, 16))
    eng = PEPSEngine(shape, D, chi, 2, "DensityMatrix", operator=H, device=cuda_device, dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg.copy()).to(cuda_device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(cuda_device), cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    c2, ctx, le = oracle_sweep(T, shape, D, "DensityMatrix", chi, H, cfg, u)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    assert np.all(same | (res.margin.cpu().numpy() < 1e-4))
    amp = np.exp(res.logamp.cpu().numpy() + 1j * res.sign.cpu().numpy())
    assert np.max(np.abs(amp[same] / ctx.amp[same] - 1)) < 1e-4
    o, o_ref = res.O.cpu().numpy()[same], le.local_log_derivatives[same]
    assert np.max(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < 5e-5
    e, e_ref = res.E.cpu().numpy()[same], le.local_estimate[same]
    assert np.max(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref))) < 5e-5
