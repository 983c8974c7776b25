"""CUDA engine (sm_103a, via the C ABI) against the FP64 oracle on seeded inputs.

Tolerances (tests/helpers.py): FP32 rounding level (2e-5) without active
truncation; with truncation a 2e-5 median and 2e-3 worst case per sample,
because the kept subspace at a cut moves by ~eps_fp32 / relative gap.
Sampled configurations must be identical except for chains with an accept
decision within 1e-4 of its threshold (reported as `margin`).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import (CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, E_BAR, O_BAR, TRUNC_MAX_TOL, TRUNC_MEDIAN_TOL,
                           assert_parity, accuracy, complex_tensors, fp32, hamiltonian, make_case, oracle_sweep)
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

pytestmark = pytest.mark.gpu

CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((2, 3), 3, 16, "NoTruncation", "tfim"),
    ((3, 3), 3, 4, "ZipUp", "heisenberg"),
    ((4, 4), 2, 4, "ZipUp", "tfim"),
    ((4, 4), 3, 6, "ZipUp", "heisenberg"),
    ((3, 4), 2, 3, "ZipUp", "heisenberg"),
    ((3, 3), 2, 4, "Variational", "heisenberg"),
    ((4, 4), 3, 6, "Variational", "tfim"),
    ((3, 4), 2, 3, "Variational", "heisenberg"),
    # DensityMatrix where every kept eigenvector has a nonzero eigenvalue (chi <= D)
    ((3, 3), 2, 2, "DensityMatrix", "heisenberg"),
    ((4, 4), 3, 3, "DensityMatrix", "tfim"),
]


def _run(device, shape, D, chi, strategy, H, T, cfg, u, full=False, options=None):
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device=device, options=options)
    tens = torch.from_numpy(pack_tensors(T)).to(device)
    c = torch.from_numpy(cfg.copy()).to(device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(device), cache, full_gradient=full)
    torch.cuda.synchronize()
    eng.raise_on_status()
    return res


def _compare(res, c2, ctx, le, truncating, full=False, margin_tol=1e-4, median_tol=TRUNC_MEDIAN_TOL,
             max_tol=TRUNC_MAX_TOL):
    cfg = res.configs.cpu().numpy()
    same = np.all(cfg == c2, axis=1)
    margin = res.margin.cpu().numpy()
    # chains that differ must have had a decision within margin_tol of its threshold
    assert np.all(same | (margin < margin_tol)), "configs differ away from any acceptance threshold"
    assert same.mean() > 0.9
    amp = (res.sign * torch.exp(res.logamp)).cpu().numpy()
    tol = dict(median_tol=median_tol, max_tol=max_tol)
    assert_parity(np.abs(amp[same] / ctx.amp[same] - 1), truncating, **tol)
    e, e_ref = res.E.cpu().numpy()[same], le.local_estimate[same]
    assert_parity(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref)), truncating, **tol)
    o, o_ref = res.O.cpu().numpy()[same], le.local_log_derivatives[same]
    assert_parity(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), truncating, **tol)
    if not full:
        assert np.array_equal(res.p.cpu().numpy()[same], le.active_slice_indices[same])


@pytest.mark.parametrize("shape,D,chi,strategy,model", CASES)
@pytest.mark.parametrize("full", [False, True])
def test_sweep_matches_oracle(cuda_device, shape, D, chi, strategy, model, full):
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, 32, seed=D + chi)
    res = _run(cuda_device, shape, D, chi, strategy, H, T, cfg, u, full)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    _compare(res, c2, ctx, le, strategy != "NoTruncation", full)


def test_config1_tfim_4x4_D2_chi4_256_chains(cuda_device):
    """The CPU-runnable configuration: 4x4 TFIM (J=1, h=3), D=2, ZipUp(4), 256 chains."""
    shape, D, chi = (4, 4), 2, 4
    H = hamiltonian("tfim", shape)
    T, cfg, u = make_case(shape, D, 256, seed=0)
    res = _run(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    _compare(res, c2, ctx, le, True)


def test_config2_heisenberg_8x8_D4_chi16_subset(cuda_device):
    """8x8 Heisenberg, D=4, ZipUp(16): 24 chains against the oracle (full-size runs use properties)."""
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 24, seed=0)
    res = _run(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    _compare(res, c2, ctx, le, True, median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    # the batch mean is dominated by the few samples with a near-degenerate cut
    # (measured on sm_103a: 6.5e-4 over these 24 chains)
    e_mean, e_ref = res.E.cpu().numpy()[same].mean(), le.local_estimate[same].mean()
    assert abs(e_mean - e_ref) / abs(e_ref) < 2e-3


def test_config2_variational_8x8_D4_chi16(cuda_device):
    """8x8 Heisenberg, D=4, Variational(16) with 2 sweeps, 64 chains against the oracle.  The QR/ALS
    compression has no eigen-gap amplification, so the FP32 tier meets the accuracy bars here (measured
    on sm_103a: batch-mean E 1.1e-6 of the energy scale, O_k 2.5e-5; on 256 other chains 3.6e-6 and
    5.9e-5)."""
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 64, seed=0)
    res = _run(cuda_device, shape, D, chi, "Variational", H, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "Variational", chi, H, cfg, u)
    acc = accuracy(res, c2, ctx, le)
    assert acc["same_configs"] >= 0.9, acc
    assert acc["amp_rel_median"] < 1e-4 and acc["amp_rel_max"] < 1e-2, acc
    assert acc["e_mean_scaled"] < E_BAR and acc["eloc_rel_max"] < 1e-2, acc
    assert acc["o_frob"] < O_BAR, acc


def test_amp_grad_and_local_energy_match_oracle(cuda_device):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, 48, seed=5)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = eng.amp_grad(tens, c, full_gradient=False)
    e = eng.local_energy(tens, c, la, sg)
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert_parity(np.abs((sg * torch.exp(la)).cpu().numpy() / amp - 1), True)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(e.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


@pytest.mark.parametrize("opts", [{"vchunk": 1, "vert_smem": 1}, {"trunc_method": "jacobi"}, {"smem_kb": 0},
                                  {"smem_kb": 24}, {"threads": 256, "smem_kb": 96}],
                         ids=["chunk1", "jacobi", "all-global", "mat-global", "256-threads"])
def test_alternative_engine_paths(cuda_device, opts):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 32, seed=21)
    res = _run(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u, options=opts)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    _compare(res, c2, ctx, le, True)


def test_two_sweeps_match_oracle_sampler(cuda_device):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 32, seed=11)
    u2 = np.random.default_rng(12).random(u.shape)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg.copy()).to(cuda_device)
    cache = eng.init_cache(tens, c)
    eng.sweep(tens, c, torch.from_numpy(u).to(cuda_device), cache)
    res = eng.sweep(tens, c, torch.from_numpy(u2).to(cuda_device), cache)
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    init, trans, est = oracle.build_mc_kernels(model, H)
    sampler = oracle.make_mc_sampler(trans, est)
    (cfg_o, _), (_, le, _) = sampler(fp32(T), cfg.astype(np.int64), np.stack([u, u2]),
                                     init(fp32(T), cfg.astype(np.int64)), n_steps=2)
    same = np.all(res.configs.cpu().numpy() == cfg_o, axis=1)
    assert same.mean() > 0.9
    e_ref = le.local_estimate[1][same]
    assert_parity(np.abs(res.E.cpu().numpy()[same] - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


COMPLEX_CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((4, 4), 3, 6, "ZipUp", "tfim"),
    ((4, 4), 3, 6, "ZipUp", "heisenberg"),
    ((3, 4), 2, 3, "Variational", "heisenberg"),
]


@pytest.mark.parametrize("shape,D,chi,strategy,model", COMPLEX_CASES)
@pytest.mark.parametrize("full", [False, True])
def test_complex_sweep_matches_oracle(cuda_device, shape, D, chi, strategy, model, full):
    """complex64 PEPS against the complex128 oracle (amplitude log|psi| + i phase, complex O_k, E_loc)."""
    H = hamiltonian(model, shape)
    T = complex_tensors(shape, D, seed=D + chi)
    n_sites = shape[0] * shape[1]
    rng = np.random.default_rng(3)
    cfg = rng.integers(0, 2, (32, n_sites)).astype(np.int32)
    u = rng.random((32, n_sites))
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device=cuda_device, dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg.copy()).to(cuda_device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(cuda_device), cache, full_gradient=full)
    torch.cuda.synchronize()
    eng.raise_on_status()
    c2, ctx, le = oracle_sweep(T, shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    assert np.all(same | (res.margin.cpu().numpy() < 1e-4)) and same.mean() > 0.9
    trunc = strategy != "NoTruncation"
    amp = np.exp(res.logamp.cpu().numpy() + 1j * res.sign.cpu().numpy())
    assert_parity(np.abs(amp[same] / ctx.amp[same] - 1), trunc)
    e, e_ref = res.E.cpu().numpy()[same], le.local_estimate[same]
    assert_parity(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref)), trunc)
    o, o_ref = res.O.cpu().numpy()[same], le.local_log_derivatives[same]
    assert_parity(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), trunc)
