"""The mixed-precision tier on sm_103a (via the C ABI) against the FP64 oracle.

The boundary-MPS chain (zip-up theta, its truncation, the stored boundary
tensors) runs in FP64 and everything else in FP32, so amplitudes agree with
the oracle at the FP64 level and energies / log-derivatives at the FP32 level.
At 8x8, D=4, chi=16 that meets the accuracy bars -- batch-mean E within 1e-5
of the energy scale mean|E_loc|, O_k within 1e-4 Frobenius over the batch --
which the FP32 tier misses (its truncations move by eps_fp32 / relative gap).
"""
from __future__ import annotations

import json

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import (E_BAR, EXACT_TOL, MIXED_AMP_TOL, O_BAR, accuracy, fp32, hamiltonian, make_case,
                           oracle_sweep)
from vmc_gb300.engine import PEPSBatch, PEPSEngine
from vmc_gb300.lowering import pack_tensors

pytestmark = pytest.mark.gpu

MIXED = {"precision": "mixed"}


def _sweep(device, shape, D, chi, strategy, H, T, cfg, u, options, full=False):
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device=device, options=options)
    tens = torch.from_numpy(pack_tensors(T)).to(device)
    c = torch.from_numpy(cfg.copy()).to(device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(device), cache, full_gradient=full)
    torch.cuda.synchronize()
    eng.raise_on_status()
    return eng, res


CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((3, 3), 3, 4, "ZipUp", "heisenberg"),
    ((4, 4), 2, 4, "ZipUp", "tfim"),
    ((4, 4), 3, 6, "ZipUp", "heisenberg"),
    ((6, 6), 4, 16, "ZipUp", "heisenberg"),
    ((4, 4), 3, 3, "DensityMatrix", "heisenberg"),
]


@pytest.mark.parametrize("shape,D,chi,strategy,model", CASES)
@pytest.mark.parametrize("full", [False, True])
def test_mixed_sweep_matches_oracle(cuda_device, shape, D, chi, strategy, model, full):
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, 32, seed=D + chi)
    _, res = _sweep(cuda_device, shape, D, chi, strategy, H, T, cfg, u, MIXED, full)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    assert np.all(same | (res.margin.cpu().numpy() < 1e-4)) and same.mean() > 0.9
    acc = accuracy(res, c2, ctx, le)
    assert acc["amp_rel_max"] < MIXED_AMP_TOL, acc
    assert acc["eloc_rel_max"] < 5 * EXACT_TOL, acc
    assert acc["o_frob"] < EXACT_TOL, acc


@pytest.mark.parametrize("opts", [{"smem_kb": 0}, {"smem_kb": 200, "threads": 256}, {"threads": 64}],
                         ids=["arena-in-slot", "arena-in-smem-256", "64-threads"])
def test_mixed_launch_configurations_match_oracle(cuda_device, opts):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 32, seed=21)
    _, res = _sweep(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u, dict(MIXED, **opts))
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    acc = accuracy(res, c2, ctx, le)
    assert acc["same_configs"] > 0.9 and acc["amp_rel_max"] < MIXED_AMP_TOL and acc["o_frob"] < EXACT_TOL, acc


def test_mixed_amp_grad_local_energy_and_recompute(cuda_device):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 48, seed=5)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device, options=MIXED)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = eng.amp_grad(tens, c, full_gradient=False)
    e = eng.local_energy(tens, c, la, sg)
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert np.max(np.abs((sg * torch.exp(la)).cpu().numpy() / amp - 1)) < MIXED_AMP_TOL
    o_ref = grads / amp[:, None]
    assert np.max(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < EXACT_TOL
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert np.max(np.abs(e.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref))) < 5 * EXACT_TOL
    # recomputed bottom rows give the bits of init_cache + sweep
    c1 = torch.from_numpy(cfg.copy()).to(cuda_device)
    cache = eng.init_cache(tens, c1)
    ref = eng.sweep(tens, c1, torch.from_numpy(u).to(cuda_device), cache)
    c2 = torch.from_numpy(cfg.copy()).to(cuda_device)
    rec = eng.sweep(tens, c2, torch.from_numpy(u).to(cuda_device), None)
    torch.cuda.synchronize()
    assert torch.equal(ref.configs, rec.configs) and torch.equal(ref.E, rec.E) and torch.equal(ref.O, rec.O)


def test_mixed_plans_batch_with_the_single_call_bits(cuda_device):
    specs = [((4, 4), 3, 6, 40, 3), ((6, 6), 4, 16, 24, 4)]
    jobs, refs = [], []
    for shape, D, chi, n, seed in specs:
        H = hamiltonian("heisenberg", shape)
        T, cfg, u = make_case(shape, D, n, seed=seed)
        eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device, options=MIXED)
        tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
        uu = torch.from_numpy(u).to(cuda_device)
        c = torch.from_numpy(cfg.copy()).to(cuda_device)
        cache = eng.init_cache(tens, c)
        refs.append(eng.sweep(tens, c.clone(), uu, cache.clone()))
        cache2 = eng.init_cache(tens, torch.from_numpy(cfg.copy()).to(cuda_device))
        jobs.append(eng.sweep_job(tens, torch.from_numpy(cfg.copy()).to(cuda_device), uu, cache2))
    outs = PEPSBatch().run(jobs)
    torch.cuda.synchronize()
    for ref, out in zip(refs, outs):
        assert torch.equal(ref.configs, out.configs) and torch.equal(ref.E, out.E) and torch.equal(ref.O, out.O)


def test_config2_mixed_meets_the_accuracy_bar_on_256_chains(cuda_device):
    """8x8 Heisenberg, D=4, chi=16, ZipUp(16), 256 chains, one sweep: the mixed tier meets both bars;
    the FP32 tier's errors on the same chains are measured beside it and reported."""
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 256, seed=0)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    _, res = _sweep(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u, MIXED)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    assert np.all(same | (res.margin.cpu().numpy() < 1e-4)) and same.mean() > 0.95
    acc = accuracy(res, c2, ctx, le)
    _, res32 = _sweep(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u, None)
    acc32 = accuracy(res32, c2, ctx, le)
    print(json.dumps({"mixed": acc, "fp32": acc32}))
    assert acc["amp_rel_max"] < MIXED_AMP_TOL, acc
    assert acc["e_mean_scaled"] < E_BAR, acc
    assert acc["o_frob"] < O_BAR, acc
    assert acc32["o_frob"] > 10 * acc["o_frob"], (acc, acc32)


def test_mixed_tier_at_8x8_D5_chi25(cuda_device):
    """8x8 Heisenberg, D=5, ZipUp(25) (125 x 125 truncations), 16 chains: the double-float chain keeps
    the amplitudes at ~1e-11 and O_k at ~1e-6; E_loc carries the FP32 energy contractions' rounding,
    which grows with D (host emulation of the same chains: per sample up to 9e-5)."""
    shape, D, chi = (8, 8), 5, 25
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 16, seed=7)
    _, res = _sweep(cuda_device, shape, D, chi, "ZipUp", H, T, cfg, u, MIXED)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    acc = accuracy(res, c2, ctx, le)
    assert acc["same_configs"] >= 0.9, acc
    assert acc["amp_rel_max"] < MIXED_AMP_TOL * 100, acc
    assert acc["o_frob"] < 1e-5, acc
    assert acc["eloc_rel_max"] < 1e-3 and acc["e_mean_scaled"] < 1e-4, acc
