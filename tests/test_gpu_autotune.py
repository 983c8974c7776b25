"""The autotuner on the GPU: every candidate launch configuration runs and matches the FP64 oracle,
and an engine built with options="auto" uses the cached winner."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, assert_parity, fp32, hamiltonian, make_case
from vmc_gb300.autotune import CANDIDATES, tune
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("options", CANDIDATES)
def test_candidate_matches_oracle(cuda_device, options):
    shape, D, chi = (6, 6), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, 6, seed=12)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device, options=options)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, sg)
    torch.cuda.synchronize()
    eng.raise_on_status()
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    assert_parity(np.abs((sg * torch.exp(la)).cpu().numpy() / amp - 1), True, **tol)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True, **tol)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(E.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True, **tol)


def test_tune_then_auto(cuda_device, tmp_path, monkeypatch):
    monkeypatch.setenv("VMC_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    entry = tune((6, 6), 4, 16, device=cuda_device)
    rates = [c["samples_per_s"] for c in entry["candidates"]]
    assert len(rates) == len(CANDIDATES) and min(rates) > 0 and entry["samples_per_s"] == max(rates)
    eng = PEPSEngine((6, 6), 4, 16, 2, "ZipUp", operator=hamiltonian("heisenberg", (6, 6)), device=cuda_device,
                     options="auto")
    assert eng.options == entry["options"]


@pytest.mark.parametrize("policy", [3, 4], ids=["mma-sync", "tcgen05"])
@pytest.mark.parametrize("threads", [128, 256])
def test_tensor_core_policy_at_large_bonds(cuda_device, threads, policy):
    """tile_policies 3 (3xTF32 mma.sync GEMMs) and 4 (3xTF32 tcgen05 GEMMs, accumulators in tensor memory)
    where their GEMMs engage: 4x4, D=6, chi=36 against the FP64 oracle, with the bars of an active
    truncation (the FFMA tiles give a median of 3e-6 and a maximum of 8e-5 on these samples)."""
    shape, D, chi = (4, 4), 6, 36
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, 6, seed=21)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device,
                     options={"threads": threads, "smem_kb": -1, "tile_policy": policy})
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, sg)
    torch.cuda.synchronize()
    eng.raise_on_status()
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert_parity(np.abs((sg * torch.exp(la)).cpu().numpy() / amp - 1), True)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(E.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)
