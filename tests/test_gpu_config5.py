"""The larger lattices and bond dimensions of the uneven-batch workload (Heisenberg, real FP32):
6x6 D=4 chi=16 and 8x8 D=5 chi=25 against the FP64 oracle on a few chains; 12x12 D=6 chi=36 and
16x16 D=6 chi=48 (truncation matrices of 216 and 288, arena in global memory) through properties
that hold exactly at any size."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import (CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, assert_parity, fp32, hamiltonian, make_case,
                           oracle_sweep)
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors, params_per_site
from vmc_gb300.synthetic import random_tensors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,D,chi,n", [((6, 6), 4, 16, 8), ((8, 8), 5, 25, 4)])
def test_amplitudes_gradients_energies_match_oracle(cuda_device, shape, D, chi, n):
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, n, seed=3)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, sg)
    torch.cuda.synchronize()
    eng.raise_on_status()
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    assert_parity(np.abs((sg * torch.exp(la)).cpu().numpy() / amp - 1), True, **tol)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.cpu().numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True, **tol)
    assert_parity(np.abs(E.cpu().numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True, **tol)


def test_sweep_6x6_matches_oracle(cuda_device):
    shape, D, chi = (6, 6), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 8, seed=4)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg.copy()).to(cuda_device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(cuda_device), cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    same = np.all(res.configs.cpu().numpy() == c2, axis=1)
    assert np.all(same | (res.margin.cpu().numpy() < 1e-4)) and same.mean() > 0.7
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    amp = (res.sign * torch.exp(res.logamp)).cpu().numpy()
    assert_parity(np.abs(amp[same] / ctx.amp[same] - 1), True, **tol)
    e_ref = le.local_estimate[same]
    assert_parity(np.abs(res.E.cpu().numpy()[same] - e_ref) / np.maximum(1.0, np.abs(e_ref)), True, **tol)


@pytest.mark.parametrize("shape,D,chi", [((12, 12), 6, 36), ((16, 16), 6, 48)])
def test_large_shapes_exact_properties(cuda_device, shape, D, chi):
    """u = 0 accepts every proposal (one sweep flips every site); outputs are finite; sum A.O over the
    sites of a row is one value per row and 1 on the last row."""
    R, C = shape
    n = 8
    H = hamiltonian("heisenberg", shape)
    T = random_tensors(shape, D, seed=0)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    cfg = torch.from_numpy(np.random.default_rng(5).integers(0, 2, (n, R * C)).astype(np.int32)).to(cuda_device)
    c = cfg.clone()
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.zeros((n, R * C), dtype=torch.float64, device=cuda_device), cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    assert torch.equal(res.configs, 1 - cfg)
    assert torch.isfinite(res.E).all() and torch.isfinite(res.O).all() and torch.isfinite(res.logamp).all()
    pps = params_per_site(shape, D)
    off, vals = 0, []
    for site in range(R * C):
        r, col = divmod(site, C)
        A = torch.from_numpy(np.asarray(T[r][col], dtype=np.float32)).to(cuda_device).reshape(2, -1)
        vals.append((A[res.configs[:, site].long()] * res.O[:, off:off + pps[site]]).sum(1).double())
        off += pps[site]
    v = torch.stack(vals, 1).reshape(n, R, C)
    assert float((v[:, R - 1, :] - 1).abs().max()) < 1e-3
    mean = v.mean(dim=2, keepdim=True)
    spread = (v - mean).abs().amax(dim=2) / mean.abs().squeeze(2).clamp_min(1e-2)
    assert float(spread.median()) < 1e-3
