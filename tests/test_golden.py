"""Committed golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py).

CPU: the oracle still reproduces them and the seeded generator still yields
their inputs.  GPU: the CUDA engine reproduces them through the C ABI without
running the oracle (which cannot travel where no CPU time is budgeted).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, TRUNC_MAX_TOL, TRUNC_MEDIAN_TOL, assert_parity
from vmc_gb300.lowering import pack_tensors
from vmc_gb300.operators import heisenberg, transverse_field_ising
from vmc_gb300.synthetic import initial_configs, random_tensors, uniform_stream

GOLDEN = Path(__file__).parent / "golden"
NAMES = ["heis3x3_D2_exact", "tfim4x4_D2_chi4", "heis8x8_D4_chi16"]


def _load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def _spec(g):
    shape = tuple(int(x) for x in g["shape"])
    D, chi = int(g["bond_dim"]), int(g["chi"])
    return shape, D, chi, str(g["model"])


@pytest.mark.parametrize("name", NAMES)
def test_generator_reproduces_inputs(name):
    g = _load(name)
    shape, D, chi, _ = _spec(g)
    n = g["configs_in"].shape[0]
    assert np.array_equal(pack_tensors(random_tensors(shape, D, seed=0)), g["tensors"])
    assert np.array_equal(initial_configs(n, shape[0] * shape[1], seed=0), g["configs_in"])
    assert np.array_equal(next(uniform_stream(n, shape[0] * shape[1], seed=0)), g["uniforms"])


@pytest.mark.parametrize("name", ["heis3x3_D2_exact", "tfim4x4_D2_chi4"])
def test_oracle_reproduces_fixture(name):
    g = _load(name)
    shape, D, chi, model = _spec(g)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in random_tensors(shape, D, seed=0)]
    H = heisenberg(shape) if model == "heisenberg" else transverse_field_ising(shape)
    strat = oracle.NoTruncation() if chi == 0 else oracle.ZipUp(chi)
    om = oracle.PEPS(T, shape, D, strategy=strat)
    init, trans, est = oracle.build_mc_kernels(om, H)
    cfg = g["configs_in"].astype(np.int64)
    c2, ctx = trans(T, cfg, g["uniforms"], init(T, cfg))
    _, le = est(T, c2, ctx)
    assert np.array_equal(c2, g["configs_out"])
    assert np.allclose(ctx.amp, g["amp"], rtol=1e-10, atol=0)
    assert np.allclose(le.local_estimate, g["local_energy"], rtol=1e-9, atol=1e-12)


def test_config1_full_sum_energy_matches_boundary_mps_evaluation():
    """Second oracle (exact full sum over all 2^16 states of the 4x4 TFIM): the fixture's exact <H>
    equals sum |psi|^2 E_loc / sum |psi|^2 from the oracle's boundary-MPS evaluation (NoTruncation)."""
    from oracle import exact

    g = _load("tfim4x4_D2_chi4")
    shape = (4, 4)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in random_tensors(shape, 2, seed=0)]
    om = oracle.PEPS(T, shape, 2, strategy=oracle.NoTruncation())
    states = exact.all_configs(16)
    amps = oracle.value(om, states)
    e_loc = oracle.local_estimate(om, states, transverse_field_ising(shape), amps)
    w = amps ** 2
    assert abs(np.sum(w * e_loc) / np.sum(w) - g["exact_energy"]) < 1e-9 * abs(g["exact_energy"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_cuda_engine_reproduces_fixture(cuda_device, name):
    from vmc_gb300.engine import PEPSEngine

    g = _load(name)
    shape, D, chi, model = _spec(g)
    H = heisenberg(shape) if model == "heisenberg" else transverse_field_ising(shape)
    eng = PEPSEngine(shape, D, chi if chi else 16, 2, "ZipUp" if chi else "NoTruncation", operator=H,
                     device=cuda_device)
    tens = torch.from_numpy(g["tensors"]).to(cuda_device)
    cfg = torch.from_numpy(g["configs_in"]).to(cuda_device)
    cache = eng.init_cache(tens, cfg)
    res = eng.sweep(tens, cfg, torch.from_numpy(g["uniforms"]).to(cuda_device), cache)
    torch.cuda.synchronize()
    same = np.all(res.configs.cpu().numpy() == g["configs_out"], axis=1)
    assert np.all(same | (g["margin"] < 1e-4))
    amp = (res.sign * torch.exp(res.logamp)).cpu().numpy()
    trunc = chi != 0
    big = D == 4 and chi == 16
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL if big else TRUNC_MEDIAN_TOL,
               max_tol=CONFIG2_MAX_TOL if big else TRUNC_MAX_TOL)
    assert_parity(np.abs(amp[same] / g["amp"][same] - 1), trunc, **tol)
    e_ref = g["local_energy"][same]
    assert_parity(np.abs(res.E.cpu().numpy()[same] - e_ref) / np.maximum(1, np.abs(e_ref)), trunc, **tol)
    o_ref = g["log_derivatives"][same].astype(np.float64)
    assert_parity(np.linalg.norm(res.O.cpu().numpy()[same] - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), trunc,
                  **tol)
