"""Lattices with a single row, a single column or a single site (no vertical or no horizontal bonds,
boundary MPS of one tensor): one transition + estimate of the engine (host emulation of the kernels)
against the FP64 oracle, for every strategy and both precision tiers."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import fp32, hamiltonian, make_case, oracle_sweep
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

SHAPES = [(1, 4), (4, 1), (1, 1), (2, 1), (1, 2), (2, 2)]
RUNS = [("ZipUp", 4, "fp32"), ("ZipUp", 4, "mixed"), ("NoTruncation", 16, "fp32"), ("NoTruncation", 16, "mixed"),
        ("Variational", 4, "fp32")]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("strategy,chi,precision", RUNS)
def test_degenerate_lattice_sweep_matches_oracle(emu_lib, shape, strategy, chi, precision):
    H = hamiltonian("tfim", shape)
    T, cfg, u = make_case(shape, 2, 3, seed=1)
    eng = PEPSEngine(shape, 2, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib,
                     options={"precision": precision})
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache)
    assert eng.status() == 0
    c2, ctx, le = oracle_sweep(fp32(T), shape, 2, strategy, chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert np.max(np.abs(amp / ctx.amp - 1)) < 1e-6
    e_ref = le.local_estimate
    assert np.max(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref))) < 1e-6
    o_ref = le.local_log_derivatives
    assert np.max(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < 1e-6
    assert np.array_equal(res.p.numpy(), le.active_slice_indices)


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("mixed", 1e-6)])
def test_largest_truncation_matches_oracle(emu_lib, precision, tol):
    """The largest cut a plan accepts: chi * D = 512 (4x6, D=8, chi=64; the boundary bond between the
    middle columns reaches D^3 = 512 before the cut keeps 64), one chain."""
    shape, D, chi = (4, 6), 8, 64
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 1, seed=2)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib,
                     options={"precision": precision})
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache)
    assert eng.status() == 0
    assert float(res.gap.min()) < 1.0  # a cut discarded eigenvalues
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert np.max(np.abs(amp / ctx.amp - 1)) < tol
    o_ref = le.local_log_derivatives
    assert np.max(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < tol
    # energies come from FP32 environments in both tiers
    e_ref = le.local_estimate
    assert np.max(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref))) < 1e-4


def test_plans_beyond_the_largest_truncation_are_refused(emu_lib):
    from vmc_gb300._abi import VmcError

    with pytest.raises(VmcError, match="not implement|unsupported"):
        PEPSEngine((4, 6), 8, 65, 2, "ZipUp", operator=None, device="cpu", lib=emu_lib)
