"""The mixed-precision tier (boundary-MPS chain in double-float, FP32 elsewhere) in the host-emulation build
against the FP64 oracle: amplitudes at the FP64 level, energies and log-derivatives at the FP32
level, and at 8x8, D=4, chi=16 the accuracy bars (batch-mean E within 1e-5 of the energy scale,
O_k within 1e-4 Frobenius over the batch) that the FP32 tier misses."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from tests.helpers import (E_BAR, EXACT_TOL, MIXED_AMP_TOL, O_BAR, accuracy, fp32, hamiltonian, make_case,
                           oracle_sweep)
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

MIXED = {"precision": "mixed"}


def _sweep(emu_lib, shape, D, chi, strategy, H, T, cfg, u, options, full=False):
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib, options=options)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, full_gradient=full)
    assert eng.status() == 0
    return eng, res


CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((3, 3), 3, 4, "ZipUp", "heisenberg"),
    ((4, 4), 2, 4, "ZipUp", "tfim"),
    ((4, 4), 3, 6, "ZipUp", "heisenberg"),
    ((3, 4), 2, 3, "ZipUp", "heisenberg"),
]


@pytest.mark.parametrize("shape,D,chi,strategy,model", CASES)
@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("smem_kb", [0, -1, 200], ids=["arena-in-slot", "default-budget", "arena-in-smem"])
def test_mixed_sweep_matches_oracle(emu_lib, shape, D, chi, strategy, model, full, smem_kb):
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, 6, seed=D + chi)
    _, res = _sweep(emu_lib, shape, D, chi, strategy, H, T, cfg, u, dict(MIXED, smem_kb=smem_kb), full)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    assert np.array_equal(res.configs.numpy(), c2)
    acc = accuracy(res, c2, ctx, le)
    assert acc["amp_rel_max"] < MIXED_AMP_TOL, acc
    assert acc["eloc_rel_max"] < EXACT_TOL, acc
    o, o_ref = res.O.numpy(), le.local_log_derivatives
    assert np.max(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < EXACT_TOL


def test_mixed_amp_grad_and_local_energy_match_oracle(emu_lib):
    from oracle import peps as oracle

    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, 5, seed=5)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib, options=MIXED)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    la, sg, O = eng.amp_grad(tens, c, full_gradient=False)
    e = eng.local_energy(tens, c, la, sg).numpy()
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert np.max(np.abs((sg * torch.exp(la)).numpy() / amp - 1)) < MIXED_AMP_TOL
    o_ref = grads / amp[:, None]
    assert np.max(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < EXACT_TOL
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert np.max(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref))) < EXACT_TOL


def test_config2_mixed_meets_the_accuracy_bar_where_fp32_does_not(emu_lib):
    """8x8 Heisenberg, D=4, chi=16, ZipUp(16), 6 chains: the double-float chain takes the amplitudes to the
    FP64 level and the batch-mean E and O_k inside the bars; the FP32 tier's truncations move them by
    eps_fp32 / (relative gap) and miss both."""
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 6, seed=0)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    _, res = _sweep(emu_lib, shape, D, chi, "ZipUp", H, T, cfg, u, MIXED)
    acc = accuracy(res, c2, ctx, le)
    assert acc["same_configs"] == 1.0
    assert acc["amp_rel_max"] < MIXED_AMP_TOL, acc
    assert acc["e_mean_scaled"] < E_BAR, acc
    assert acc["o_frob"] < O_BAR, acc
    _, res32 = _sweep(emu_lib, shape, D, chi, "ZipUp", H, T, cfg, u, None)
    acc32 = accuracy(res32, c2, ctx, le)
    assert acc32["amp_rel_max"] > 100 * acc["amp_rel_max"]
    assert acc32["o_frob"] > 10 * acc["o_frob"]


@pytest.mark.parametrize("dtype,strategy,opts", [
    (_abi.VMC_DTYPE_C64, _abi.VMC_STRATEGY_ZIP_UP, {}),
    (_abi.VMC_DTYPE_F32, _abi.VMC_STRATEGY_VARIATIONAL, {}),
    (_abi.VMC_DTYPE_F32, _abi.VMC_STRATEGY_ZIP_UP, {"trunc_method": 1}),
    (_abi.VMC_DTYPE_F32, _abi.VMC_STRATEGY_ZIP_UP, {"tile_policy": 3}),
], ids=["complex", "variational", "jacobi", "tensor-core-tiles"])
def test_mixed_precision_plans_outside_its_scope_are_refused(emu_lib, dtype, strategy, opts):
    o = _abi.plan_options(dict(MIXED, **opts))
    plan = ct.c_void_p()
    st = emu_lib.vmc_peps_plan_ex(ct.byref(_abi.VmcShape(4, 4)), 3, 6, 2, dtype, strategy, 2, ct.byref(o),
                                  ct.byref(plan))
    assert st == _abi.VMC_ERR_UNSUPPORTED
    st = emu_lib.vmc_gi_plan(ct.byref(_abi.VmcShape(3, 3)), 2, 2, 4, _abi.VMC_DTYPE_F32, _abi.VMC_STRATEGY_ZIP_UP,
                             2, ct.byref(_abi.plan_options(MIXED)), ct.byref(plan))
    assert st == _abi.VMC_ERR_UNSUPPORTED


@pytest.mark.parametrize("dtype,opts,gi", [
    (_abi.VMC_DTYPE_C64, {}, False),
    (_abi.VMC_DTYPE_F32, {"threads": 64}, False),
    (_abi.VMC_DTYPE_F32, {"precision": "mixed"}, False),
    (_abi.VMC_DTYPE_F32, {}, True),
], ids=["complex", "two-warps", "mixed", "gi"])
def test_tcgen05_tiles_outside_their_scope_are_refused(emu_lib, dtype, opts, gi):
    """tile_policy 4 runs real FP32 standard plans in CTAs of at least four warps (one per TMEM lane
    quadrant of the 128-row accumulator)."""
    o = _abi.plan_options(dict({"tile_policy": 4}, **opts))
    plan = ct.c_void_p()
    if gi:
        st = emu_lib.vmc_gi_plan(ct.byref(_abi.VmcShape(3, 3)), 2, 2, 4, dtype, _abi.VMC_STRATEGY_ZIP_UP, 2,
                                 ct.byref(o), ct.byref(plan))
    else:
        st = emu_lib.vmc_peps_plan_ex(ct.byref(_abi.VmcShape(4, 4)), 3, 6, 2, dtype, _abi.VMC_STRATEGY_ZIP_UP, 2,
                                      ct.byref(o), ct.byref(plan))
    assert st == _abi.VMC_ERR_UNSUPPORTED
    st = emu_lib.vmc_peps_plan_ex(ct.byref(_abi.VmcShape(4, 4)), 3, 6, 2, _abi.VMC_DTYPE_F32,
                                  _abi.VMC_STRATEGY_ZIP_UP, 2, ct.byref(_abi.plan_options({"tile_policy": 4})),
                                  ct.byref(plan))
    assert st == _abi.VMC_OK
    emu_lib.vmc_plan_destroy(plan)


def test_invalid_plan_options_are_rejected(emu_lib):
    for bad in ({"precision": 2}, {"trunc_method": 2}, {"vchunk": -1}, {"vert_smem": -1}, {"tile_policy": 5},
                {"precision": 2, "tile_policy": 4}):
        plan = ct.c_void_p()
        st = emu_lib.vmc_peps_plan_ex(ct.byref(_abi.VmcShape(4, 4)), 3, 6, 2, _abi.VMC_DTYPE_F32,
                                      _abi.VMC_STRATEGY_ZIP_UP, 2, ct.byref(_abi.plan_options(bad)), ct.byref(plan))
        assert st == _abi.VMC_ERR_INVALID, bad
