"""Calls over zero chains (the reference vmaps over a batch axis of any length, including 0): every
entry point returns VMC_OK with empty outputs, through the Python engine and through the C ABI with null
buffers; the VJP of no samples is zero.  Host emulation of the kernels: no GPU needed."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from tests.helpers import complex_tensors, hamiltonian, make_case
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors


@pytest.mark.parametrize("precision,dtype", [("fp32", "float32"), ("mixed", "float32"), ("fp32", "complex64")])
def test_engine_calls_over_zero_chains(emu_lib, precision, dtype):
    shape, D, chi = (3, 3), 2, 4
    H = hamiltonian("heisenberg", shape)
    T = complex_tensors(shape, D, seed=1) if dtype == "complex64" else make_case(shape, D, 1, seed=1)[0]
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib, dtype=dtype,
                     options={"precision": precision})
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.zeros((0, 9), dtype=torch.int32)
    u = torch.zeros((0, eng.n_draws), dtype=torch.float64)
    cache = eng.init_cache(tens, c)
    assert cache.numel() == 0
    for cch in (cache, None):  # cached and recomputing sweeps
        res = eng.sweep(tens, c, u, cch)
        assert res.configs.shape == (0, 9) and res.O.shape == (0, eng.n_params_sliced)
        assert res.E.shape == (0,) and res.logamp.shape == (0,)
    la, sg, O = eng.amp_grad(tens, c, full_gradient=True)
    assert la.shape == (0,) and O.shape == (0, eng.n_params_full)
    assert eng.local_energy(tens, c, la, sg).shape == (0,)
    g = eng.vjp(tens, c, torch.zeros(0, dtype=torch.float64))
    assert g.shape == (eng.n_params_full,) and not bool(g.abs().any())
    assert eng.status() == 0


def test_c_abi_accepts_null_buffers_over_zero_chains(emu_lib):
    shape, D, chi = (3, 3), 2, 4
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("tfim", shape), device="cpu", lib=emu_lib)
    lib, pl, null = emu_lib, eng._plan, None
    assert lib.vmc_peps_init_cache(pl, null, null, null, 0, null, null, 0, null) == _abi.VMC_OK
    assert lib.vmc_peps_sweep(pl, null, null, null, null, null, 0, null, 0, null, null, null, null, null, null,
                              null, null, 0, null) == _abi.VMC_OK
    assert lib.vmc_peps_sweep_recompute(pl, null, null, null, null, null, 0, 0, null, null, null, null, null, null,
                                        null, null, 0, null) == _abi.VMC_OK
    assert lib.vmc_peps_amp_grad(pl, null, null, null, 0, 0, null, null, null, null, null, 0, null) == _abi.VMC_OK
    assert lib.vmc_peps_amp_grad_noalloc(pl, null, null, null, 0, 0, null, null, null, null, null) == _abi.VMC_OK
    assert lib.vmc_peps_local_energy(pl, null, null, null, 0, null, null, null, null, 0, null) == _abi.VMC_OK
    grad = np.full(eng.n_params_full, 7.0)
    gp = grad.ctypes.data_as(ct.c_void_p)
    assert lib.vmc_peps_vjp(pl, null, null, null, 0, null, gp, null, 0, null) == _abi.VMC_OK
    assert not grad.any()
    # the VJP needs its output even over no samples; a negative count stays invalid
    assert lib.vmc_peps_vjp(pl, null, null, null, 0, null, null, null, 0, null) == _abi.VMC_ERR_INVALID
    assert lib.vmc_peps_amp_grad(pl, null, null, null, -1, 0, null, null, null, null, null, 0, null) == \
        _abi.VMC_ERR_INVALID
    # one chain with null buffers is still refused
    assert lib.vmc_peps_amp_grad(pl, null, null, null, 1, 0, null, null, null, null, null, 0, null) == \
        _abi.VMC_ERR_INVALID
