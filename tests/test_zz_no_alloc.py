"""vmc_peps_amp_grad_noalloc (a variant of vmc_peps_amp_grad whose workspace is a fixed device
array of the library) against vmc_peps_amp_grad, through the C ABI.  Collected last on purpose:
it must pass on a device that earlier tests have used, as well as on its own."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from tests.helpers import hamiltonian, make_case
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

pytestmark = pytest.mark.gpu


def _vp(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(eng, tens, c, full):
    n = c.shape[0]
    dev = tens.device
    np_ = eng.n_params_full if full else eng.n_params_sliced
    O = torch.empty((n, np_), dtype=torch.float32, device=dev)
    la = torch.empty(n, dtype=torch.float64, device=dev)
    sg = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    st = eng.lib.vmc_peps_amp_grad_noalloc(eng._plan, eng._stream(), _vp(tens), _vp(c), n, int(full), _vp(O),
                                           _vp(la), _vp(sg), None, _vp(status))
    assert st == _abi.VMC_OK, eng.lib.vmc_status_string(st)
    return la, sg, O, status


@pytest.mark.parametrize("shape,D,chi,n", [((4, 4), 3, 6, 64), ((8, 8), 4, 16, 96)])
@pytest.mark.parametrize("full", [False, True])
def test_noalloc_equals_workspace_entry_point_on_two_consecutive_calls(cuda_device, shape, D, chi, n, full):
    T, cfg, _ = make_case(shape, D, n, seed=13)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device=cuda_device)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la0, sg0, O0 = eng.amp_grad(tens, c, full_gradient=full)
    for _ in range(2):
        la, sg, O, status = _noalloc(eng, tens, c, full)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        # each chain runs in one CTA whatever the grid, so the results are bitwise equal
        assert torch.equal(la, la0) and torch.equal(sg, sg0) and torch.equal(O, O0)


def test_noalloc_rejects_plans_larger_than_its_scratch(cuda_device):
    shape, D, chi = (16, 16), 6, 64   # one CTA slot alone exceeds 64 MiB
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", device=cuda_device)
    assert eng.lib.vmc_workspace_size(eng._plan, 1) > (64 << 20)
    tens = torch.zeros(eng.n_params_full, dtype=torch.float32, device=cuda_device)
    c = torch.zeros((2, 256), dtype=torch.int32, device=cuda_device)
    out = torch.empty(2, dtype=torch.float64, device=cuda_device)
    status = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    st = eng.lib.vmc_peps_amp_grad_noalloc(eng._plan, eng._stream(), _vp(tens), _vp(c), 2, 0, None, _vp(out),
                                           _vp(out), None, _vp(status))
    assert st == _abi.VMC_ERR_SCRATCH
    assert b"64 MiB" in eng.lib.vmc_status_string(st)
