"""vmc_peps_amp_grad_noalloc in the host-emulation build (its fixed scratch array is host memory
there): the size check, the grid clamp to the CTA slots that fit the array, and equality with
vmc_peps_amp_grad.  The GPU test (test_zz_no_alloc.py) runs the same comparison on the device."""
from __future__ import annotations

import ctypes as ct

import torch

from tests.helpers import hamiltonian, make_case
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

SCRATCH = 64 << 20


def _vp(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(eng, tens, c, full):
    n = c.shape[0]
    np_ = eng.n_params_full if full else eng.n_params_sliced
    O = torch.empty((n, np_), dtype=torch.float32)
    la = torch.empty(n, dtype=torch.float64)
    sg = torch.empty(n, dtype=torch.float64)
    status = torch.zeros(1, dtype=torch.int32)
    st = eng.lib.vmc_peps_amp_grad_noalloc(eng._plan, None, _vp(tens), _vp(c), n, int(full), _vp(O), _vp(la),
                                           _vp(sg), None, _vp(status))
    return st, la, sg, O


def test_noalloc_gives_the_workspace_entry_points_bits(emu_lib):
    shape, D, chi = (4, 4), 3, 6
    T, cfg, _ = make_case(shape, D, 7, seed=13)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device="cpu",
                     lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    for full in (False, True):
        la0, sg0, O0 = eng.amp_grad(tens, c, full_gradient=full)
        for _ in range(2):
            st, la, sg, O = _noalloc(eng, tens, c, full)
            assert st == _abi.VMC_OK
            assert torch.equal(la, la0) and torch.equal(sg, sg0) and torch.equal(O, O0)


def test_noalloc_clamps_the_grid_to_the_slots_that_fit(emu_lib):
    """A plan whose slot fits the array only a few times still evaluates every chain (CTAs loop over
    chains), with the bits of the workspace entry point."""
    shape, D, chi = (8, 8), 5, 25
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device="cpu",
                     lib=emu_lib, options={"smem_kb": 0})
    one = eng.lib.vmc_workspace_size(eng._plan, 1)
    assert one < SCRATCH
    slot = eng.lib.vmc_workspace_size(eng._plan, 2) - one
    fit = (SCRATCH - (one - slot)) // slot
    n = int(min(fit + 1, eng.resident_chains + 1))
    assert n > fit or n > eng.resident_chains  # more chains than the clamp's CTAs
    T, cfg, _ = make_case(shape, D, n, seed=3)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    la0, sg0, O0 = eng.amp_grad(tens, c)
    st, la, sg, O = _noalloc(eng, tens, c, False)
    assert st == _abi.VMC_OK
    assert torch.equal(la, la0) and torch.equal(sg, sg0) and torch.equal(O, O0)


def test_noalloc_rejects_plans_larger_than_its_scratch(emu_lib):
    shape, D, chi = (16, 16), 6, 64   # one CTA slot alone exceeds 64 MiB
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", device="cpu", lib=emu_lib)
    assert eng.lib.vmc_workspace_size(eng._plan, 1) > SCRATCH
    tens = torch.zeros(eng.n_params_full, dtype=torch.float32)
    c = torch.zeros((2, 256), dtype=torch.int32)
    out = torch.empty(2, dtype=torch.float64)
    status = torch.zeros(1, dtype=torch.int32)
    st = eng.lib.vmc_peps_amp_grad_noalloc(eng._plan, None, _vp(tens), _vp(c), 2, 0, None, _vp(out), _vp(out), None,
                                           _vp(status))
    assert st == _abi.VMC_ERR_SCRATCH
