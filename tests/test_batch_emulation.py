"""Uneven batches (vmc_peps_batch) in the host-emulation build: several plans -- lattices, bond
dimensions, strategies, element types of one kind -- in one launch give, chain for chain, the bits
of the single calls, and malformed batches return status codes without launching."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from tests.helpers import complex_tensors, hamiltonian, make_case
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSBatch, PEPSEngine
from vmc_gb300.lowering import pack_tensors

# (shape, D, chi, strategy, model, n_chains): uneven lattices, bonds and strategies
JOBS = [
    ((3, 3), 2, 4, "ZipUp", "heisenberg", 5),
    ((4, 4), 3, 6, "Variational", "tfim", 3),
    ((3, 4), 2, 3, "ZipUp", "heisenberg", 4),
    ((2, 3), 2, 16, "NoTruncation", "tfim", 2),
]


def _setup(emu_lib, spec, seed, dtype="float32"):
    shape, D, chi, strategy, model, n = spec
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, n, seed=seed)
    if dtype == "complex64":
        T = complex_tensors(shape, D, seed=seed)
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib, dtype=dtype)
    return eng, torch.from_numpy(pack_tensors(T)), torch.from_numpy(cfg), torch.from_numpy(u)


def _fields(res):
    return {k: getattr(res, k) for k in ("configs", "O", "p", "E", "logamp", "sign", "margin", "gap")
            if getattr(res, k) is not None}


def _assert_same_bits(a, b):
    fa, fb = _fields(a), _fields(b)
    assert fa.keys() == fb.keys()
    for k in fa:
        x, y = fa[k], fb[k]
        if x.is_complex():
            x, y = torch.view_as_real(x), torch.view_as_real(y)
        assert torch.equal(x.contiguous().view(torch.uint8), y.contiguous().view(torch.uint8)), k


@pytest.mark.parametrize("full", [False, True])
def test_uneven_sweeps_match_single_calls_bit_for_bit(emu_lib, full):
    cases = [_setup(emu_lib, spec, seed=3 + i) for i, spec in enumerate(JOBS)]
    singles, batch_jobs = [], []
    for eng, tens, cfg, u in cases:
        cache = eng.init_cache(tens, cfg.clone())
        cache_b = cache.clone()
        singles.append((eng.sweep(tens, cfg.clone(), u, cache, full_gradient=full), cache))
        batch_jobs.append(eng.sweep_job(tens, cfg.clone(), u, cache_b, full_gradient=full))
    batch = PEPSBatch()
    outs = batch.run(batch_jobs)
    assert batch.status() == 0
    for (eng, tens, cfg, u), (ref, cache), job, out in zip(cases, singles, batch_jobs, outs):
        _assert_same_bits(ref, out)
        # the caches differ only in the padding of each environment tensor, which nothing reads:
        # the next sweep from either gives the same bits
        u2 = torch.flip(u, (0,)).contiguous()
        _assert_same_bits(eng.sweep(tens, ref.configs.clone(), u2, cache.clone()),
                          eng.sweep(tens, out.configs.clone(), u2, job.cache.clone()))


def test_every_job_kind_in_one_batch(emu_lib):
    (e1, t1, c1, u1), (e2, t2, c2, u2), (e3, t3, c3, _) = (
        _setup(emu_lib, spec, seed=20 + i) for i, spec in enumerate(JOBS[:3]))
    # single calls
    cache_ref = e1.init_cache(t1, c1.clone())
    la, sg, O, gap = e2.amp_grad(t2, c2, full_gradient=True, want_gap=True)
    la3, sg3, _ = e3.amp_grad(t3, c3, want_O=False)
    E3 = e3.local_energy(t3, c3, la3, sg3)
    # the same work as one batch, in another order
    jobs = [e3.local_energy_job(t3, c3, la3, sg3), e1.init_cache_job(t1, c1.clone()),
            e2.amp_grad_job(t2, c2, full_gradient=True, want_gap=True)]
    outs = PEPSBatch().run(jobs)
    _assert_same_bits(e1.sweep(t1, c1.clone(), u1, cache_ref), e1.sweep(t1, c1.clone(), u1, jobs[1].cache))
    assert torch.equal(outs[2].O, O) and torch.equal(outs[2].logamp, la) and torch.equal(outs[2].sign, sg)
    assert torch.equal(outs[2].gap, gap)
    assert torch.equal(outs[0].E, E3)


def test_complex_batch_matches_single_calls(emu_lib):
    cases = [_setup(emu_lib, spec, seed=40 + i, dtype="complex64") for i, spec in enumerate(JOBS[:3])]
    singles, jobs = [], []
    for eng, tens, cfg, u in cases:
        cache = eng.init_cache(tens, cfg.clone())
        cache_b = cache.clone()
        singles.append(eng.sweep(tens, cfg.clone(), u, cache))
        jobs.append(eng.sweep_job(tens, cfg.clone(), u, cache_b))
    for ref, out in zip(singles, PEPSBatch().run(jobs)):
        _assert_same_bits(ref, out)


def test_reruns_reuse_the_workspace(emu_lib):
    eng, tens, cfg, _ = _setup(emu_lib, JOBS[0], seed=7)
    b = PEPSBatch()
    b.run([eng.amp_grad_job(tens, cfg)])
    ws = b._ws.data_ptr()
    out = b.run([eng.amp_grad_job(tens, cfg)])[0]
    assert b._ws.data_ptr() == ws
    la, sg, O = eng.amp_grad(tens, cfg)
    assert torch.equal(out.O, O) and torch.equal(out.logamp, la)


def _job_array(jobs):
    return (_abi.VmcPepsJob * len(jobs))(*[j.c_struct() for j in jobs])


def test_malformed_batches_return_status_codes(emu_lib):
    eng, tens, cfg, u = _setup(emu_lib, JOBS[0], seed=9)
    ceng, ctens, ccfg, _ = _setup(emu_lib, JOBS[0], seed=9, dtype="complex64")
    status = torch.zeros(1, dtype=torch.int32)
    ws = torch.zeros(1 << 16, dtype=torch.uint8)

    def run(jobs, nbytes=None):
        arr = _job_array(jobs)
        n = len(jobs)
        return emu_lib.vmc_peps_batch(arr, n, None, ct.c_void_p(ws.data_ptr()),
                                      ws.numel() if nbytes is None else nbytes, ct.c_void_p(status.data_ptr()))

    good = eng.amp_grad_job(tens, cfg)
    # mixed element types
    assert run([good, ceng.amp_grad_job(ctens, ccfg)]) == _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_batch_workspace_size(_job_array([good, ceng.amp_grad_job(ctens, ccfg)]), 2) == 0
    # the same lattice on the tensor-core kernel (tile policy 3) cannot share the launch
    shape, D, chi, strategy, model, _ = JOBS[0]
    teng = PEPSEngine(shape, D, chi, 2, strategy, operator=hamiltonian(model, shape), device="cpu", lib=emu_lib,
                      options={"threads": 128, "smem_kb": -1, "tile_policy": 3})
    assert run([good, teng.amp_grad_job(tens, cfg)]) == _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_batch_workspace_size(_job_array([teng.amp_grad_job(tens, cfg)] * 2), 2) > 0
    # a sweep without uniforms, an unknown kind
    bad = eng.sweep_job(tens, cfg.clone(), u, eng.init_cache(tens, cfg.clone()))
    bad.uniforms = None
    assert run([good, bad]) == _abi.VMC_ERR_INVALID
    odd = eng.amp_grad_job(tens, cfg)
    odd.kind = 7
    assert run([odd]) == _abi.VMC_ERR_INVALID
    # too many jobs, none, a workspace that is too small
    assert run([good] * (_abi.VMC_MAX_BATCH_JOBS + 1)) == _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_peps_batch(None, 0, None, ct.c_void_p(ws.data_ptr()), ws.numel(),
                                  ct.c_void_p(status.data_ptr())) == _abi.VMC_ERR_INVALID
    need = emu_lib.vmc_batch_workspace_size(_job_array([good]), 1)
    assert need > 0 and run([good], nbytes=need - 1) == _abi.VMC_ERR_WORKSPACE
    # zero chains: nothing to launch
    empty = eng.amp_grad_job(tens, cfg[:0])
    assert run([empty]) == _abi.VMC_OK
    with pytest.raises(ValueError):
        PEPSBatch().run([good, ceng.amp_grad_job(ctens, ccfg)])


@pytest.mark.parametrize("full", [False, True])
def test_recomputing_sweeps_equal_init_cache_then_sweep(emu_lib, full):
    """A sweep without a cache recomputes the bottom environments in the launch: same bits as
    init_cache + sweep, alone and as a batch job next to a cached one."""
    cases = [_setup(emu_lib, spec, seed=60 + i) for i, spec in enumerate(JOBS[:3])]
    for eng, tens, cfg, u in cases:
        ref = eng.sweep(tens, cfg.clone(), u, eng.init_cache(tens, cfg.clone()), full_gradient=full)
        _assert_same_bits(ref, eng.sweep(tens, cfg.clone(), u, None, full_gradient=full))
    jobs, refs = [], []
    for i, (eng, tens, cfg, u) in enumerate(cases):
        cache = eng.init_cache(tens, cfg.clone())
        refs.append(eng.sweep(tens, cfg.clone(), u, cache.clone(), full_gradient=full))
        jobs.append(eng.sweep_job(tens, cfg.clone(), u, cache if i == 1 else None, full_gradient=full))
    for ref, out in zip(refs, PEPSBatch().run(jobs)):
        _assert_same_bits(ref, out)


@pytest.mark.parametrize("layout", ["slot", "shared"])
def test_either_batch_layout_gives_the_single_call_bits(emu_lib, layout):
    """The batch runs every plan either with its shared-memory buffer placement or with all buffers
    in the CTA slot (chosen by cost share); the placement moves data, not arithmetic."""
    cases = [_setup(emu_lib, spec, seed=80 + i) for i, spec in enumerate(JOBS)]
    refs, jobs = [], []
    for eng, tens, cfg, u in cases:
        cache = eng.init_cache(tens, cfg.clone())
        refs.append(eng.sweep(tens, cfg.clone(), u, cache.clone()))
        jobs.append(eng.sweep_job(tens, cfg.clone(), u, cache))
    for ref, out in zip(refs, PEPSBatch().run(jobs, layout=layout)):
        _assert_same_bits(ref, out)
