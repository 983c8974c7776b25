"""The engine's device code, compiled for the host (one thread per CTA), against the FP64 oracle.

This checks every index map, buffer layout and control path of the fused
kernel on CPU; thread-level concurrency is covered by the -m gpu tests.
"""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import assert_parity, complex_tensors, fp32, hamiltonian, make_case, oracle_sweep
from vmc_gb300 import _abi
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors
from vmc_gb300.operators import LocalHamiltonian, OneSiteTerm, HorizontalTwoSiteTerm, VerticalTwoSiteTerm, DiagonalTerm


def _engine(emu_lib, shape, D, chi, strategy, H, d=2, options=None):
    return PEPSEngine(shape, D, chi, d, strategy, operator=H, device="cpu", lib=emu_lib, options=options)


def _sweep(eng, T, cfg, u, full=False, deltas=None):
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    d = None if deltas is None else torch.from_numpy(deltas.astype(np.int32))
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, deltas=d, full_gradient=full)
    return res, cache, tens


CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((2, 3), 3, 16, "NoTruncation", "tfim"),
    ((3, 3), 3, 4, "ZipUp", "heisenberg"),
    ((4, 4), 2, 4, "ZipUp", "tfim"),
    ((4, 4), 3, 6, "ZipUp", "heisenberg"),
    ((3, 4), 2, 3, "ZipUp", "heisenberg"),
    ((3, 3), 2, 4, "Variational", "heisenberg"),
    ((4, 4), 3, 6, "Variational", "tfim"),
    ((3, 4), 2, 3, "Variational", "heisenberg"),
]


@pytest.mark.parametrize("shape,D,chi,strategy,model", CASES)
@pytest.mark.parametrize("full", [False, True])
def test_sweep_matches_oracle(emu_lib, shape, D, chi, strategy, model, full):
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, 6, seed=D + chi)
    eng = _engine(emu_lib, shape, D, chi, strategy, H)
    res, _, _ = _sweep(eng, T, cfg, u, full=full)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    assert np.array_equal(res.configs.numpy(), c2)
    trunc = strategy != "NoTruncation"
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert_parity(np.abs(amp / ctx.amp - 1), trunc)
    e_ref = le.local_estimate
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), trunc)
    o_ref = le.local_log_derivatives
    assert_parity(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), trunc)
    if not full:
        assert np.array_equal(res.p.numpy(), le.active_slice_indices)
    assert eng.status() == 0


def test_two_sweeps_reuse_the_bottom_cache(emu_lib):
    """Cache turnover (REFACTOR.md:39-52): the estimate's bottom envs feed the next transition."""
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 5, seed=11)
    u2 = np.random.default_rng(12).random(u.shape)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    eng.sweep(tens, c, torch.from_numpy(u), cache)
    res = eng.sweep(tens, c, torch.from_numpy(u2), cache)
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    init, trans, est = oracle.build_mc_kernels(model, H)
    sampler = oracle.make_mc_sampler(trans, est)
    (cfg_o, _), (_, le, _) = sampler(fp32(T), cfg.astype(np.int64), np.stack([u, u2]),
                                     init(fp32(T), cfg.astype(np.int64)), n_steps=2)
    assert np.array_equal(res.configs.numpy(), cfg_o)
    e_ref = le.local_estimate[1]
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


def test_amp_grad_and_local_energy_match_oracle(emu_lib):
    shape, D, chi = (3, 4), 3, 5
    H = hamiltonian("heisenberg", shape)
    T, cfg, _ = make_case(shape, D, 7, seed=5)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    la, sg, O = eng.amp_grad(tens, c, full_gradient=False)
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert_parity(np.abs((sg * torch.exp(la)).numpy() / amp - 1), True)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)
    e = eng.local_energy(tens, c, la, sg).numpy()
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


@pytest.mark.parametrize("opts", [{"vchunk": 1, "vert_smem": 1}, {"trunc_method": "jacobi"}, {"smem_kb": 0},
                                  {"smem_kb": 24}, {"tile_policy": 1}, {"tile_policy": 2},
                                  {"threads": 128, "tile_policy": 4}],
                         ids=["chunk1", "jacobi", "all-global", "mat-global", "small-tiles", "large-tiles",
                              "tcgen05-plan"])
def test_alternative_engine_paths_match_oracle(emu_lib, opts):
    """Chunked vertical energy, the Jacobi truncation and the global-memory fallbacks agree with the oracle."""
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 4, seed=21)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H, options=opts)
    res, _, _ = _sweep(eng, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    e_ref = le.local_estimate
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)
    o_ref = le.local_log_derivatives
    assert_parity(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)


def test_density_matrix_is_not_the_zipup_product(emu_lib):
    """strategy.py:153-176 carries V_k^H without S_k, so its truncations differ from ZipUp's."""
    shape, D, chi = (4, 4), 3, 6
    T, cfg, _ = make_case(shape, D, 8, seed=31)
    zu = oracle.peps_apply(fp32(T), cfg, shape, oracle.ZipUp(chi))
    dm = oracle.peps_apply(fp32(T), cfg, shape, oracle.DensityMatrix(chi))
    assert np.max(np.abs(dm / zu - 1)) > 1e-3


DM_CASES = [((3, 3), 2, 2, "heisenberg", "fp32"), ((4, 4), 3, 3, "heisenberg", "fp32"), ((4, 4), 2, 2, "tfim", "fp32"),
            ((3, 4), 2, 2, "heisenberg", "fp32"), ((4, 4), 3, 3, "heisenberg", "mixed"), ((3, 4), 2, 2, "tfim", "mixed")]


@pytest.mark.parametrize("shape,D,chi,model,precision", DM_CASES)
def test_density_matrix_matches_oracle(emu_lib, shape, D, chi, model, precision):
    """DensityMatrix with chi <= D, where every kept eigenvector of rho = theta^H theta has a nonzero
    eigenvalue.  With more (chi > rank theta at a cut) the kept vectors include arbitrary null vectors of
    theta, and the reference's result depends on which ones its eigh returns."""
    H = hamiltonian(model, shape)
    T, cfg, u = make_case(shape, D, 6, seed=D + chi)
    eng = _engine(emu_lib, shape, D, chi, "DensityMatrix", H, options={"precision": precision})
    res, _, _ = _sweep(eng, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "DensityMatrix", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert np.max(np.abs(amp / ctx.amp - 1)) < (1e-9 if precision == "mixed" else 1e-4)
    e_ref = le.local_estimate
    assert np.max(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref))) < 5e-5
    o_ref = le.local_log_derivatives
    assert np.max(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < 5e-5
    assert eng.status() == 0


def test_complex_density_matrix_matches_oracle(emu_lib):
    shape, D, chi = (4, 4), 3, 3
    H = hamiltonian("tfim", shape)
    T = complex_tensors(shape, D, seed=7)
    rng = np.random.default_rng(7)
    cfg = rng.integers(0, 2, (5, 16)).astype(np.int32)
    u = rng.random((5, 16))
    eng = PEPSEngine(shape, D, chi, 2, "DensityMatrix", operator=H, device="cpu", lib=emu_lib, dtype="complex64")
    res, _, _ = _sweep(eng, T, cfg, u)
    c2, ctx, le = oracle_sweep(T, shape, D, "DensityMatrix", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    amp = np.exp(res.logamp.numpy() + 1j * res.sign.numpy())
    assert np.max(np.abs(amp / ctx.amp - 1)) < 1e-4
    o_ref = le.local_log_derivatives
    assert np.max(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1)) < 5e-5


def test_three_state_sites_with_explicit_flip_offsets(emu_lib):
    """d = 3: flip = (s + delta) % d with explicit offsets (kernels.py:170-175)."""
    shape, D, chi, d = (3, 3), 2, 4, 3
    rng = np.random.default_rng(8)
    ops = []
    for r in range(3):
        for c in range(3):
            m = rng.standard_normal((3, 3))
            ops.append(OneSiteTerm(r, c, m + m.T))
            if c < 2:
                h = rng.standard_normal((9, 9))
                ops.append(HorizontalTwoSiteTerm(r, c, h + h.T))
            if r < 2:
                v = rng.standard_normal((9, 9))
                ops.append(VerticalTwoSiteTerm(r, c, v + v.T))
    ops.append(DiagonalTerm(((0, 0), (2, 2)), rng.standard_normal(9)))
    H = LocalHamiltonian(shape, tuple(ops))
    T, cfg, u = make_case(shape, D, 5, seed=9, phys_dim=d)
    deltas = rng.integers(1, d, size=cfg.shape)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H, d=d)
    res, _, _ = _sweep(eng, T, cfg, u, deltas=deltas)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u, deltas=deltas)
    assert np.array_equal(res.configs.numpy(), c2)
    e_ref = le.local_estimate
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


def test_config2_shape_within_fp32_tolerance(emu_lib):
    """8x8, D=4, chi=16 (active truncation): FP32 engine vs FP64 oracle on 2 chains.

    The truncated zip-up is ill-conditioned (relative singular-value gaps at the
    cut down to ~1e-3), so the tolerance is the FP32 level amplified by 1/gap."""
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 2, seed=0)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H)
    res, _, _ = _sweep(eng, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    same = np.all(res.configs.numpy() == c2, axis=1)
    gap = res.gap.numpy()
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    for i in np.nonzero(same)[0]:
        tol = 5e-6 / max(float(gap[i]), 1e-4)
        assert abs(amp[i] / ctx.amp[i] - 1) < tol
        assert abs(res.E.numpy()[i] - le.local_estimate[i]) < tol * max(1.0, abs(le.local_estimate[i])) * 10


@pytest.mark.parametrize("strategy,chi,opts", [("ZipUp", 6, None), ("ZipUp", 6, {"trunc_method": "jacobi"}),
                                               ("ZipUp", 6, {"smem_kb": 0}), ("Variational", 6, None),
                                               ("NoTruncation", 16, None), ("ZipUp", 6, {"precision": "mixed"}),
                                               ("ZipUp", 6, {"precision": "mixed", "smem_kb": 200}),
                                               ("NoTruncation", 16, {"precision": "mixed"})])
def test_stale_memory_never_reaches_the_results(emu_lib, strategy, chi, opts):
    """Workspace, cache and (in the host-emulation build, always) shared memory start as NaN: every value the
    kernel reads must have been written first, so the outputs equal those of a zeroed run."""
    shape, D = (4, 4), 3
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 4, seed=11)
    tens = torch.from_numpy(pack_tensors(T))
    outs = []
    for fill in (0.0, float("nan")):
        eng = _engine(emu_lib, shape, D, chi, strategy, H, options=opts)
        ws = eng.workspace(cfg.shape[0])
        ws[: (ws.numel() // 4) * 4].view(torch.float32).fill_(fill)
        cache = eng.new_cache(cfg.shape[0])
        cache[: (cache.numel() // 4) * 4].view(torch.float32).fill_(fill)
        c = torch.from_numpy(cfg.copy())
        eng.init_cache(tens, c, cache)
        res = eng.sweep(tens, c, torch.from_numpy(u), cache)
        assert eng.status() == 0
        outs.append(res)
    a, b = outs
    assert torch.equal(a.configs, b.configs) and torch.equal(a.E, b.E) and torch.equal(a.O, b.O)
    assert torch.isfinite(b.E).all() and torch.isfinite(b.O).all()


def test_wide_rows_keep_the_zipup_carry_in_range(emu_lib):
    """4x8, D=5, chi=25: along an 8-column row the zip-up carry shrinks at every site; unnormalised,
    its Gram matrix reaches 1e-22 and the squared off-diagonals underflow FP32.  The engine
    renormalises the carry after every cut."""
    shape, D, chi = (4, 8), 5, 25
    T, cfg, _ = make_case(shape, D, 3, seed=7)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", None)
    la, sg, O = eng.amp_grad(torch.from_numpy(pack_tensors(T)), torch.from_numpy(cfg.copy()))
    model = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert_parity(np.abs((sg * torch.exp(la)).numpy() / amp - 1), True)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)


@pytest.mark.parametrize("shape", [(3, 24), (2, 32)])
def test_wide_lattice_environments_stay_in_range(emu_lib, shape):
    """|psi| ~ 1e-63 here: row environments are renormalised at every column with their log-scales
    carried in FP64, so nothing leaves the FP32 range (Metropolis ratios, O and E_loc all match)."""
    D, chi = 4, 8
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 4, seed=2)
    eng = _engine(emu_lib, shape, D, chi, "ZipUp", H)
    res, _, _ = _sweep(eng, T, cfg, u)
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    assert float(res.logamp.max()) < -100
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert_parity(np.abs(amp / ctx.amp - 1), True)
    e_ref = le.local_estimate
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)
    o_ref = le.local_log_derivatives
    assert_parity(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)


COMPLEX_CASES = [
    ((3, 3), 2, 16, "NoTruncation", "heisenberg"),
    ((3, 3), 3, 4, "ZipUp", "tfim"),
    ((4, 4), 2, 4, "ZipUp", "heisenberg"),
    ((3, 4), 2, 3, "Variational", "heisenberg"),
]


@pytest.mark.parametrize("shape,D,chi,strategy,model", COMPLEX_CASES)
@pytest.mark.parametrize("full", [False, True])
def test_complex_sweep_matches_oracle(emu_lib, shape, D, chi, strategy, model, full):
    """complex64 PEPS (interleaved (re, im) elements): complex Gram / Householder truncation, bilinear
    amplitudes, complex O_k and E_loc against the complex128 oracle."""
    H = hamiltonian(model, shape)
    T = complex_tensors(shape, D, seed=D + chi)
    rng = np.random.default_rng(3)
    n_sites = shape[0] * shape[1]
    cfg = rng.integers(0, 2, (5, n_sites)).astype(np.int32)
    u = rng.random((5, n_sites))
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib, dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, full_gradient=full)
    c2, ctx, le = oracle_sweep(T, shape, D, strategy, chi, H, cfg, u, full_gradient=full)
    assert np.array_equal(res.configs.numpy(), c2)
    trunc = strategy != "NoTruncation"
    amp = np.exp(res.logamp.numpy() + 1j * res.sign.numpy())
    assert_parity(np.abs(amp / ctx.amp - 1), trunc)
    e_ref = le.local_estimate
    assert res.E.dtype == torch.complex128
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), trunc)
    o_ref = le.local_log_derivatives
    assert_parity(np.linalg.norm(res.O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), trunc)
    assert eng.status() == 0


def test_complex_amp_grad_and_local_energy(emu_lib):
    shape, D, chi = (4, 4), 2, 4
    H = hamiltonian("heisenberg", shape)
    T = complex_tensors(shape, D, seed=9)
    cfg = np.random.default_rng(4).integers(0, 2, (6, 16)).astype(np.int32)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib, dtype="complex64")
    tens = torch.from_numpy(pack_tensors(T))
    la, ph, O = eng.amp_grad(tens, torch.from_numpy(cfg))
    E = eng.local_energy(tens, torch.from_numpy(cfg), la, ph)
    model = oracle.PEPS(T, shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg)
    assert_parity(np.abs(np.exp(la.numpy() + 1j * ph.numpy()) / amp - 1), True)
    o_ref = grads / amp[:, None]
    assert_parity(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)
    e_ref = oracle.local_estimate(model, cfg, H, amp)
    assert_parity(np.abs(E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


def test_invalid_arguments_return_status_codes(emu_lib):
    import ctypes as ct

    plan = ct.c_void_p()
    bad = _abi.VmcShape(0, 3)
    assert emu_lib.vmc_peps_plan(ct.byref(bad), 2, 4, 2, 0, 1, 2, ct.byref(plan)) == _abi.VMC_ERR_INVALID
    ok = _abi.VmcShape(3, 3)
    assert emu_lib.vmc_peps_plan(ct.byref(ok), 2, 4, 2, 7, 1, 2, ct.byref(plan)) == _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_peps_plan(ct.byref(ok), 2, 4, 9, 0, 1, 2, ct.byref(plan)) == _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_peps_plan(ct.byref(ok), 2, 4, 2, 0, 1, 2, ct.byref(plan)) == _abi.VMC_OK
    cfg = np.zeros((2, 9), np.int32)
    tens = np.zeros(1000, np.float32)
    ws = np.zeros(16, np.uint8)
    cache = np.zeros(emu_lib.vmc_cache_size(plan, 2), np.uint8)
    st = np.zeros(1, np.int32)
    p = lambda a: a.ctypes.data_as(ct.c_void_p)
    assert emu_lib.vmc_peps_init_cache(plan, None, p(tens), p(cfg), 2, p(cache), p(ws), ws.nbytes,
                                       p(st)) == _abi.VMC_ERR_WORKSPACE
    assert emu_lib.vmc_status_string(_abi.VMC_ERR_WORKSPACE) == b"workspace too small"
    emu_lib.vmc_plan_destroy(plan)
