"""Randomised parity in the host emulation of the kernels: lattices up to 5x5, D in {2, 3}, d in {2, 3},
every strategy, real and complex64 tensors, both precision tiers, sliced and full gradients, and random
Hermitian operators (one-site, horizontal and vertical two-site terms and a diagonal term) against one
transition + estimate of the FP64 oracle, from fixed seeds.  Plans beyond the engine's largest cut
(NoTruncation bonds grow as D^rows) must be refused with VMC_ERR_UNSUPPORTED."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import complex_tensors, fp32, make_case, oracle_strategy, oracle_sweep
from vmc_gb300._abi import VMC_ERR_UNSUPPORTED, VmcError
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors
from vmc_gb300.operators import (DiagonalTerm, HorizontalTwoSiteTerm, LocalHamiltonian, OneSiteTerm,
                                 VerticalTwoSiteTerm)


def _hermitian(rng, n, cplx):
    m = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cplx else 0)
    return m + m.conj().T


def _operator(rng, shape, d, cplx):
    R, C = shape
    ops = []
    for r in range(R):
        for c in range(C):
            if rng.random() < 0.7:
                ops.append(OneSiteTerm(r, c, _hermitian(rng, d, cplx)))
            if c < C - 1 and rng.random() < 0.7:
                ops.append(HorizontalTwoSiteTerm(r, c, _hermitian(rng, d * d, cplx)))
            if r < R - 1 and rng.random() < 0.7:
                ops.append(VerticalTwoSiteTerm(r, c, _hermitian(rng, d * d, cplx)))
    if R * C >= 2:
        a = (int(rng.integers(R)), int(rng.integers(C)))
        b = a
        while b == a:
            b = (int(rng.integers(R)), int(rng.integers(C)))
        ops.append(DiagonalTerm((a, b), rng.standard_normal(d * d)))
    return LocalHamiltonian(shape, tuple(ops))


def _draw(seed):
    rng = np.random.default_rng(seed)
    shape = (int(rng.integers(1, 6)), int(rng.integers(1, 6)))
    D, d = int(rng.integers(2, 4)), int(rng.choice([2, 2, 3]))
    strategy = str(rng.choice(["ZipUp", "NoTruncation", "Variational", "DensityMatrix"]))
    chi = 64 if strategy == "NoTruncation" else int(rng.integers(2, 7))
    if strategy == "DensityMatrix":
        chi = min(chi, D)  # every kept eigenvector has a nonzero eigenvalue
    cplx = bool(rng.random() < 0.3)
    mixed = (not cplx) and strategy != "Variational" and rng.random() < 0.4
    return rng, shape, D, d, strategy, chi, cplx, "mixed" if mixed else "fp32", bool(rng.random() < 0.3)


@pytest.mark.parametrize("seed", range(96))
def test_random_case_matches_oracle(emu_lib, seed):
    rng, shape, D, d, strategy, chi, cplx, precision, full = _draw(1000 + seed)
    n, n_sites = 4, shape[0] * shape[1]
    try:
        eng = PEPSEngine(shape, D, chi, d, strategy, operator=None, device="cpu", lib=emu_lib,
                         dtype="complex64" if cplx else "float32", options={"precision": precision})
    except VmcError as e:
        assert strategy == "NoTruncation" and e.status == VMC_ERR_UNSUPPORTED and D ** (shape[0] - 1) * D > 64
        return
    if cplx:
        T = complex_tensors(shape, D, seed=seed, phys_dim=d)
        cfg = rng.integers(0, d, (n, n_sites)).astype(np.int32)
        u = rng.random((n, n_sites))
    else:
        T, cfg, u = make_case(shape, D, n, seed=seed, phys_dim=d)
        T = fp32(T)
    H = _operator(rng, shape, d, cplx)
    eng.set_operator(H)
    deltas = rng.integers(1, d, size=cfg.shape).astype(np.int32) if d > 2 else None
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, deltas=None if deltas is None else torch.from_numpy(deltas),
                    full_gradient=full)
    assert eng.status() == 0
    c2, ctx, le = oracle_sweep(T, shape, D, strategy, chi, H, cfg, u, full_gradient=full, deltas=deltas)
    same = np.all(res.configs.numpy() == c2, axis=1)
    assert np.all(same | (res.margin.numpy() < 1e-4))
    if cplx:
        amp = np.exp(res.logamp.numpy() + 1j * res.sign.numpy())
    else:
        amp = (res.sign * torch.exp(res.logamp)).numpy()
    # FP32 rounding, and up to ~eps_fp32 / gap where a cut truncates with a small relative gap
    tol = 2e-3 if float(res.gap.min()) < 1e-2 else 2e-4
    assert np.max(np.abs(amp[same] / ctx.amp[same] - 1), initial=0) < tol
    e, e_ref = res.E.numpy()[same], le.local_estimate[same]
    assert np.max(np.abs(e - e_ref) / np.maximum(1.0, np.abs(e_ref)), initial=0) < tol
    o, o_ref = res.O.numpy()[same], le.local_log_derivatives[same]
    assert np.max(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), initial=0) < tol
    if not full:
        assert np.array_equal(res.p.numpy()[same], le.active_slice_indices[same])


def _draw_gi(seed):
    rng = np.random.default_rng(seed)
    shape = (int(rng.integers(2, 6)), int(rng.integers(2, 6)))
    N = int(rng.choice([2, 2, 3]))
    dmax = int(rng.integers(1, 3))
    chi = None if rng.random() < 0.25 else int(rng.integers(2, 9))
    return rng, shape, N, dmax, chi


@pytest.mark.parametrize("seed", range(24))
def test_random_gauge_invariant_case_matches_oracle(emu_lib, seed):
    """Pure Z_N gauge (N = 2, 3), random lattices, degeneracies, chi and couplings (electric g, plaquette h)
    against the GI oracle: one plaquette sweep, amplitudes, energies, O_k and slice indices."""
    from oracle import gi as ogi
    from oracle import peps as op
    from vmc_gb300 import NoTruncation, ZipUp
    from vmc_gb300.gi import GILocalHamiltonian, GIPEPS, GIPEPSConfig, build_electric_terms
    from vmc_gb300.operators import PlaquetteTerm

    rng, shape, N, dmax, chi = _draw_gi(2000 + seed)
    (R, C), n = shape, 4
    ocfg = ogi.GIConfig(shape, N, dmax)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in ogi.init_tensors(ocfg, seed=seed)]
    model = GIPEPS(config=GIPEPSConfig(shape=shape, N=N, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax,) * N),
                   contraction_strategy=NoTruncation() if chi is None else ZipUp(chi), device="cpu", tensors=T,
                   lib=emu_lib)
    g, h = float(rng.uniform(0.2, 1.5)), float(rng.uniform(-1.5, 1.5))
    plaq = [(r, c) for r in range(R - 1) for c in range(C - 1)]
    H = GILocalHamiltonian(shape=shape, terms=build_electric_terms(shape, g, N)
                           + tuple(PlaquetteTerm(row=r, col=c, coeff=h) for r, c in plaq))
    diag = g * (2.0 - 2.0 * np.cos(2.0 * np.pi * np.arange(N) / N))
    OH = ogi.GIHamiltonian(shape, tuple(ogi.PlaquetteTerm(r, c, h) for r, c in plaq)
                           + tuple(ogi.LinkDiagonalTerm("h", ((r, c),), diag) for r in range(R) for c in range(C - 1))
                           + tuple(ogi.LinkDiagonalTerm("v", ((r, c),), diag) for r in range(R - 1) for c in range(C)))
    samples = ogi.random_physical_configuration(ocfg, n, seed=seed + 7)
    u = rng.random((n, len(plaq)))
    deltas = rng.integers(1, N, (n, len(plaq))) if N > 2 else np.ones((n, len(plaq)), dtype=np.int64)
    eng = model.engine(H)
    tens = model.packed()
    c = torch.from_numpy(samples.astype(np.int32))
    cache = eng.init_cache(tens, c.clone())
    res = eng.sweep(tens, c.clone(), torch.from_numpy(u), cache,
                    deltas=torch.from_numpy(deltas.astype(np.int32)) if N > 2 else None)
    assert eng.status() == 0
    strat = op.NoTruncation() if chi is None else op.ZipUp(chi)
    s2, amp_ref, tops, margin = ogi.transition(T, ocfg, samples, deltas.reshape(n, R - 1, C - 1),
                                               u.reshape(n, R - 1, C - 1), ogi.init_cache(T, ocfg, samples, strat),
                                               strat)
    same = np.all(res.configs.numpy() == s2, axis=1)
    assert np.all(same | (margin < 1e-4))
    grads, e_ref, _ = ogi.estimate(T, ocfg, s2, amp_ref, OH, strat, tops)
    o_ref, p_ref = ogi.local_log_derivatives(T, ocfg, s2, grads, amp_ref)
    tol = 2e-3 if float(res.gap.min()) < 1e-2 else 2e-4
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert np.max(np.abs(amp[same] / amp_ref[same] - 1), initial=0) < tol
    assert np.max(np.abs(res.E.numpy()[same] - e_ref[same]) / np.maximum(1.0, np.abs(e_ref[same])), initial=0) < tol
    o_err = np.linalg.norm(res.O.numpy()[same] - o_ref[same], axis=1) / np.linalg.norm(o_ref[same], axis=1)
    assert np.max(o_err, initial=0) < tol
    assert np.array_equal(res.p.numpy()[same], p_ref[same])


@pytest.mark.parametrize("seed", range(24))
def test_random_sr_solve_matches_oracle(seed):
    """The FP64 SR layer (QGT + DirectSolve, plain torch) on random sliced Jacobians: lattices, D, d in
    {2, 3}, real or complex parameters, imaginary or real time, sample counts on both sides of the
    parameter count, diagonal shifts 1e-4..1e-1, both spaces, against oracle/sr.py."""
    from oracle import sr as osr
    from tests.helpers import uniform_init_tensors
    from tests.test_sr_and_distributed import _ComplexModel, _Model
    from vmc_gb300 import qgt as gq
    from vmc_gb300.preconditioners import SRPreconditioner
    from oracle import peps as oracle

    rng = np.random.default_rng(4000 + seed)
    shape = (int(rng.integers(1, 4)), int(rng.integers(2, 4)))
    D, d = int(rng.integers(2, 4)), int(rng.choice([2, 3]))
    cplx = bool(rng.random() < 0.4)
    n = int(rng.integers(4, 160))
    param_space = bool(rng.random() < 0.5)
    shift = float(10 ** rng.uniform(-4, -1))
    gf = -1j if (cplx and rng.random() < 0.5) else -1.0
    T = complex_tensors(shape, D, seed=seed, phys_dim=d) if cplx else uniform_init_tensors(shape, D, phys_dim=d,
                                                                                             seed=seed)
    om = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle.NoTruncation())
    cfg = rng.integers(0, d, size=(n, shape[0] * shape[1]))
    amps, grads, p = oracle.value_and_grad(om, cfg)
    o = grads / amps[:, None]
    e = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    x_ref, m_ref = osr.sr_apply(o, p, e, pps=oracle.params_per_site(om), sliced_dims=oracle.sliced_dims(om),
                                n_samples=n, diag_shift=shift, grad_factor=gf, real_params=not cplx,
                                space=osr.ParameterSpace() if param_space else osr.SampleSpace())
    pre = SRPreconditioner(space=gq.ParameterSpace() if param_space else gq.SampleSpace(), diag_shift=shift)
    m = (_ComplexModel if cplx else _Model)(shape, D, d, T)
    upd, metrics = pre.apply(m, m.tensors, torch.zeros((n, shape[0] * shape[1])), torch.as_tensor(o),
                             torch.as_tensor(p), torch.as_tensor(e), grad_factor=gf)
    flat = torch.cat([u.reshape(-1) for row in upd for u in row]).to(torch.complex128).numpy()
    assert np.linalg.norm(flat - x_ref) / np.linalg.norm(x_ref) < 1e-5  # FP32 updates
    assert abs(float(metrics["residual_error"]) - m_ref["residual_error"]) < 1e-6 * max(1.0, m_ref["residual_error"])


@pytest.mark.parametrize("seed", range(16))
def test_random_vjp_matches_oracle(emu_lib, seed):
    """vmc_peps_vjp: sum_i w_i O_i over the full parameter layout, accumulated in FP64 in the kernel, on random
    lattices, strategies, element types and weights, against the oracle's full-gradient O."""
    rng = np.random.default_rng(5000 + seed)
    shape = (int(rng.integers(1, 5)), int(rng.integers(1, 5)))
    D, d = int(rng.integers(2, 4)), int(rng.choice([2, 3]))
    strategy = str(rng.choice(["ZipUp", "NoTruncation", "Variational"]))
    chi = 64 if strategy == "NoTruncation" else int(rng.integers(2, 7))
    cplx = bool(rng.random() < 0.4)
    n = int(rng.integers(1, 7))
    try:
        eng = PEPSEngine(shape, D, chi, d, strategy, operator=None, device="cpu", lib=emu_lib,
                         dtype="complex64" if cplx else "float32")
    except VmcError as e:
        assert strategy == "NoTruncation" and e.status == VMC_ERR_UNSUPPORTED
        return
    if cplx:
        T = complex_tensors(shape, D, seed=seed, phys_dim=d)
        cfg = rng.integers(0, d, (n, shape[0] * shape[1])).astype(np.int32)
        w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    else:
        T, cfg, _ = make_case(shape, D, n, seed=seed, phys_dim=d)
        T = fp32(T)
        w = rng.standard_normal(n)
    from oracle import peps as oracle

    model = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle_strategy(strategy, chi))
    # the engine takes occupancies as given (the sampler kernels' convention)
    amp, grads, _ = oracle.value_and_grad_occupancy(model, cfg, full_gradient=True)
    ref = (w[:, None] * grads / amp[:, None]).sum(0)
    g = eng.vjp(torch.from_numpy(pack_tensors(T)), torch.from_numpy(cfg), torch.from_numpy(w)).numpy()
    assert eng.status() == 0
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 1e-4


@pytest.mark.parametrize("seed", range(12))
def test_random_truncating_mixed_tier_amplitudes(emu_lib, seed):
    """The mixed tier on random actively truncating ZipUp / DensityMatrix cases (3..5 x 3..5, chi < D^2):
    amplitudes at the FP64 level of the double-float chain (< 1e-10, against FP32's ~1e-6), O_k at the FP32
    level of the environments."""
    from tests.helpers import hamiltonian

    rng = np.random.default_rng(9000 + seed)
    shape = (int(rng.integers(3, 6)), int(rng.integers(3, 6)))
    D = int(rng.integers(2, 4))
    chi = int(rng.integers(2, D * D))
    strategy = str(rng.choice(["ZipUp", "DensityMatrix"]))
    if strategy == "DensityMatrix":
        chi = min(chi, D)
    T, cfg, u = make_case(shape, D, 4, seed=seed)
    T = fp32(T)
    H = hamiltonian(str(rng.choice(["heisenberg", "tfim"])), shape)
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib,
                     options={"precision": "mixed"})
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache)
    c2, ctx, le = oracle_sweep(T, shape, D, strategy, chi, H, cfg, u)
    same = np.all(res.configs.numpy() == c2, axis=1)
    assert np.all(same | (res.margin.numpy() < 1e-4))
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert np.max(np.abs(amp[same] / ctx.amp[same] - 1), initial=0) < 1e-10
    o, o_ref = res.O.numpy()[same], le.local_log_derivatives[same]
    assert np.max(np.linalg.norm(o - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), initial=0) < 1e-5


@pytest.mark.parametrize("seed", range(12))
def test_sample_and_parameter_space_solves_agree(seed):
    """Push-through identity O^H (O O^H + l)^-1 v = (O^H O + l)^-1 O^H v: the SampleSpace and ParameterSpace
    DirectSolve updates are the same vector, in the oracle (preconditioners.py:117-152) and in the FP64 torch
    SR layer, on random sliced Jacobians (both sides of the parameter count, real and complex)."""
    from oracle import peps as oracle
    from oracle import sr as osr
    from tests.helpers import uniform_init_tensors
    from tests.test_sr_and_distributed import _ComplexModel, _Model
    from vmc_gb300 import qgt as gq
    from vmc_gb300.preconditioners import SRPreconditioner

    rng = np.random.default_rng(7000 + seed)
    shape, D, d = (int(rng.integers(1, 3)), int(rng.integers(2, 4))), int(rng.integers(2, 4)), int(rng.choice([2, 3]))
    cplx = bool(rng.random() < 0.5)
    n = int(rng.integers(4, 200))
    shift = float(10 ** rng.uniform(-3, -1))
    T = complex_tensors(shape, D, seed=seed, phys_dim=d) if cplx else uniform_init_tensors(shape, D, phys_dim=d,
                                                                                             seed=seed)
    om = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle.NoTruncation())
    cfg = rng.integers(0, d, size=(n, shape[0] * shape[1]))
    amps, grads, p = oracle.value_and_grad(om, cfg)
    o = grads / amps[:, None]
    e = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    kw = dict(pps=oracle.params_per_site(om), sliced_dims=oracle.sliced_dims(om), n_samples=n, diag_shift=shift,
              grad_factor=-1.0, real_params=not cplx)
    xs, _ = osr.sr_apply(o, p, e, space=osr.SampleSpace(), **kw)
    xp, _ = osr.sr_apply(o, p, e, space=osr.ParameterSpace(), **kw)
    assert np.linalg.norm(xs - xp) <= 1e-8 * np.linalg.norm(xp)
    m = (_ComplexModel if cplx else _Model)(shape, D, d, T)
    outs = []
    for space in (gq.SampleSpace(), gq.ParameterSpace()):
        upd, _ = SRPreconditioner(space=space, diag_shift=shift).apply(
            m, m.tensors, torch.zeros((n, shape[0] * shape[1])), torch.as_tensor(o), torch.as_tensor(p),
            torch.as_tensor(e), grad_factor=-1.0)
        outs.append(torch.cat([u.reshape(-1) for row in upd for u in row]).to(torch.complex128).numpy())
    assert np.linalg.norm(outs[0] - outs[1]) <= 1e-6 * np.linalg.norm(outs[1])  # FP32 updates
