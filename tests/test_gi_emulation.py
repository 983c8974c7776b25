"""The gauge-invariant engine path (GI plan: slices selected by links, plaquette sweeps, link-diagonal
and plaquette energies) in the host-emulation build against the FP64 GI oracle."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import gi as ogi
from oracle import peps as op
from tests.helpers import assert_parity
from vmc_gb300 import NoTruncation, ZipUp
from vmc_gb300.gi import GIPEPS, GIPEPSConfig, build_gi_mc_kernels, z2_pure_gauge_hamiltonian

CASES = [((3, 3), 2, None), ((3, 4), 2, 4), ((4, 4), 2, 6)]


def _fp32(T):
    return [[t.astype(np.float32).astype(np.float64) for t in row] for row in T]


def _setup(emu_lib, shape, dmax, chi, seed, n):
    ocfg = ogi.GIConfig(shape, 2, dmax)
    T = _fp32(ogi.init_tensors(ocfg, seed=seed))
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax))
    model = GIPEPS(config=cfg, contraction_strategy=NoTruncation() if chi is None else ZipUp(chi), device="cpu",
                   tensors=T, lib=emu_lib)
    samples = ogi.random_physical_configuration(ocfg, n, seed=seed + 1)
    strat = op.NoTruncation() if chi is None else op.ZipUp(chi)
    return ocfg, T, model, samples, strat


def _forward_top_envs(T, cfg, samples, strat):
    _, h, v = ogi.unflatten_sample(samples, cfg.shape)
    top = tuple(op._ones(samples.shape[0], 3, np.float64) for _ in range(cfg.shape[1]))
    envs = []
    for r in range(cfg.shape[0]):
        envs.append(top)
        top = strat.apply(top, ogi.row_mpo(T, cfg, h, v, r))
    return envs


@pytest.mark.parametrize("shape,dmax,chi", CASES)
def test_amplitudes_gradients_energies(emu_lib, shape, dmax, chi):
    ocfg, T, model, samples, strat = _setup(emu_lib, shape, dmax, chi, seed=3, n=6)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    OH = ogi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    eng = model.engine(H)
    tens = model.packed()
    c = torch.from_numpy(samples.astype(np.int32))
    la, sg, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, sg)
    amp_ref = ogi.amplitude(T, ocfg, samples, strat)
    trunc = chi is not None
    amp = (sg * torch.exp(la)).numpy()
    assert_parity(np.abs(amp / amp_ref - 1), trunc)
    grads, e_ref, _ = ogi.estimate(T, ocfg, samples, amp_ref, OH, strat, _forward_top_envs(T, ocfg, samples, strat))
    o_ref, p_ref = ogi.local_log_derivatives(T, ocfg, samples, grads, amp_ref)
    assert_parity(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), trunc)
    assert_parity(np.abs(E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), trunc)
    assert eng.status() == 0


@pytest.mark.parametrize("shape,dmax,chi", CASES)
def test_sweep_matches_oracle(emu_lib, shape, dmax, chi):
    ocfg, T, model, samples, strat = _setup(emu_lib, shape, dmax, chi, seed=5, n=8)
    R, C = shape
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    OH = ogi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    u = np.random.default_rng(9).random((8, (R - 1) * (C - 1)))
    init, trans, est = build_gi_mc_kernels(model, H)
    c = torch.from_numpy(samples.astype(np.int32))
    cache = init(model.tensors, c)
    c2, _, ctx = trans(model.tensors, c, torch.from_numpy(u), cache)
    _, le = est(model.tensors, c2, ctx)
    ocache = ogi.init_cache(T, ocfg, samples, strat)
    s2, amp_ref, tops, margin = ogi.transition(T, ocfg, samples, np.ones((8, R - 1, C - 1), dtype=np.int64),
                                               u.reshape(8, R - 1, C - 1), ocache, strat)
    same = np.all(c2.numpy() == s2, axis=1)
    assert np.all(same | (margin < 1e-4)) and same.mean() > 0.7
    grads, e_ref, _ = ogi.estimate(T, ocfg, s2, amp_ref, OH, strat, tops)
    o_ref, p_ref = ogi.local_log_derivatives(T, ocfg, s2, grads, amp_ref)
    trunc = chi is not None
    amp = le.amp.numpy()
    assert_parity(np.abs(amp[same] / amp_ref[same] - 1), trunc)
    e = le.local_estimate.numpy()
    assert_parity(np.abs(e[same] - e_ref[same]) / np.maximum(1.0, np.abs(e_ref[same])), trunc)
    o = le.local_log_derivatives.numpy()
    assert_parity(np.linalg.norm(o[same] - o_ref[same], axis=1) / np.linalg.norm(o_ref[same], axis=1), trunc)
    assert np.array_equal(le.active_slice_indices.numpy()[same], p_ref[same])


def test_full_gradient_in_the_reference_layout(emu_lib):
    ocfg, T, model, samples, strat = _setup(emu_lib, (3, 3), 2, None, seed=7, n=4)
    H = z2_pure_gauge_hamiltonian((3, 3))
    init, trans, est = build_gi_mc_kernels(model, H, full_gradient=True)
    c = torch.from_numpy(samples.astype(np.int32))
    u = torch.ones((4, 4), dtype=torch.float64)  # u = 1 rejects every proposal: the sample stays
    c2, _, ctx = trans(model.tensors, c, u, init(model.tensors, c))
    _, le = est(model.tensors, c2, ctx)
    assert np.array_equal(c2.numpy(), samples)
    amp_ref = ogi.amplitude(T, ocfg, samples, strat)
    grads, _, _ = ogi.estimate(T, ocfg, samples, amp_ref, ogi.GIHamiltonian((3, 3), ()), strat,
                               _forward_top_envs(T, ocfg, samples, strat))
    o_ref, _ = ogi.local_log_derivatives(T, ocfg, samples, grads, amp_ref, full_gradient=True)
    o = le.local_log_derivatives.numpy()
    assert o.shape == o_ref.shape
    assert np.linalg.norm(o - o_ref) / np.linalg.norm(o_ref) < 1e-5


def test_complex_gi_matches_oracle(emu_lib):
    shape, dmax, chi = (3, 4), 2, 4
    ocfg = ogi.GIConfig(shape, 2, dmax)
    T = [[t.astype(np.complex64).astype(np.complex128) for t in row]
         for row in ogi.init_tensors(ocfg, seed=11, dtype=np.complex128)]
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax), dtype=torch.complex64)
    model = GIPEPS(config=cfg, contraction_strategy=ZipUp(chi), device="cpu", tensors=T, lib=emu_lib)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    eng = model.engine(H)
    samples = ogi.random_physical_configuration(ocfg, 6, seed=12)
    c = torch.from_numpy(samples.astype(np.int32))
    la, ph, O = eng.amp_grad(model.packed(), c)
    E = eng.local_energy(model.packed(), c, la, ph)
    strat = op.ZipUp(chi)
    amp_ref = ogi.amplitude(T, ocfg, samples, strat)
    assert_parity(np.abs(np.exp(la.numpy() + 1j * ph.numpy()) / amp_ref - 1), True)
    grads, e_ref, _ = ogi.estimate(T, ocfg, samples, amp_ref, ogi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4),
                                   strat, _forward_top_envs_c(T, ocfg, samples, strat))
    o_ref, _ = ogi.local_log_derivatives(T, ocfg, samples, grads, amp_ref)
    assert_parity(np.linalg.norm(O.numpy() - o_ref, axis=1) / np.linalg.norm(o_ref, axis=1), True)
    assert_parity(np.abs(E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


def _forward_top_envs_c(T, cfg, samples, strat):
    _, h, v = ogi.unflatten_sample(samples, cfg.shape)
    top = tuple(op._ones(samples.shape[0], 3, np.complex128) for _ in range(cfg.shape[1]))
    envs = []
    for r in range(cfg.shape[0]):
        envs.append(top)
        top = strat.apply(top, ogi.row_mpo(T, cfg, h, v, r))
    return envs


def test_tdvp_on_a_gi_model_with_full_gradients(emu_lib):
    """The reference's lattice-gauge drivers run TDVPDriver(full_gradient=True) on a GIPEPS
    (examples/lgt/z2_pure_gauge.py:79-95): the same on the engine, imaginary time."""
    from vmc_gb300.drivers import ImaginaryTimeUnit, TDVPDriver
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import SampleSpace

    shape = (3, 3)
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(2, 2))
    model = GIPEPS(rngs=1, config=cfg, contraction_strategy=ZipUp(4), device="cpu", lib=emu_lib)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    drv = TDVPDriver(model, H, preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=0.1), dt=0.05,
                     time_unit=ImaginaryTimeUnit(), n_samples=64, n_chains=32, full_gradient=True)
    t0 = [[t.clone() for t in row] for row in model.tensors]
    drv.run(0.1)
    assert drv.step_count == 2 and np.isfinite(drv.energy["mean"])
    assert any(not torch.equal(a, b) for ra, rb in zip(t0, drv._tensors) for a, b in zip(ra, rb))
    # the sliced solve (full_gradient=False) with the per-site slice counts of the GI model
    sliced = TDVPDriver(model, H, preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=0.1), dt=0.05,
                        time_unit=ImaginaryTimeUnit(), n_samples=64, n_chains=32)
    sliced.run(0.05)
    assert np.isfinite(sliced.energy["mean"])


def test_sliced_and_full_sr_updates_agree_on_a_gi_model(emu_lib):
    """The sliced Jacobian expanded with the GI model's per-site slice counts is the full Jacobian:
    both SR solves give the same update (ParameterSpace, preconditioners.py:265-330)."""
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import ParameterSpace

    ocfg, T, model, samples, strat = _setup(emu_lib, (3, 3), 2, None, seed=31, n=24)
    H = z2_pure_gauge_hamiltonian((3, 3))
    outs = []
    for full in (False, True):
        init, trans, est = build_gi_mc_kernels(model, H, full_gradient=full)
        c = torch.from_numpy(samples.astype(np.int32))
        u = torch.ones((24, 4), dtype=torch.float64)  # keep the samples: both solves see the same ones
        c2, _, ctx = trans(model.tensors, c, u, init(model.tensors, c))
        _, le = est(model.tensors, c2, ctx)
        upd, _ = SRPreconditioner(space=ParameterSpace(), diag_shift=0.1).apply(
            model, model.tensors, c2, le.local_log_derivatives, le.active_slice_indices, le.local_estimate)
        outs.append(torch.cat([x.reshape(-1) for row in upd for x in row]))
    assert torch.allclose(outs[0], outs[1], rtol=1e-6, atol=1e-9)


def test_z3_pure_gauge_matches_oracle(emu_lib):
    """Z3 (examples/lgt/z3_pure_gauge.py): 27 slices on a bulk site, +-1 plaquette flips distinct,
    explicit flip offsets; sweep, amplitudes, O_k and energies against the oracle."""
    from vmc_gb300.gi import GILocalHamiltonian, build_electric_terms
    from vmc_gb300.operators import PlaquetteTerm

    shape, dmax, chi, n = (3, 3), 2, 8, 8
    R, C = shape
    ocfg = ogi.GIConfig(shape, 3, dmax)
    T = _fp32(ogi.init_tensors(ocfg, seed=21))
    cfg = GIPEPSConfig(shape=shape, N=3, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax, dmax))
    model = GIPEPS(config=cfg, contraction_strategy=ZipUp(chi), device="cpu", tensors=T, lib=emu_lib)
    terms = build_electric_terms(shape, 0.5, 3) + tuple(PlaquetteTerm(row=r, col=c, coeff=-1.0)
                                                        for r in range(R - 1) for c in range(C - 1))
    H = GILocalHamiltonian(shape=shape, terms=terms)
    diag = 0.5 * (2.0 - 2.0 * np.cos(2.0 * np.pi * np.arange(3) / 3))
    OH = ogi.GIHamiltonian(shape, tuple(ogi.PlaquetteTerm(r, c, -1.0) for r in range(R - 1) for c in range(C - 1))
                           + tuple(ogi.LinkDiagonalTerm("h", ((r, c),), diag) for r in range(R) for c in range(C - 1))
                           + tuple(ogi.LinkDiagonalTerm("v", ((r, c),), diag) for r in range(R - 1) for c in range(C)))
    samples = ogi.random_physical_configuration(ocfg, n, seed=22)
    rng = np.random.default_rng(23)
    u = rng.random((n, (R - 1) * (C - 1)))
    deltas = rng.integers(1, 3, (n, (R - 1) * (C - 1)))
    eng = model.engine(H)
    assert eng.phys_dim == 27 and eng.needs_deltas
    tens = model.packed()
    c = torch.from_numpy(samples.astype(np.int32))
    cache = eng.init_cache(tens, c.clone())
    res = eng.sweep(tens, c.clone(), torch.from_numpy(u), cache, deltas=torch.from_numpy(deltas.astype(np.int32)))
    strat = op.ZipUp(chi)
    s2, amp_ref, tops, margin = ogi.transition(T, ocfg, samples, deltas.reshape(n, R - 1, C - 1),
                                               u.reshape(n, R - 1, C - 1), ogi.init_cache(T, ocfg, samples, strat),
                                               strat)
    same = np.all(res.configs.numpy() == s2, axis=1)
    assert np.all(same | (margin < 1e-4)) and same.mean() > 0.7 and (s2 != samples).any()
    grads, e_ref, _ = ogi.estimate(T, ocfg, s2, amp_ref, OH, strat, tops)
    o_ref, p_ref = ogi.local_log_derivatives(T, ocfg, s2, grads, amp_ref)
    amp = (res.sign * torch.exp(res.logamp)).numpy()
    assert_parity(np.abs(amp[same] / amp_ref[same] - 1), True)
    assert_parity(np.abs(res.E.numpy()[same] - e_ref[same]) / np.maximum(1.0, np.abs(e_ref[same])), True)
    assert_parity(np.linalg.norm(res.O.numpy()[same] - o_ref[same], axis=1) / np.linalg.norm(o_ref[same], axis=1),
                  True)
    assert np.array_equal(res.p.numpy()[same], p_ref[same])
