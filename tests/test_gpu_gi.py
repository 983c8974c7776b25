"""The gauge-invariant (pure Z2 gauge) engine on the GPU: parity with the FP64 GI oracle on small
lattices, and at the lattice-gauge workload's size (9x9 vertices, 2 states per charge sector, chi=32)
exact properties -- every sampled configuration obeys Gauss's law, re-evaluating the samples gives the
sweep's amplitudes bit for bit, energies are finite."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import gi as ogi
from oracle import peps as op
from tests.helpers import CONFIG2_MAX_TOL, CONFIG2_MEDIAN_TOL, assert_parity
from vmc_gb300 import ZipUp
from vmc_gb300.gi import GIPEPS, GIPEPSConfig, build_gi_mc_kernels, z2_pure_gauge_hamiltonian

pytestmark = pytest.mark.gpu


def _model(dev, shape, dmax, chi, T=None, seed=0):
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax))
    return GIPEPS(rngs=seed, config=cfg, contraction_strategy=ZipUp(chi), device=dev, tensors=T)


@pytest.mark.parametrize("shape,dmax,chi", [((3, 4), 2, 4), ((4, 4), 2, 6)])
def test_sweep_matches_oracle(cuda_device, shape, dmax, chi):
    R, C = shape
    ocfg = ogi.GIConfig(shape, 2, dmax)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in ogi.init_tensors(ocfg, seed=4)]
    model = _model(cuda_device, shape, dmax, chi, T)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4)
    n = 16
    samples = ogi.random_physical_configuration(ocfg, n, seed=5)
    u = np.random.default_rng(6).random((n, (R - 1) * (C - 1)))
    init, trans, est = build_gi_mc_kernels(model, H)
    c = torch.from_numpy(samples.astype(np.int32)).to(cuda_device)
    c2, _, ctx = trans(model.tensors, c, torch.from_numpy(u).to(cuda_device), init(model.tensors, c))
    _, le = est(model.tensors, c2, ctx)
    torch.cuda.synchronize()
    model.engine(H).raise_on_status()
    strat = op.ZipUp(chi)
    s2, amp_ref, tops, margin = ogi.transition(T, ocfg, samples, np.ones((n, R - 1, C - 1), dtype=np.int64),
                                               u.reshape(n, R - 1, C - 1), ogi.init_cache(T, ocfg, samples, strat),
                                               strat)
    same = np.all(c2.cpu().numpy() == s2, axis=1)
    assert np.all(same | (margin < 1e-4)) and same.mean() > 0.7
    grads, e_ref, _ = ogi.estimate(T, ocfg, s2, amp_ref, ogi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4), strat,
                                   tops)
    o_ref, p_ref = ogi.local_log_derivatives(T, ocfg, s2, grads, amp_ref)
    tol = dict(median_tol=CONFIG2_MEDIAN_TOL, max_tol=CONFIG2_MAX_TOL)
    assert_parity(np.abs(le.amp.cpu().numpy()[same] / amp_ref[same] - 1), True, **tol)
    e = le.local_estimate.cpu().numpy()
    assert_parity(np.abs(e[same] - e_ref[same]) / np.maximum(1.0, np.abs(e_ref[same])), True, **tol)
    o = le.local_log_derivatives.cpu().numpy()
    assert_parity(np.linalg.norm(o[same] - o_ref[same], axis=1) / np.linalg.norm(o_ref[same], axis=1), True, **tol)
    assert np.array_equal(le.active_slice_indices.cpu().numpy()[same], p_ref[same])


def test_lattice_gauge_workload_size_exact_properties(cuda_device):
    shape, dmax, chi, n = (9, 9), 2, 32, 256
    R, C = shape
    model = _model(cuda_device, shape, dmax, chi, seed=1)
    H = z2_pure_gauge_hamiltonian(shape, h=0.625, g=0.4)
    eng = model.engine(H)
    c = model.random_physical_configuration(2, n)
    init, trans, est = build_gi_mc_kernels(model, H)
    cache = init(model.tensors, c)
    gen = torch.Generator(device=cuda_device).manual_seed(3)
    for _ in range(2):
        c, _, ctx = trans(model.tensors, c, gen, cache)
        cache, le = est(model.tensors, c, ctx)
    torch.cuda.synchronize()
    eng.raise_on_status()
    st = c.cpu().numpy().astype(np.int64)
    _, h, v = ogi.unflatten_sample(st, shape)
    # Gauss's law at every vertex: in - out flux = 0 mod 2 (model.py:170-175 with Qx = 0)
    nl = np.pad(h, ((0, 0), (0, 0), (1, 0)))
    nr = np.pad(h, ((0, 0), (0, 0), (0, 1)))
    nu = np.pad(v, ((0, 0), (1, 0), (0, 0)))
    nd = np.pad(v, ((0, 0), (0, 1), (0, 0)))
    assert np.all((nl + nd - nu - nr) % 2 == 0)
    assert torch.isfinite(le.local_estimate).all() and torch.isfinite(le.log_amp).all()
    la, sg, _ = eng.amp_grad(model.packed(), c, want_O=False)
    assert torch.equal(la, le.log_amp) and torch.equal(sg, le.sign)
