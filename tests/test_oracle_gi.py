"""The gauge-invariant (pure Z_N gauge) oracle, pinned without the reference: the slice index is a
bijection of the independent links, E_loc equals a dense Hamiltonian built over every gauge-invariant
configuration, gradients match finite differences, ZipUp in its exact regime equals NoTruncation, and
the plaquette Metropolis sweep samples |psi|^2."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from oracle import gi
from oracle import peps as op


def _forward_top_envs(tensors, cfg, samples, strategy):
    _, h, v = gi.unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    top = tuple(op._ones(samples.shape[0], 3, np.asarray(tensors[0][0]).dtype) for _ in range(C))
    envs = []
    for r in range(R):
        envs.append(top)
        top = strategy.apply(top, gi.row_mpo(tensors, cfg, h, v, r))
    return envs


@pytest.mark.parametrize("N", [2, 3])
def test_slice_index_is_a_bijection_of_the_independent_links(N):
    cfg = gi.GIConfig((3, 4), N, 2)
    R, C = cfg.shape
    for r in range(R):
        for c in range(C):
            nc = gi.n_configs(cfg, r, c)
            seen = set()
            # every assignment of the site's links (the dependent one varies too and must not matter)
            for vals in itertools.product(range(N), repeat=4):
                h = np.zeros((1, R, C - 1), dtype=np.int64)
                v = np.zeros((1, R - 1, C), dtype=np.int64)
                if c > 0: h[0, r, c - 1] = vals[0]
                if c < C - 1: h[0, r, c] = vals[1]
                if r > 0: v[0, r - 1, c] = vals[2]
                if r < R - 1: v[0, r, c] = vals[3]
                k = int(gi.site_cfg_index(cfg, h, v, r, c)[0])
                assert 0 <= k < nc
                seen.add(k)
            assert seen == set(range(nc))


@pytest.mark.parametrize("shape,N", [((3, 3), 2), ((2, 3), 3), ((3, 4), 2)])
def test_local_energy_equals_dense_hamiltonian(shape, N):
    cfg = gi.GIConfig(shape, N, 2)
    T = gi.init_tensors(cfg, seed=1)
    H = gi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4, N=N)
    strat = op.NoTruncation()
    e_exact, samples, psi, e_loc = gi.dense_hamiltonian_energy(T, cfg, H, strat)
    top = _forward_top_envs(T, cfg, samples, strat)
    grads, energy, _ = gi.estimate(T, cfg, samples, psi, H, strat, top)
    assert np.allclose(energy, e_loc, rtol=1e-10, atol=1e-10)
    w = psi ** 2
    assert abs(np.sum(w * energy) / np.sum(w) - e_exact) < 1e-10


def test_gradients_match_finite_differences():
    cfg = gi.GIConfig((3, 3), 2, 2)
    T = gi.init_tensors(cfg, seed=2)
    strat = op.NoTruncation()
    samples = gi.random_physical_configuration(cfg, 5, seed=3)
    amp = gi.amplitude(T, cfg, samples, strat)
    top = _forward_top_envs(T, cfg, samples, strat)
    grads, _, _ = gi.estimate(T, cfg, samples, amp, gi.GIHamiltonian(cfg.shape, ()), strat, top)
    o, p = gi.local_log_derivatives(T, cfg, samples, grads, amp)
    o_full, _ = gi.local_log_derivatives(T, cfg, samples, grads, amp, full_gradient=True)
    eps = 1e-6
    rng = np.random.default_rng(0)
    for _ in range(12):
        r, c = rng.integers(0, 3, 2)
        t = T[r][c]
        flat = rng.integers(0, t.size)
        Tp = [[x.copy() for x in row] for row in T]
        Tp[r][c].reshape(-1)[flat] += eps
        Tm = [[x.copy() for x in row] for row in T]
        Tm[r][c].reshape(-1)[flat] -= eps
        fd = (gi.amplitude(Tp, cfg, samples, strat) - gi.amplitude(Tm, cfg, samples, strat)) / (2 * eps) / amp
        off = sum(x.size for row in T for x in row[:0]) + sum(T[rr][cc].size for rr in range(3) for cc in range(3)
                                                              if rr * 3 + cc < r * 3 + c)
        assert np.allclose(o_full[:, off + flat], fd, rtol=1e-5, atol=1e-7)
    # the sliced O is the active slice of the full one; p holds the slice index
    assert p.shape == o.shape and p.max() < 8


def test_zipup_in_its_exact_regime_equals_no_truncation():
    cfg = gi.GIConfig((3, 4), 2, 2)
    T = gi.init_tensors(cfg, seed=4)
    samples = gi.random_physical_configuration(cfg, 6, seed=5)
    a = gi.amplitude(T, cfg, samples, op.NoTruncation())
    b = gi.amplitude(T, cfg, samples, op.ZipUp(64))
    assert np.allclose(a, b, rtol=1e-10)


def test_plaquette_sweeps_sample_psi_squared():
    cfg = gi.GIConfig((2, 3), 2, 2)
    T = gi.init_tensors(cfg, seed=6)
    strat = op.NoTruncation()
    e, all_samples, psi, _ = gi.dense_hamiltonian_energy(T, cfg, gi.z2_pure_gauge_hamiltonian(cfg.shape), strat)
    target = psi ** 2 / np.sum(psi ** 2)
    n = 4000
    rng = np.random.default_rng(7)
    samples = gi.random_physical_configuration(cfg, n, seed=8)
    R, C = cfg.shape
    counts = np.zeros(len(target))
    index = {tuple(s): i for i, s in enumerate(all_samples)}
    for sweep in range(12):
        cache = gi.init_cache(T, cfg, samples, strat)
        deltas = np.ones((n, R - 1, C - 1), dtype=np.int64)
        u = rng.random((n, R - 1, C - 1))
        samples, amp, _, _ = gi.transition(T, cfg, samples, deltas, u, cache, strat)
        assert np.allclose(amp, gi.amplitude(T, cfg, samples, strat), rtol=1e-10)
        if sweep >= 4:
            for s in samples:
                counts[index[tuple(s)]] += 1
    freq = counts / counts.sum()
    assert np.abs(freq - target).max() < 0.02


@pytest.mark.parametrize("seed", range(8))
def test_random_gi_energies_equal_the_dense_hamiltonian(seed):
    """Random lattices (2..3 x 2..4), N in {2, 3}, degeneracies 1-2 and couplings: the GI oracle's E_loc over
    every gauge-invariant configuration equals (H psi)/psi of the dense Hamiltonian, and ZipUp in its exact
    regime equals NoTruncation."""
    rng = np.random.default_rng(600 + seed)
    N = int(rng.choice([2, 3]))
    shape = (int(rng.integers(2, 4)), int(rng.integers(2, 5 if N == 2 else 4)))
    dmax = int(rng.integers(1, 3))
    cfg = gi.GIConfig(shape, N, dmax)
    T = gi.init_tensors(cfg, seed=seed)
    H = gi.z2_pure_gauge_hamiltonian(shape, h=float(rng.uniform(-1.5, 1.5)), g=float(rng.uniform(0.2, 1.5)), N=N)
    strat = op.NoTruncation()
    e_exact, samples, psi, e_loc = gi.dense_hamiltonian_energy(T, cfg, H, strat)
    top = _forward_top_envs(T, cfg, samples, strat)
    _, energy, _ = gi.estimate(T, cfg, samples, psi, H, strat, top)
    mask = np.abs(psi) > 1e-8 * np.abs(psi).max()
    assert np.allclose(energy[mask], e_loc[mask], rtol=1e-9, atol=1e-9)
    b = gi.amplitude(T, cfg, samples, op.ZipUp(256))
    assert np.allclose(b, psi, rtol=1e-9, atol=1e-12 * np.abs(psi).max())
