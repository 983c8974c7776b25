"""Pins the oracle's sequential Metropolis sampler (tests/test_sequential_sampling.py:126-208)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import exact
from oracle import peps as oracle
from tests.helpers import uniform_init_tensors
from vmc_gb300.operators import LocalHamiltonian


@pytest.mark.parametrize("seed", [42, 91])
def test_sampled_histogram_matches_exact_probabilities(seed):
    """3x3, D=3, NoTruncation: histogram vs |psi|^2, max abs deviation 2e-3 (40,960 samples)."""
    shape, D = (3, 3), 3
    T = uniform_init_tensors(shape, D, seed=seed)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    basis = exact.all_configs(9)
    probs = np.abs(oracle.value(model, basis)) ** 2
    probs /= probs.sum()
    init, trans, est = oracle.build_mc_kernels(model, LocalHamiltonian(shape, ()))
    rng = np.random.default_rng(seed)
    n_chains, n_steps, burn = 2048, 20, 5
    cfg = rng.integers(0, 2, size=(n_chains, 9))
    cache = init(T, cfg)
    counts = np.zeros(512)
    weights = 1 << np.arange(8, -1, -1)
    for step in range(burn + n_steps):
        cfg, ctx = trans(T, cfg, rng.random((n_chains, 9)), cache)
        cache, _ = est(T, cfg, ctx)
        if step >= burn:
            counts += np.bincount(cfg @ weights, minlength=512)
    emp = counts / counts.sum()
    assert np.max(np.abs(emp - probs)) < 2e-3


def test_full_and_sliced_gradients_consistent_and_p_matches():
    """test_sequential_sampling.py:152-208: identical samples for full/sliced, sliced == full[active], p."""
    shape, D = (3, 3), 3
    T = uniform_init_tensors(shape, D, seed=10001)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    H = LocalHamiltonian(shape, ())
    rng = np.random.default_rng(17)
    cfg0 = rng.integers(0, 2, size=(10, 9))
    u = rng.random((3, 10, 9))
    out = {}
    for full in (False, True):
        init, trans, est = oracle.build_mc_kernels(model, H, full_gradient=full)
        sampler = oracle.make_mc_sampler(trans, est)
        (_, _), (hist, le, _) = sampler(T, cfg0.copy(), u, init(T, cfg0), n_steps=3)
        out[full] = (hist, le)
    assert np.array_equal(out[False][0], out[True][0])
    sl, fu = out[False][1], out[True][1]
    assert fu.active_slice_indices is None
    assert fu.local_log_derivatives.shape[-1] == 2 * sl.local_log_derivatives.shape[-1]
    pps = oracle.params_per_site(model)
    samples = out[False][0].reshape(-1, 9)
    o_s = sl.local_log_derivatives.reshape(samples.shape[0], -1)
    o_f = fu.local_log_derivatives.reshape(samples.shape[0], -1)
    off_s = off_f = 0
    for site, n in enumerate(pps):
        blk = o_f[:, off_f:off_f + 2 * n].reshape(-1, 2, n)
        sel = blk[np.arange(samples.shape[0]), samples[:, site]]
        assert np.max(np.abs(sel - o_s[:, off_s:off_s + n])) < 1e-14
        off_s += n
        off_f += 2 * n
    _, _, p_ref = oracle.value_and_grad(model, samples)
    assert np.array_equal(sl.active_slice_indices.reshape(samples.shape[0], -1), p_ref)


def test_sample_counts_and_trim():
    """src/vmc/core/sampling.py:76-82."""
    assert oracle.sample_counts(4096, 4096) == (4096, 4096, 1, 4096)
    assert oracle.sample_counts(100, 8) == (100, 8, 13, 104)
    x = np.arange(13 * 8 * 3).reshape(13, 8, 3)
    t = oracle.trim_samples(x, 104, 100)
    assert t.shape == (100, 3) and np.array_equal(t[0], x[0, 0])
