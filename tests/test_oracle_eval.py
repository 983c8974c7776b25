"""Pins the FP64 oracle's amplitudes and gradients with exact, reference-independent answers.

Restates tests/test_peps_eval.py:18-77 (sliced gradients vs autodiff over all
configurations), tests/test_gradients_finite_diff.py:35-78 (central finite
differences) and tests/test_peps_strategy_equivalence.py:16-41 (strategies vs
NoTruncation in the exact regime) of the reference.
"""
from __future__ import annotations

import string

import numpy as np
import pytest
import torch

from oracle import exact
from oracle import peps as oracle
from tests.helpers import uniform_init_tensors
from vmc_gb300.synthetic import random_tensors


def _torch_amplitude(tensors, config, shape):
    """Independent brute-force contraction in torch (autograd-able), row transfer vectors."""
    n_rows, n_cols = shape
    letters = string.ascii_letters
    state = torch.ones((1,) * n_cols, dtype=torch.float64)
    for r in range(n_rows):
        state = state[..., None]
        for c in range(n_cols):
            a = tensors[r][c][int(config[r * n_cols + c])]  # (up, down, left, right)
            legs = list(letters[:n_cols])
            src = "".join(legs) + "H"
            out = legs.copy()
            out[c] = "D"
            state = torch.einsum(f"{src},{legs[c]}DHR->{''.join(out)}R", state, a)
        state = state[..., 0]
    return state.reshape(())


def test_all_configs_amplitudes_and_sliced_gradients_match_autodiff():
    """tests/test_peps_eval.py:18-77: 3x3, D=4, NoTruncation, all 512 configurations, 1e-12."""
    shape, D = (3, 3), 4
    T = uniform_init_tensors(shape, D, seed=0)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    cfg = exact.all_configs(9)
    amp, grads, p = oracle.value_and_grad(model, cfg)
    amp_brute = exact.brute_amplitudes(T, cfg, shape)
    assert np.max(np.abs(amp - amp_brute)) < 1e-12 * max(1.0, np.abs(amp_brute).max())

    tt = [[torch.tensor(t, requires_grad=True) for t in row] for row in T]
    leaves = [t for row in tt for t in row]
    pps = oracle.params_per_site(model)
    for i in range(0, 512, 37):  # a spread of configurations
        a = _torch_amplitude(tt, cfg[i], shape)
        gfull = torch.autograd.grad(a, leaves)
        sliced = []
        for s, g in enumerate(gfull):
            sliced.append(g[cfg[i][s]].reshape(-1).numpy())
        ref = np.concatenate(sliced)
        assert float(a) == pytest.approx(amp[i], rel=1e-12, abs=1e-14)
        assert np.max(np.abs(grads[i] - ref)) < 1e-12 * max(1.0, np.abs(ref).max())
    assert p.shape == grads.shape
    assert np.array_equal(p[:, :pps[0]], np.repeat(cfg[:, :1], pps[0], axis=1).astype(np.int8))


def test_full_gradient_matches_central_finite_differences():
    """tests/test_gradients_finite_diff.py:35-78: 2x3, D=3, eps=1e-6, tol 1e-5."""
    shape, D = (2, 3), 3
    T = uniform_init_tensors(shape, D, seed=1)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    rng = np.random.default_rng(1)
    sample = rng.integers(0, 2, size=(1, 6))
    _, grad, _ = oracle.value_and_grad(model, sample, full_gradient=True)
    flat = np.concatenate([t.reshape(-1) for row in T for t in row])
    shapes = [t.shape for row in T for t in row]

    def amp_of(x):
        out, off = [], 0
        for r in range(shape[0]):
            row = []
            for c in range(shape[1]):
                sh = shapes[r * shape[1] + c]
                n = int(np.prod(sh))
                row.append(x[off:off + n].reshape(sh))
                off += n
            out.append(row)
        return oracle.peps_apply(out, sample, shape, oracle.NoTruncation())[0]

    eps = 1e-6
    fd = np.zeros_like(flat)
    for i in range(flat.size):
        e = np.zeros_like(flat)
        e[i] = eps
        fd[i] = 0.5 * (amp_of(flat + e) - amp_of(flat - e)) / eps
    assert np.max(np.abs(grad[0] - fd)) < 1e-5


@pytest.mark.parametrize("strategy", [oracle.ZipUp(16), oracle.DensityMatrix(16), oracle.Variational(16, 2)],
                         ids=["ZipUp", "DensityMatrix", "Variational"])
def test_strategies_match_no_truncation_in_exact_regime(strategy):
    """tests/test_peps_strategy_equivalence.py:16-41: 3x3, D=4, 64 samples, tol 1e-7."""
    shape, D = (3, 3), 4
    T = uniform_init_tensors(shape, D, seed=0)
    rng = np.random.default_rng(0)
    samples = rng.integers(0, 2, size=(64, 9))
    ref = oracle.peps_apply(T, samples, shape, oracle.NoTruncation())
    amps = oracle.peps_apply(T, samples, shape, strategy)
    assert np.max(np.abs(amps - ref)) < 1e-7 * max(1.0, np.abs(ref).max())


def test_config1_zipup_truncation_regime():
    """4x4, D=2 (the CPU-runnable case).  The zip-up SVD at a cut sees only the
    local theta matrix (rank up to 8 here), not the rank-4 Schmidt decomposition
    of the whole boundary state, so ZipUp(4) is an ACTIVE truncation (large
    deviations from the exact amplitude) while ZipUp(8) is exact."""
    shape, D = (4, 4), 2
    T = random_tensors(shape, D, seed=0)
    rng = np.random.default_rng(5)
    samples = rng.integers(0, 2, size=(256, 16))
    ref = oracle.peps_apply(T, samples, shape, oracle.NoTruncation())
    brute = exact.brute_amplitudes(T, samples, shape)
    assert np.max(np.abs(ref / brute - 1)) < 1e-11
    exact8 = oracle.peps_apply(T, samples, shape, oracle.ZipUp(8))
    assert np.max(np.abs(exact8 / ref - 1)) < 1e-9
    trunc4 = oracle.peps_apply(T, samples, shape, oracle.ZipUp(4))
    assert np.median(np.abs(trunc4 / ref - 1)) > 1e-2


def test_spin_and_occupancy_inputs_agree():
    """compat.py:38: peps_apply accepts +-1 spins or 0/1 occupancies (spin_to_occupancy is idempotent)."""
    shape, D = (2, 2), 2
    T = uniform_init_tensors(shape, D, seed=3)
    occ = exact.all_configs(4)
    spins = 2 * occ - 1
    a = oracle.peps_apply(T, occ, shape, oracle.NoTruncation())
    b = oracle.peps_apply(T, spins, shape, oracle.NoTruncation())
    assert np.array_equal(a, b)
