"""Randomised known-answer pins of the oracle itself (test infrastructure checking test infrastructure):
on random small lattices, bond dimensions, physical dimensions 2 and 3, real and complex tensors and random
Hermitian operators, the oracle's boundary-MPS amplitudes equal an independent full contraction over all
configurations; every strategy equals NoTruncation in the exact regime (tests/test_peps_strategy_equivalence.py
restated); E_loc equals (H psi)/psi with a matrix-free dense H (tests/test_local_estimate_exact.py
restated); the full gradient equals central finite differences (tests/test_gradients_finite_diff.py)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import exact
from oracle import peps as oracle
from tests.helpers import complex_tensors, uniform_init_tensors
from vmc_gb300.operators import (DiagonalTerm, HorizontalTwoSiteTerm, LocalHamiltonian, OneSiteTerm,
                                 VerticalTwoSiteTerm)


def _draw(seed):
    rng = np.random.default_rng(8000 + seed)
    d = int(rng.choice([2, 3]))
    while True:
        shape = (int(rng.integers(1, 4)), int(rng.integers(1, 4)))
        if d ** (shape[0] * shape[1]) <= 729:
            break
    D = int(rng.integers(2, 4))
    cplx = bool(rng.random() < 0.4)
    T = complex_tensors(shape, D, seed=seed, phys_dim=d) if cplx else uniform_init_tensors(shape, D, phys_dim=d,
                                                                                             seed=seed)
    return rng, shape, D, d, cplx, T


def _operator(rng, shape, d, cplx):
    def herm(n):
        m = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cplx else 0)
        return m + m.conj().T

    R, C = shape
    ops = [OneSiteTerm(r, c, herm(d)) for r in range(R) for c in range(C) if rng.random() < 0.7]
    ops += [HorizontalTwoSiteTerm(r, c, herm(d * d)) for r in range(R) for c in range(C - 1) if rng.random() < 0.7]
    ops += [VerticalTwoSiteTerm(r, c, herm(d * d)) for r in range(R - 1) for c in range(C) if rng.random() < 0.7]
    if R * C >= 2:
        ops.append(DiagonalTerm(((0, 0), (R - 1, C - 1)), rng.standard_normal(d * d)))
    return LocalHamiltonian(shape, tuple(ops))


@pytest.mark.parametrize("seed", range(16))
def test_random_oracle_amplitudes_strategies_and_energies(seed):
    rng, shape, D, d, cplx, T = _draw(seed)
    n = shape[0] * shape[1]
    states = exact.all_configs(n, d)
    model = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle.NoTruncation())
    amp, _, _ = oracle.value_and_grad_occupancy(model, states)
    psi = exact.brute_amplitudes(T, states, shape)
    scale = np.abs(psi).max()
    assert np.max(np.abs(amp - psi)) < 1e-12 * scale
    # every strategy in the exact regime (chi at least every exact boundary bond)
    chi = D ** max(shape)
    for strat in (oracle.ZipUp(chi), oracle.DensityMatrix(chi), oracle.Variational(chi, 2)):
        a, _, _ = oracle.value_and_grad_occupancy(oracle.PEPS(T, shape, D, phys_dim=d, strategy=strat), states)
        assert np.max(np.abs(a - psi)) < 1e-7 * scale, type(strat).__name__
    # E_loc = (H psi) / psi
    H = _operator(rng, shape, d, cplx)
    e_loc = oracle.local_estimate_occupancy(model, states, H, amp)
    hpsi = exact.apply_local_hamiltonian(psi, H.terms, shape, d)
    mask = np.abs(psi) > 1e-6 * scale
    assert np.max(np.abs(e_loc[mask] - hpsi[mask] / psi[mask]) / np.maximum(1.0, np.abs(e_loc[mask]))) < 1e-8


@pytest.mark.parametrize("seed", range(6))
def test_random_oracle_full_gradient_matches_finite_differences(seed):
    rng, shape, D, d, cplx, T = _draw(100 + seed)
    if cplx:  # finite differences along the real parameters of real tensors
        T = uniform_init_tensors(shape, D, phys_dim=d, seed=seed)
    model = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle.NoTruncation())
    sample = rng.integers(0, d, size=(1, shape[0] * shape[1]))
    _, grad, _ = oracle.value_and_grad_occupancy(model, sample, full_gradient=True)
    flat = np.concatenate([t.reshape(-1) for row in T for t in row])
    shapes = [t.shape for row in T for t in row]

    def amp_of(x):
        out, off = [], 0
        for r in range(shape[0]):
            row = []
            for c in range(shape[1]):
                sh = shapes[r * shape[1] + c]
                k = int(np.prod(sh))
                row.append(x[off:off + k].reshape(sh))
                off += k
            out.append(row)
        return exact.brute_amplitudes(out, sample, shape)[0]

    eps = 1e-6
    fd = np.array([0.5 * (amp_of(flat + eps * e) - amp_of(flat - eps * e)) / eps for e in np.eye(flat.size)])
    assert np.max(np.abs(grad[0] - fd)) < 1e-5 * max(1.0, np.abs(fd).max())
