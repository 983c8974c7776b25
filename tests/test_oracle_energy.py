"""Pins the oracle's local energies and MC estimators against exact answers.

Restates tests/test_local_estimate_exact.py:24-124 (E_loc == (H psi)/psi with a
dense/matrix-free H instead of NetKet's) and
tests/test_mc_energy_grad_evaluator.py:58-189 (MC energy and gradient vs the
exact full sum) of the reference.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import exact
from oracle import peps as oracle
from tests.helpers import uniform_init_tensors
from vmc_gb300.operators import (
    DiagonalTerm,
    HorizontalTwoSiteTerm,
    LocalHamiltonian,
    OneSiteTerm,
    VerticalTwoSiteTerm,
    heisenberg,
    transverse_field_ising,
)


def _marshall_heisenberg(shape):
    """The reference test's bond operator sz.sz - 2 (s+s- + s-s+) (test_local_estimate_exact.py:20-47)."""
    szsz = np.diag([1.0, -1.0, -1.0, 1.0])
    exch = np.zeros((4, 4))
    exch[1, 2] = exch[2, 1] = 2.0
    return heisenberg(shape, bond_op=szsz - exch)


@pytest.mark.parametrize("kind", ["marshall", "heisenberg_S", "tfim"])
def test_local_estimate_matches_matrix_free_hamiltonian(kind):
    """tests/test_local_estimate_exact.py:24-79: 2x3, D=3, NoTruncation, all states, 1e-9."""
    shape = (2, 3)
    H = {"marshall": _marshall_heisenberg, "heisenberg_S": heisenberg,
         "tfim": transverse_field_ising}[kind](shape)
    T = uniform_init_tensors(shape, 3, seed=1)
    model = oracle.PEPS(T, shape, 3, strategy=oracle.NoTruncation())
    states = exact.all_configs(6)
    amps = oracle.value(model, states)
    e_loc = oracle.local_estimate(model, states, H, amps)
    psi = exact.brute_amplitudes(T, states, shape)
    hpsi = exact.apply_local_hamiltonian(psi, H.terms, shape, 2)
    mask = np.abs(amps) > 1e-12
    assert np.max(np.abs(e_loc[mask] - hpsi[mask] / psi[mask])) < 1e-9


def test_local_estimate_uses_operator_columns():
    """The reference evaluates op[:, s] (energy.py:176-200); pin it with non-symmetric operators."""
    shape = (2, 2)
    rng = np.random.default_rng(4)
    terms = (OneSiteTerm(0, 1, rng.standard_normal((2, 2))),
             HorizontalTwoSiteTerm(1, 0, rng.standard_normal((4, 4))),
             VerticalTwoSiteTerm(0, 0, rng.standard_normal((4, 4))),
             DiagonalTerm(((0, 0), (1, 1)), rng.standard_normal(4)))
    H = LocalHamiltonian(shape, terms)
    T = uniform_init_tensors(shape, 2, seed=2)
    model = oracle.PEPS(T, shape, 2, strategy=oracle.NoTruncation())
    states = exact.all_configs(4)
    amps = oracle.value(model, states)
    e_loc = oracle.local_estimate(model, states, H, amps)
    psi = exact.brute_amplitudes(T, states, shape)
    hpsi = exact.apply_local_hamiltonian(psi, H.terms, shape, 2)
    assert np.max(np.abs(e_loc - hpsi / psi)) < 1e-10


def test_mc_energy_and_gradient_match_full_sum():
    """tests/test_mc_energy_grad_evaluator.py:160-189: 3x3, D=3, Heisenberg, 8192 samples, 6 sigma."""
    shape, D = (3, 3), 3
    H = _marshall_heisenberg(shape)
    T = uniform_init_tensors(shape, D, seed=1)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    states = exact.all_configs(9)
    amps, grads, _ = oracle.value_and_grad(model, states, full_gradient=True)
    e_all = oracle.local_estimate(model, states, H, amps)
    e_exact, g_exact = exact.full_sum_energy_and_grad(amps, grads / amps[:, None], e_all)

    n_chains, n_steps, burn = 1024, 8, 4
    rng = np.random.default_rng(0)
    init, trans, est = oracle.build_mc_kernels(model, H, full_gradient=True)
    cfg = rng.integers(0, 2, size=(n_chains, 9))
    cache = init(T, cfg)
    es, os_ = [], []
    for step in range(burn + n_steps):
        cfg, ctx = trans(T, cfg, rng.random((n_chains, 9)), cache)
        cache, le = est(T, cfg, ctx)
        if step >= burn:
            es.append(le.local_estimate)
            os_.append(le.local_log_derivatives)
    e = np.concatenate(es)
    o = np.concatenate(os_)
    e_mc = e.mean()
    contrib = (e - e_mc)[:, None] * o.conj()
    g_mc = contrib.mean(axis=0)
    e_err = np.sqrt(np.mean(np.abs(e - e_mc) ** 2) / e.shape[0])
    g_err = np.sqrt(np.mean(np.abs(contrib - g_mc) ** 2, axis=0) / e.shape[0])
    assert abs(e_mc - e_exact) < 6.0 * (e_err + 1e-12)
    assert np.linalg.norm(g_mc - g_exact) < 6.0 * (np.linalg.norm(g_err) + 1e-12)
