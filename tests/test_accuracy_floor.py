"""Where the accuracy floor of a truncated boundary-MPS contraction comes from, measured on the FP64
oracle with FP32 / TF32 / BF16 rounding injected at one place at a time (the experiments behind the
design's accuracy findings):

- 8x8 Heisenberg, D=4, ZipUp(16) (strategy.py:128-150): an exact (FP64) decomposition of FP32-rounded
  theta, or FP32 storage of the boundary tensors and carry, stays inside the bars (batch-mean E within
  1e-5 of the energy scale, O_k within 1e-4 Frobenius); what misses them is FP32 arithmetic inside the
  decomposition (the engine's FP32 tier, checked in test_mixed_emulation.py).
- The gauge-invariant PEPS (pure Z2, model.py:392-1046): contraction operands rounded to TF32 or BF16
  (results to FP32, SVD in FP64) miss the bars by orders of magnitude; FP32 operands do not.

Rounding keeps the oracle's exponent range (frexp-based): the oracle does not normalise its tensors.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle.gi as ogi
import oracle.peps as op
from tests.helpers import E_BAR, O_BAR, fp32, hamiltonian, make_case, oracle_sweep


def _round(x, bits):
    x = np.asarray(x)
    if not np.issubdtype(x.dtype, np.floating):
        return x
    m, e = np.frexp(x)
    s = float(2 ** bits)
    return np.ldexp(np.round(m * s) / s, e)


def _zip_up_rounded(round_theta, round_out):
    """strategy.py:128-150 with theta and/or the outputs (kept tensors, carry) rounded to 24 bits."""
    def apply(mps, mpo, chi):
        new, carry = [], None
        for i, (m, w) in enumerate(zip(mps, mpo)):
            theta, left, phys, dr, wr = op.contract_theta(m, w, carry)
            if round_theta:
                theta = _round(theta, 24)
            z = theta.shape[0]
            if i == len(mps) - 1:
                t = theta.reshape(z, left, phys, dr * wr)
                new.append(_round(t, 24) if round_out else t)
                break
            u, s, vh = np.linalg.svd(theta.reshape(z, left * phys, dr * wr), full_matrices=False)
            k = min(chi, s.shape[-1])
            uk = u[..., :k].reshape(z, left, phys, k)
            new.append(_round(uk, 24) if round_out else uk)
            carry = (s[..., :k, None] * vh[..., :k, :]).reshape(z, k, dr, wr)
            if round_out:
                carry = _round(carry, 24)
        return tuple(new)
    return apply


def _errors(ref, got):
    (c_ref, ctx_ref, le_ref), (c, ctx, le) = ref, got
    same = np.all(c == c_ref, axis=1)
    e, e_ref = le.local_estimate[same], le_ref.local_estimate[same]
    o, o_ref = le.local_log_derivatives[same], le_ref.local_log_derivatives[same]
    return (same.mean(), abs(e.mean() - e_ref.mean()) / np.abs(e_ref).mean(),
            np.linalg.norm(o - o_ref) / np.linalg.norm(o_ref))


@pytest.mark.parametrize("round_theta,round_out", [(True, False), (False, True), (True, True)],
                         ids=["theta", "stored", "both"])
def test_exact_decomposition_of_fp32_inputs_meets_the_bars(monkeypatch, round_theta, round_out):
    shape, D, chi = (8, 8), 4, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 16, seed=0)
    T32 = fp32(T)
    ref = oracle_sweep(T32, shape, D, "ZipUp", chi, H, cfg, u)
    monkeypatch.setattr(op, "apply_mpo_zip_up", _zip_up_rounded(round_theta, round_out))
    same, de, do = _errors(ref, oracle_sweep(T32, shape, D, "ZipUp", chi, H, cfg, u))
    assert same == 1.0
    assert de < E_BAR and do < O_BAR, (de, do)


def _gi_run(T, cfg, H, strat, samples, deltas, u):
    cache = ogi.init_cache(T, cfg, samples, strat)
    s, amp, top, _ = ogi.transition(T, cfg, samples, deltas, u, cache, strat)
    grads, e, _ = ogi.estimate(T, cfg, s, amp, H, strat, top)
    o, _ = ogi.local_log_derivatives(T, cfg, s, grads, amp)
    return s, e, o


@pytest.mark.parametrize("bits,fails", [(24, False), (11, True), (8, True)], ids=["fp32", "tf32", "bf16"])
def test_gi_contraction_operand_precision(monkeypatch, bits, fails):
    shape, chi, n = (6, 6), 16, 16
    cfg = ogi.GIConfig(shape, 2, 2)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in ogi.init_tensors(cfg, seed=0)]
    H = ogi.z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.5, N=2)
    strat = op.ZipUp(chi)
    samples = ogi.random_physical_configuration(cfg, n, seed=3)
    rng = np.random.default_rng(4)
    u = rng.random((n, shape[0] - 1, shape[1] - 1))
    deltas = np.ones((n, shape[0] - 1, shape[1] - 1), dtype=np.int64)
    s_ref, e_ref, o_ref = _gi_run(T, cfg, H, strat, samples, deltas, u)

    ein, plaq, zip_up = op._ein, ogi._plaquette_amp, op.apply_mpo_zip_up

    def ein_r(sub, *ops, path=None):
        return _round(ein(sub, *[_round(x, bits) for x in ops], path=path), 24)

    def plaq_r(*a):
        return _round(plaq(*[_round(x, bits) if isinstance(x, np.ndarray) else x for x in a]), 24)

    monkeypatch.setattr(op, "_ein", ein_r)
    monkeypatch.setattr(ogi, "_ein", ein_r)
    monkeypatch.setattr(ogi, "_plaquette_amp", plaq_r)
    monkeypatch.setattr(op, "apply_mpo_zip_up", lambda m, w, c: tuple(_round(x, 24) for x in zip_up(m, w, c)))
    s, e, o = _gi_run(T, cfg, H, strat, samples, deltas, u)
    same = np.all(s == s_ref, axis=1)
    de = abs(e[same].mean() - e_ref[same].mean()) / np.abs(e_ref[same]).mean()
    do = np.linalg.norm(o[same] - o_ref[same]) / np.linalg.norm(o_ref[same])
    if fails:
        # TF32 (2^-11) and BF16 (2^-8) operands: O_k at least 10x beyond its bar
        assert do > 10 * O_BAR, (de, do)
    else:
        assert de < E_BAR and do < O_BAR, (de, do)
