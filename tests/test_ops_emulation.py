"""The torch.library operators and the engine's vector-Jacobian product in the host-emulation build.

peps_apply's backward (vmc_peps_vjp: w_i = g_i psi_i, accumulated in the kernel) against the oracle's
hand-written adjoint (compat.py:49-61 restated) for real and complex PEPS; the operators' schemas, fake
implementations and autograd registration through torch.library.opcheck; and build_mc_kernels' cache
budget, over which the sweeps recompute the bottom environments with the same results."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import complex_tensors, fp32, hamiltonian, make_case
from vmc_gb300 import PEPS, ZipUp, ops
from vmc_gb300.compat import peps_apply
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.kernels import build_mc_kernels
from vmc_gb300.lowering import pack_tensors


def _model(emu_lib, T, shape, D, chi, dtype=torch.float32):
    return PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device="cpu", lib=emu_lib, tensors=T,
                dtype=dtype)


def _oracle_grad(T, shape, D, chi, cfg, g):
    """sum_i g_i conj(dpsi_i/dtheta) over the full layout, from the oracle's adjoint."""
    model = oracle.PEPS(T, shape, D, strategy=oracle.ZipUp(chi))
    amp, grads, _ = oracle.value_and_grad(model, cfg, full_gradient=True)
    return amp, (g[:, None] * np.conj(grads)).sum(0)


@pytest.mark.parametrize("cplx", [False, True], ids=["real", "complex"])
def test_peps_apply_backward_is_the_oracle_adjoint(emu_lib, cplx):
    shape, D, chi = (3, 4), 3, 6
    if cplx:
        T = complex_tensors(shape, D, seed=4)
        cfg = np.random.default_rng(4).integers(0, 2, (7, 12)).astype(np.int32)
    else:
        T, cfg, _ = make_case(shape, D, 7, seed=4)
        T = fp32(T)
    model = _model(emu_lib, T, shape, D, chi, torch.complex64 if cplx else torch.float32)
    packed = model.packed().clone().requires_grad_(True)
    amp = peps_apply(packed, torch.from_numpy(cfg), shape, None, model=model)
    rng = np.random.default_rng(5)
    g = rng.standard_normal(7) + (1j * rng.standard_normal(7) if cplx else 0)
    (amp * torch.from_numpy(np.conj(g) if cplx else g)).real.sum().backward()
    amp_ref, grad_ref = _oracle_grad(T, shape, D, chi, cfg, g)
    assert np.allclose(amp.detach().numpy(), amp_ref, rtol=2e-5, atol=0)
    got = packed.grad.numpy()
    assert np.linalg.norm(got - grad_ref) / np.linalg.norm(grad_ref) < 2e-5


def test_vjp_equals_the_weighted_sum_of_log_derivative_rows(emu_lib):
    """vmc_peps_vjp accumulates sum_i w_i O_i in FP64: the rows vmc_peps_amp_grad writes, weighted."""
    shape, D, chi = (4, 4), 3, 6
    T, cfg, _ = make_case(shape, D, 9, seed=6)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", device="cpu", lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    _, _, O = eng.amp_grad(tens, c, full_gradient=True)
    w = torch.from_numpy(np.random.default_rng(1).standard_normal(9))
    want = (w[:, None] * O.double()).sum(0)
    got = eng.vjp(tens, c, w)
    assert torch.allclose(got, want, rtol=1e-12, atol=1e-12)
    assert eng.status() == 0


def test_operators_pass_opcheck(emu_lib):
    shape, D, chi = (3, 3), 2, 4
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 5, seed=7)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib)
    h = ops.register_engine(eng)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg)
    la, sg, _ = eng.amp_grad(tens, c)
    torch.library.opcheck(ops.amp_grad, (h, tens, c, False))
    torch.library.opcheck(ops.vjp, (h, tens, c, torch.ones(5, dtype=torch.float64)))
    torch.library.opcheck(ops.local_energy, (h, tens, c, la, sg))
    torch.library.opcheck(ops.peps_amplitude, (h, tens.clone().requires_grad_(True), c))
    cache = eng.init_cache(tens, c.clone())
    torch.library.opcheck(ops.sweep, (h, tens, c.clone(), torch.from_numpy(u), cache, None, False),
                          test_utils=("test_schema", "test_faketensor"))


def test_over_the_cache_budget_sweeps_recompute_with_the_same_results(emu_lib):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 6, seed=8)
    model = _model(emu_lib, fp32(T), shape, D, chi)
    outs = []
    for budget in (None, 0):
        init, trans, est = build_mc_kernels(model, H, cache_budget_bytes=budget)
        cache = init(model.tensors, torch.from_numpy(cfg))
        assert (cache.bottom_envs is None) == (budget == 0)
        c2, _, ctx = trans(model.tensors, torch.from_numpy(cfg), torch.from_numpy(u), cache)
        outs.append((c2, ctx.estimates))
    (ca, ea), (cb, eb) = outs
    assert torch.equal(ca, cb)
    assert torch.equal(ea.local_estimate, eb.local_estimate)
    assert torch.equal(ea.local_log_derivatives, eb.local_log_derivatives)
