"""The vector-Jacobian product, the torch.library operators and the cache-budget recompute switch on
sm_103a (through the C ABI)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import fp32, hamiltonian, make_case
from vmc_gb300 import PEPS, ZipUp, ops
from vmc_gb300.compat import peps_apply
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.kernels import build_mc_kernels
from vmc_gb300.lowering import pack_tensors

pytestmark = pytest.mark.gpu


def test_peps_apply_backward_matches_the_oracle_adjoint(cuda_device):
    shape, D, chi = (4, 4), 3, 6
    T, cfg, _ = make_case(shape, D, 64, seed=4)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, tensors=fp32(T))
    packed = model.packed().clone().requires_grad_(True)
    amp = peps_apply(packed, torch.from_numpy(cfg).to(cuda_device), shape, None, model=model)
    g = np.random.default_rng(5).standard_normal(64)
    (amp * torch.from_numpy(g).to(cuda_device)).sum().backward()
    om = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    amp_ref, grads, _ = oracle.value_and_grad(om, cfg, full_gradient=True)
    assert np.allclose(amp.detach().cpu().numpy(), amp_ref, rtol=1e-4, atol=0)
    want = (g[:, None] * grads).sum(0)
    got = packed.grad.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-4


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_vjp_equals_weighted_rows_at_8x8(cuda_device, precision):
    """8x8 D4 chi16, 1216 chains: the kernel-accumulated sum_i w_i O_i equals the weighted rows of
    vmc_peps_amp_grad (FP64 atomics: order of the additions only)."""
    shape, D, chi, n = (8, 8), 4, 16, 1216
    T, cfg, _ = make_case(shape, D, n, seed=6)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", device=cuda_device, precision=precision)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    _, _, O = eng.amp_grad(tens, c, full_gradient=True)
    w = torch.from_numpy(np.random.default_rng(1).standard_normal(n)).to(cuda_device)
    want = (w[:, None] * O.double()).sum(0)
    got = eng.vjp(tens, c, w)
    torch.cuda.synchronize()
    eng.raise_on_status()
    assert torch.linalg.norm(got - want) / torch.linalg.norm(want) < 1e-10


def test_operators_fake_shapes_match_real_outputs(cuda_device):
    shape, D, chi = (4, 4), 3, 6
    T, cfg, u = make_case(shape, D, 8, seed=7)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device=cuda_device)
    h = ops.register_engine(eng)
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    la, sg, O = ops.amp_grad(h, tens, c, True)
    E = ops.local_energy(h, tens, c, la, sg)
    torch.library.opcheck(ops.amp_grad, (h, tens, c, False))
    torch.library.opcheck(ops.local_energy, (h, tens, c, la, sg))
    torch.library.opcheck(ops.vjp, (h, tens, c, torch.ones(8, dtype=torch.float64, device=cuda_device)))
    assert O.shape == (8, eng.n_params_full) and E.shape == (8,)


def test_cache_budget_switch_at_16x16_D6_chi48(cuda_device):
    """16x16, D=6, chi=48 (the uneven batch's largest lattice): ~14 MB of bottom environments per chain.
    Over the budget, init_cache keeps none and the sweep recomputes them in the launch; the sampled
    configurations, energies and log-derivatives are the same bits as with the cache."""
    shape, D, chi, n = (16, 16), 6, 48, 16
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, n, seed=9)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, tensors=T)
    per_chain = model.engine(H).cache_bytes(1)
    assert per_chain > 10 << 20
    outs = []
    for budget in (None, per_chain * n - 1):
        init, trans, est = build_mc_kernels(model, H, cache_budget_bytes=budget)
        c0 = torch.from_numpy(cfg).to(cuda_device)
        cache = init(model.tensors, c0)
        assert (cache.bottom_envs is None) == (budget is not None)
        c2, _, ctx = trans(model.tensors, c0, torch.from_numpy(u).to(cuda_device), cache)
        torch.cuda.synchronize()
        outs.append((c2, ctx.estimates))
    (ca, ea), (cb, eb) = outs
    assert torch.equal(ca, cb) and torch.equal(ea.local_estimate, eb.local_estimate)
    assert torch.equal(ea.local_log_derivatives, eb.local_log_derivatives)
    assert torch.isfinite(ea.local_estimate).all()
