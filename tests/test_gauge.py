"""Gauge removal in the SR solve (vmc_gb300.gauge; the reference ships only its configuration, so parity
is unpinned).  Checked here: every bond generator is an exact null direction of untruncated amplitudes
(the oracle's log-derivatives annihilate it) and the global scale moves every log psi by n_sites; and the
SR update with gauge removal equals the reference's formulation (preconditioners.py:288-309: solve with
O Q, return Q y) evaluated with an explicit dense Q."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import fp32, hamiltonian, make_case
from vmc_gb300 import PEPS, NoTruncation, ZipUp
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.gauge import GaugeConfig, compute_gauge_projection, gauge_generators
from vmc_gb300.lowering import pack_tensors
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import ParameterSpace, SampleSpace


def _model(T, shape, D, chi=4):
    return PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device="cpu", tensors=T)


def test_bond_generators_are_null_directions_of_exact_amplitudes():
    shape, D = (3, 3), 2
    T, cfg, _ = make_case(shape, D, 40, seed=2)
    T = fp32(T)  # the model's parameters are FP32
    model = _model(T, shape, D)
    G = gauge_generators(model).numpy()
    assert G.shape == ((sum(np.asarray(t).size for row in T for t in row)), 12 * D * D + 1)
    om = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    amp, grads, _ = oracle.value_and_grad(om, cfg, full_gradient=True)
    O = grads / amp[:, None]
    bonds = O @ G[:, :-1]
    # zero up to the rounding of O itself (amplitudes are sums with heavy cancellation): compare with
    # random directions of the same norms, along which d log psi is O(|O| |r|)
    R = np.random.default_rng(0).standard_normal(G[:, :-1].shape)
    R *= np.linalg.norm(G[:, :-1], axis=0) / np.linalg.norm(R, axis=0)
    assert np.max(np.abs(bonds)) < 1e-9 * np.median(np.abs(O @ R))
    # d log psi along theta = one per site
    assert np.allclose(O @ G[:, -1], shape[0] * shape[1], rtol=1e-10)


def test_projection_is_orthogonal_and_spans_the_generators():
    shape, D = (3, 4), 3
    T, _, _ = make_case(shape, D, 1, seed=3)
    model = _model(T, shape, D)
    proj, info = compute_gauge_projection(GaugeConfig(), model, None, return_info=True)
    U = proj.U
    assert torch.allclose(U.T @ U, torch.eye(U.shape[1], dtype=U.dtype), atol=1e-12)
    G = gauge_generators(model)
    assert torch.linalg.norm(proj.project(G)) < 1e-10 * torch.linalg.norm(G)
    # the scalar bond gauges are dependent around each of the 6 plaquettes of the 3 x 4 lattice
    assert info["n_generators"] == 17 * D * D + 1 and info["rank"] == 17 * D * D - 6 + 1
    Q = proj.dense()
    assert Q.shape == (proj.n_params, proj.n_params - info["rank"])
    x = torch.randn(proj.n_params, dtype=torch.float64)
    assert torch.allclose(Q @ (Q.T @ x), proj.project(x), atol=1e-10)


@pytest.mark.parametrize("space", [SampleSpace(), ParameterSpace()], ids=["sample", "parameter"])
def test_sr_update_with_gauge_removal_matches_the_dense_formulation(emu_lib, space):
    shape, D, chi, n = (3, 3), 2, 4, 48
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, n, seed=5)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, full_gradient=True)
    model = _model(fp32(T), shape, D, chi)
    shift = 1e-3
    pre = SRPreconditioner(space=space, diag_shift=shift, gauge_config=GaugeConfig())
    upd, metrics = pre.apply(model, model.tensors, res.configs, res.O, None, res.E)
    x = model.packed(upd)
    # the reference's flow with an explicit Q
    Q = compute_gauge_projection(GaugeConfig(), model, model.tensors).dense()
    O = res.O.double()
    o_eff = O @ Q
    oc = o_eff - o_eff.mean(0)
    e = res.E.double()
    dv = (e - e.mean()) / n
    if isinstance(space, SampleSpace):
        y = torch.linalg.solve(oc @ oc.T / n + shift * torch.eye(n, dtype=torch.float64), dv)
        red = oc.T @ y
    else:
        red = torch.linalg.solve(oc.T @ oc / n + shift * torch.eye(Q.shape[1], dtype=torch.float64), oc.T @ dv)
    want = 2.0 * (Q @ red)
    assert torch.linalg.norm(x - want) / torch.linalg.norm(want) < 1e-6  # x is returned in FP32
    # no component along the gauge directions
    proj = compute_gauge_projection(GaugeConfig(), model, model.tensors)
    assert torch.linalg.norm(proj.U.T @ x.double()) < 1e-6 * torch.linalg.norm(x)
    assert metrics["gauge_rank"] == proj.rank


def test_qr_solve_with_gauge_removal_matches_the_dense_formulation(emu_lib, monkeypatch):
    """QRSolve (ParameterSpace, full Jacobian, diag shift unused): the min-norm solution of (O P) x = dv
    against the reference's Q (O Q)^+ dv with an explicit Q.  The pivoted QR runs in the host build."""
    import vmc_gb300.linalg as linalg
    from vmc_gb300.preconditioners import QRSolve

    monkeypatch.setattr(linalg, "_resolve_lib", lambda lib, device: emu_lib)

    shape, D, chi, n = (3, 3), 2, 4, 40
    H = hamiltonian("tfim", shape)
    T, cfg, u = make_case(shape, D, n, seed=6)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u), cache, full_gradient=True)
    model = _model(fp32(T), shape, D, chi)
    pre = SRPreconditioner(space=ParameterSpace(), strategy=QRSolve(), gauge_config=GaugeConfig())
    upd, metrics = pre.apply(model, model.tensors, res.configs, res.O, None, res.E)
    x = model.packed(upd).double()
    Q = compute_gauge_projection(GaugeConfig(), model, model.tensors).dense()
    oc = res.O.double() @ Q
    oc = oc - oc.mean(0)
    e = res.E.double()
    dv = (e - e.mean()) / n
    want = 2.0 * (Q @ (torch.linalg.pinv(oc, rtol=1e-12) @ dv))
    assert torch.linalg.norm(x - want) / torch.linalg.norm(want) < 1e-5


@pytest.mark.parametrize("seed", range(8))
def test_random_lattices_gauge_projection_and_null_directions(seed):
    """Random lattices (1..4 x 1..4), D in {2, 3}, d in {2, 3}: U is orthonormal and removes every generator,
    its rank is the numerical rank of the generators, and every bond generator annihilates the oracle's
    exact log-derivatives."""
    rng = np.random.default_rng(600 + seed)
    shape = (int(rng.integers(1, 5)), int(rng.integers(1, 5)))
    D, d = int(rng.integers(2, 4)), int(rng.choice([2, 3]))
    R_, C_ = shape
    T, cfg, _ = make_case(shape, D, 12, seed=seed, phys_dim=d)
    T = fp32(T)
    model = PEPS(shape=shape, bond_dim=D, phys_dim=d, contraction_strategy=NoTruncation(), device="cpu", tensors=T)
    G = gauge_generators(model)
    n_bonds = R_ * (C_ - 1) + (R_ - 1) * C_
    assert G.shape[1] == n_bonds * D * D + 1
    proj, info = compute_gauge_projection(GaugeConfig(), model, None, return_info=True)
    U = proj.U
    assert torch.allclose(U.T @ U, torch.eye(U.shape[1], dtype=U.dtype), atol=1e-12)
    assert torch.linalg.norm(proj.project(G)) < 1e-10 * torch.linalg.norm(G)
    # at most one per generator less one scalar dependency per plaquette; boundary tensors of rank < D
    # (d < D at a corner) add exact dependencies X = u v^T with A u = 0 and v^T B = 0
    assert info["rank"] <= n_bonds * D * D - (R_ - 1) * (C_ - 1) + 1
    sv = np.linalg.svd(G.numpy(), compute_uv=False)
    assert info["rank"] == int((sv > 1e-10 * sv[0]).sum())
    om = oracle.PEPS(T, shape, D, phys_dim=d, strategy=oracle.NoTruncation())
    amp, grads, _ = oracle.value_and_grad_occupancy(om, cfg, full_gradient=True)
    O = grads / amp[:, None]
    Gn = G.numpy()
    if n_bonds:
        Rr = np.random.default_rng(seed).standard_normal(Gn[:, :-1].shape)
        Rr *= np.linalg.norm(Gn[:, :-1], axis=0) / np.linalg.norm(Rr, axis=0)
        assert np.max(np.abs(O @ Gn[:, :-1])) < 1e-8 * np.median(np.abs(O @ Rr))
    assert np.allclose(O @ Gn[:, -1], R_ * C_, rtol=1e-9)
