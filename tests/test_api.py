"""The reference-facing Python surface: operators, lowering, kernels, sampler, compat, driver."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import exact
from oracle import peps as oracle
from tests.helpers import fp32, uniform_init_tensors
from vmc_gb300.lowering import lower_operator, pack_tensors, params_per_site
from vmc_gb300.operators import (
    DiagonalTerm,
    HorizontalTwoSiteTerm,
    LocalHamiltonian,
    OneSiteTerm,
    PlaquetteTerm,
    VerticalTwoSiteTerm,
    bucket_terms,
    heisenberg,
    transverse_field_ising,
)


def test_bucket_terms_groups_by_kind_and_location():
    """src/vmc/operators/local_terms.py:165-200."""
    H = transverse_field_ising((3, 4))
    diag, one, hor, ver, plaq = bucket_terms(H.terms, (3, 4))
    assert len(diag) == 3 * 3 + 2 * 4
    assert all(len(one[r][c]) == 1 for r in range(3) for c in range(4))
    assert len(hor) == 3 and len(hor[0]) == 3 and len(ver) == 2 and len(plaq) == 2
    with pytest.raises(TypeError):
        bucket_terms((object(),), (2, 2))


def test_lowering_sums_terms_at_a_location():
    ops = (OneSiteTerm(0, 0, np.eye(2)), OneSiteTerm(0, 0, 2 * np.eye(2)),
           HorizontalTwoSiteTerm(1, 0, np.eye(4)), VerticalTwoSiteTerm(0, 1, 3 * np.eye(4)),
           DiagonalTerm(((0, 0), (1, 1)), [1.0, 2.0, 3.0, 4.0]))
    lo = lower_operator(LocalHamiltonian((2, 2), ops), (2, 2), 2)
    assert np.allclose(lo.onesite[0], 3 * np.eye(2)) and lo.onesite_mask.tolist() == [1, 0, 0, 0]
    assert lo.horiz_mask.tolist() == [0, 1] and np.allclose(lo.horiz[1], np.eye(4))
    assert lo.vert_mask.tolist() == [0, 1] and np.allclose(lo.vert[1], 3 * np.eye(4))
    assert lo.diag_sites.tolist() == [0, 3] and lo.diag_values.tolist() == [1.0, 2.0, 3.0, 4.0]
    with pytest.raises(NotImplementedError):
        lower_operator(LocalHamiltonian((2, 2), (PlaquetteTerm(0, 0, 1.0),)), (2, 2), 2)
    with pytest.raises(NotImplementedError):
        lower_operator(LocalHamiltonian((2, 2), (OneSiteTerm(0, 0, 1j * np.eye(2)),)), (2, 2), 2)


def test_pack_order_is_ravel_pytree_order():
    T = uniform_init_tensors((2, 3), 2, seed=0)
    flat = pack_tensors(T)
    assert flat.shape[0] == sum(t.size for row in T for t in row)
    assert np.allclose(flat[:T[0][0].size], T[0][0].reshape(-1))
    assert params_per_site((2, 3), 2) == oracle.params_per_site(oracle.PEPS(T, (2, 3), 2))


def test_heisenberg_bond_operator_is_s_dot_s():
    """S_i.S_j = 1/4 (zz + xx + yy) in the Sz basis."""
    sx = np.array([[0, 1], [1, 0]]) / 2
    sy = np.array([[0, -1j], [1j, 0]]) / 2
    sz = np.diag([1, -1]) / 2
    ss = (np.kron(sx, sx) + np.kron(sy, sy) + np.kron(sz, sz)).real
    # occupancy 0 <-> spin up: the same matrix in this basis ordering
    assert np.allclose(heisenberg((2, 2)).terms[0].op, ss)


def test_product_package_refuses_cpu():
    """No CPU fallback: without a CUDA device the engine raises instead of computing."""
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from vmc_gb300._lib import EngineUnavailable
    from vmc_gb300.engine import PEPSEngine

    with pytest.raises(EngineUnavailable):
        PEPSEngine((2, 2), 2, 4)


# ----------------------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_build_mc_kernels_and_sampler_match_oracle(cuda_device):
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.kernels import build_mc_kernels
    from vmc_gb300.sampling import _sample_counts, _trim_samples, make_mc_sampler

    shape, D, chi = (4, 4), 2, 4
    H = transverse_field_ising(shape)
    T = uniform_init_tensors(shape, D, seed=4)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), tensors=T, device=cuda_device)
    n_samples, n_chains, length, total = _sample_counts(96, 32)
    rng = np.random.default_rng(0)
    cfg0 = rng.integers(0, 2, size=(n_chains, 16)).astype(np.int32)
    u = rng.random((length, n_chains, 16))
    init_cache, transition, estimate = build_mc_kernels(model, H)
    sampler = make_mc_sampler(transition, estimate)
    cache = init_cache(model.tensors, torch.from_numpy(cfg0).to(cuda_device))
    (_, _, _), (hist, est) = sampler(model.tensors, torch.from_numpy(cfg0).to(cuda_device),
                                     torch.from_numpy(u).to(cuda_device), cache, n_steps=length)
    om = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(chi))
    oi, ot, oe = oracle.build_mc_kernels(om, H)
    osampler = oracle.make_mc_sampler(ot, oe)
    (_, _), (ohist, ole, _) = osampler(fp32(T), cfg0.astype(np.int64), u, oi(fp32(T), cfg0.astype(np.int64)),
                                       n_steps=length)
    s = _trim_samples(hist, total, n_samples).cpu().numpy()
    so = oracle.trim_samples(ohist, total, n_samples)
    assert (s == so).all(axis=1).mean() > 0.9
    e = _trim_samples(est.local_estimate, total, n_samples).cpu().numpy()
    eo = oracle.trim_samples(ole.local_estimate, total, n_samples)
    same = (s == so).all(axis=1)
    assert np.median(np.abs(e[same] - eo[same]) / np.maximum(1, np.abs(eo[same]))) < 2e-5


@pytest.mark.gpu
def test_peps_apply_autograd_uses_the_handwritten_adjoint(cuda_device):
    """compat.py:31-64: d amp / d tensors from the engine adjoint == exact gradient (NoTruncation)."""
    from vmc_gb300 import NoTruncation, PEPS
    from vmc_gb300.compat import _value_and_grad, peps_apply

    shape, D = (3, 3), 3
    T = uniform_init_tensors(shape, D, seed=1)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=NoTruncation(), tensors=T, device=cuda_device)
    samples = exact.all_configs(9)[::17]
    packed = model.packed().clone().requires_grad_(True)
    amp = peps_apply(packed, torch.from_numpy(samples).to(cuda_device), shape, model.strategy, model=model)
    w = torch.linspace(-1, 1, amp.shape[0], device=cuda_device, dtype=torch.float64)
    (amp * w).sum().backward()
    om = oracle.PEPS(fp32(T), shape, D, strategy=oracle.NoTruncation())
    a_ref, g_ref, _ = oracle.value_and_grad(om, samples, full_gradient=True)
    assert np.max(np.abs(amp.detach().cpu().numpy() / a_ref - 1)) < 2e-5
    grad_ref = (w.cpu().numpy()[:, None] * g_ref).sum(0)
    assert np.linalg.norm(packed.grad.cpu().numpy() - grad_ref) / np.linalg.norm(grad_ref) < 1e-4
    amp2, grads, p = _value_and_grad(model, torch.from_numpy(samples).to(cuda_device))
    _, g_sl, p_ref = oracle.value_and_grad(om, samples)
    assert np.array_equal(p.cpu().numpy(), p_ref)
    assert np.linalg.norm(grads.cpu().numpy() - g_sl) / np.linalg.norm(g_sl) < 1e-4


@pytest.mark.gpu
def test_local_estimate_and_log_value(cuda_device):
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.compat import _value, local_estimate

    shape, D = (3, 4), 2
    H = heisenberg(shape)
    T = uniform_init_tensors(shape, D, seed=2)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(8), tensors=T, device=cuda_device)
    samples = torch.from_numpy(np.random.default_rng(1).integers(0, 2, (20, 12))).to(cuda_device)
    amps = _value(model, samples)
    e = local_estimate(model, samples, H, amps)
    om = oracle.PEPS(fp32(T), shape, D, strategy=oracle.ZipUp(8))
    a_ref = oracle.value(om, samples.cpu().numpy())
    e_ref = oracle.local_estimate(om, samples.cpu().numpy(), H, a_ref)
    assert np.max(np.abs(amps.cpu().numpy() / a_ref - 1)) < 1e-4
    assert np.median(np.abs(e.cpu().numpy() - e_ref)) < 1e-4
    logpsi = model(samples)
    assert torch.allclose(logpsi.real, torch.log(torch.abs(amps)))


@pytest.mark.gpu
def test_tdvp_driver_imaginary_time_steps(cuda_device):
    """tdvp.py:205-237: chunked runs advance step_count and t; the energy stays finite."""
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.drivers import ImaginaryTimeUnit, RealTimeUnit, TDVPDriver
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import SampleSpace

    shape, D = (3, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4),
                 tensors=uniform_init_tensors(shape, D, seed=3), device=cuda_device)
    drv = TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=ImaginaryTimeUnit(),
                     preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=1e-2), n_samples=64,
                     n_chains=64)
    for _ in range(2):
        drv.run(0.02)
    assert drv.step_count == 4 and abs(drv.t - 0.04) < 1e-12
    assert np.isfinite(drv.energy["mean"])
    with pytest.raises(NotImplementedError):
        TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=RealTimeUnit(),
                   preconditioner=SRPreconditioner())


def _checkpoint_driver(lib, n_chains=8):
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.drivers import ImaginaryTimeUnit, TDVPDriver
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import SampleSpace

    shape, D = (2, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), tensors=uniform_init_tensors(shape, D, seed=3),
                 device="cpu", lib=lib)
    return TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=ImaginaryTimeUnit(),
                      preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=1e-2), n_samples=16,
                      n_chains=n_chains, sampler_key=5)


def test_tdvp_checkpoint_resumes_bit_identically(emu_lib, tmp_path):
    """Driver state (tdvp.py:76-93) saved mid-run and loaded into a fresh driver continues the run
    exactly: same uniforms, same samples, same parameters (engine: host-emulation build)."""
    a = _checkpoint_driver(emu_lib)
    a.run(0.02)
    a.save(tmp_path / "driver.pt")
    a.run(0.02)
    b = _checkpoint_driver(emu_lib)
    b.load(tmp_path / "driver.pt")
    assert b.step_count == 2 and abs(b.t - 0.02) < 1e-15
    b.run(0.02)
    assert a.step_count == b.step_count == 4 and a.t == b.t
    for ra, rb in zip(a._tensors, b._tensors):
        for x, y in zip(ra, rb):
            assert torch.equal(x, y)
    assert a.energy == b.energy
    with pytest.raises(ValueError):
        _checkpoint_driver(emu_lib, n_chains=4).load(tmp_path / "driver.pt")


def test_complex_peps_apply_autograd_and_log_value(emu_lib):
    """Complex PEPS through the public surface (host-emulation engine): amplitudes and log psi, and
    torch's convention for the holomorphic amplitude, grad of Re(sum w psi) = conj(sum w dpsi/dA)."""
    from tests.helpers import complex_tensors
    from vmc_gb300 import NoTruncation, PEPS
    from vmc_gb300.compat import peps_apply

    shape, D = (2, 3), 2
    T = complex_tensors(shape, D, seed=6)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=NoTruncation(), tensors=T, device="cpu",
                 lib=emu_lib, dtype=torch.complex64)
    samples = exact.all_configs(6)[::5]
    packed = model.packed().clone().requires_grad_(True)
    amp = peps_apply(packed, torch.from_numpy(samples), shape, model.strategy, model=model)
    om = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    a_ref, g_ref, _ = oracle.value_and_grad(om, samples, full_gradient=True)
    assert amp.dtype == torch.complex128
    assert np.max(np.abs(amp.detach().numpy() / a_ref - 1)) < 2e-5
    w = torch.linspace(-1, 1, amp.shape[0], dtype=torch.float64)
    (amp * w).real.sum().backward()
    expect = np.conj((w.numpy()[:, None] * g_ref).sum(0))
    assert np.linalg.norm(packed.grad.numpy() - expect) / np.linalg.norm(expect) < 1e-4
    logpsi = model(torch.from_numpy(samples))
    assert torch.allclose(torch.exp(logpsi), amp.detach(), rtol=1e-5)


def test_real_time_tdvp_on_a_complex_peps(emu_lib):
    """tdvp.py with RealTimeUnit (grad factor -i) needs complex parameters: one RK4 step runs on a
    complex PEPS and keeps the parameters complex; a real PEPS is refused."""
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.drivers import RealTimeUnit, TDVPDriver
    from vmc_gb300.preconditioners import SRPreconditioner
    from vmc_gb300.qgt import SampleSpace

    shape, D = (2, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), device="cpu", lib=emu_lib,
                 dtype=torch.complex64, rngs=1)
    drv = TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=RealTimeUnit(),
                     preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=1e-2), n_samples=16,
                     n_chains=8)
    before = [[t.clone() for t in row] for row in drv._tensors]
    drv.run(0.01)
    assert drv.step_count == 1 and drv._tensors[0][0].dtype == torch.complex64
    delta = sum(float((a - b).abs().sum()) for ra, rb in zip(drv._tensors, before) for a, b in zip(ra, rb))
    assert np.isfinite(delta) and delta > 0
    real_model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), device="cpu", lib=emu_lib)
    with pytest.raises(NotImplementedError):
        TDVPDriver(real_model, transverse_field_ising(shape), dt=0.01, time_unit=RealTimeUnit(),
                   preconditioner=SRPreconditioner())
