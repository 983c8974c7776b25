"""Fault injection on the host: corrupted inputs come back as errors, never as out-of-bounds reads on the
device.  A configuration value outside [0, d) (a gauge link outside [0, N)) is refused by the engine's
entry points before any launch; non-finite site tensors raise VMC_DEV_NONFINITE from the device status
word; flip offsets of d > 2 sweeps follow Python's modulo (the reference's ``(s + delta) % d``,
kernels.py:170-175), so any integer offset is in range.  Host emulation of the kernels, and the refusal
on the GPU (where nothing is launched)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import complex_tensors, hamiltonian, make_case
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors


def _case(dtype, seed=4, n=5):
    shape, D = (3, 3), 2
    if dtype == "complex64":
        T = complex_tensors(shape, D, seed=seed)
        rng = np.random.default_rng(seed)
        cfg = rng.integers(0, 2, (n, 9)).astype(np.int32)
        u = rng.random((n, 9))
    else:
        T, cfg, u = make_case(shape, D, n, seed=seed)
    return shape, D, T, cfg.astype(np.int32), u


def _check_refused(eng, tens, cfg, u, device):
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
    for bad_value in (2, -1):
        bad = cfg.copy()
        bad[1, 4] = bad_value
        c = to(bad)
        with pytest.raises(ValueError, match="must lie in"):
            eng.amp_grad(tens, c)
        with pytest.raises(ValueError, match="must lie in"):
            eng.init_cache(tens, c)
        with pytest.raises(ValueError, match="must lie in"):
            eng.local_energy(tens, c, torch.zeros(len(bad), dtype=torch.float64, device=device),
                             torch.ones(len(bad), dtype=torch.float64, device=device))
        with pytest.raises(ValueError, match="must lie in"):
            eng.vjp(tens, c, torch.ones(len(bad), dtype=torch.float64, device=device))
        with pytest.raises(ValueError, match="must lie in"):
            eng.sweep(tens, c, to(u), eng.new_cache(len(bad)))
        with pytest.raises(ValueError, match="must lie in"):
            eng.amp_grad_job(tens, c)
    assert eng.status() == 0  # nothing was launched
    la, _, _ = eng.amp_grad(tens, to(cfg))  # in-range values still run
    assert bool(torch.isfinite(la).all())


@pytest.mark.parametrize("precision,dtype", [("fp32", "float32"), ("mixed", "float32"), ("fp32", "complex64")])
def test_out_of_range_configurations_are_refused(emu_lib, precision, dtype):
    shape, D, T, cfg, u = _case(dtype)
    eng = PEPSEngine(shape, D, 4, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device="cpu", lib=emu_lib,
                     dtype=dtype, options={"precision": precision})
    _check_refused(eng, torch.from_numpy(pack_tensors(T)), cfg, u, "cpu")


def test_out_of_range_gauge_links_are_refused(emu_lib):
    from oracle import gi as ogi
    from vmc_gb300 import ZipUp
    from vmc_gb300.gi import GIPEPS, GIPEPSConfig, z2_pure_gauge_hamiltonian

    shape = (3, 3)
    ocfg = ogi.GIConfig(shape, 2, 2)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in ogi.init_tensors(ocfg, seed=2)]
    model = GIPEPS(config=GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(2, 2)),
                   contraction_strategy=ZipUp(4), device="cpu", tensors=T, lib=emu_lib)
    eng = model.engine(z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.4))
    samples = ogi.random_physical_configuration(ocfg, 3, seed=5).astype(np.int32)
    bad = samples.copy()
    bad[1, -1] = 2  # a Z2 link value of 2
    with pytest.raises(ValueError, match=r"\[0, 2\)"):
        eng.amp_grad(model.packed(), torch.from_numpy(bad))
    la, _, _ = eng.amp_grad(model.packed(), torch.from_numpy(samples))
    assert bool(torch.isfinite(la).all()) and eng.status() == 0


def test_negative_and_large_flip_offsets_follow_python_modulo(emu_lib):
    shape, D, chi, d = (3, 3), 2, 4, 3
    T, cfg, u = make_case(shape, D, 4, seed=6, phys_dim=d)
    rng = np.random.default_rng(6)
    deltas = rng.integers(1, d, size=cfg.shape).astype(np.int32)
    shifted = deltas + d * rng.integers(-3, 4, size=cfg.shape).astype(np.int32)  # same offsets mod d
    eng = PEPSEngine(shape, D, chi, d, "ZipUp", operator=None, device="cpu", lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    out = []
    for dl in (deltas, shifted):
        c = torch.from_numpy(cfg.copy())
        cache = eng.init_cache(tens, c)
        out.append(eng.sweep(tens, c, torch.from_numpy(u), cache, deltas=torch.from_numpy(dl)))
    assert eng.status() == 0
    assert torch.equal(out[0].configs, out[1].configs) and torch.equal(out[0].O, out[1].O)
    assert torch.equal(out[0].E, out[1].E)


@pytest.mark.parametrize("bad_value", [float("nan"), float("inf")])
def test_non_finite_site_tensors_raise(emu_lib, bad_value):
    shape, D, T, cfg, _ = _case("float32")
    eng = PEPSEngine(shape, D, 4, 2, "ZipUp", operator=hamiltonian("tfim", shape), device="cpu", lib=emu_lib)
    tens = torch.from_numpy(pack_tensors(T))
    tens[3] = bad_value
    la, sg, _ = eng.amp_grad(tens, torch.from_numpy(cfg))
    eng.local_energy(tens, torch.from_numpy(cfg), la, sg)
    with pytest.raises(FloatingPointError):
        eng.raise_on_status()
    assert eng.status() == 0  # raise_on_status read and cleared the word


@pytest.mark.gpu
def test_out_of_range_configurations_are_refused_on_the_gpu(cuda_device):
    shape, D, T, cfg, u = _case("float32")
    eng = PEPSEngine(shape, D, 4, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device=cuda_device)
    _check_refused(eng, torch.from_numpy(pack_tensors(T)).to(cuda_device), cfg, u, cuda_device)


def test_public_api_refuses_out_of_range_configurations(emu_lib):
    """Through the reference-facing calls: peps_apply (the torch.library operator) and init_cache of
    build_mc_kernels."""
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.compat import peps_apply
    from vmc_gb300.kernels import build_mc_kernels

    shape, D, T, cfg, _ = _case("float32")
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), device="cpu", lib=emu_lib, tensors=T)
    bad = torch.from_numpy(cfg.copy())
    bad[0, 0] = 7
    with pytest.raises(ValueError, match="must lie in"):
        peps_apply(model.packed(), bad, shape, None, model=model)
    init_cache, _, _ = build_mc_kernels(model, hamiltonian("tfim", shape))
    with pytest.raises(ValueError, match="must lie in"):
        init_cache(model.tensors, bad)
