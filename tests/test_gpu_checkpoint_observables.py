"""Checkpoint/resume and the LGT run log on the GPU: a TDVPDriver and a GraphTDVPDriver saved mid-run
and loaded into fresh drivers continue bit for bit; the electric (link-diagonal) energy of sampled
Z2 gauge configurations equals the engine's local energy of the electric-only Hamiltonian, and the
run's SimulationData JSON round-trips."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import gi as ogi
from tests.helpers import uniform_init_tensors
from vmc_gb300 import PEPS, ZipUp
from vmc_gb300.drivers import ImaginaryTimeUnit, TDVPDriver
from vmc_gb300.gi import GIPEPS, GIPEPSConfig, GILocalHamiltonian, build_electric_terms, z2_pure_gauge_hamiltonian
from vmc_gb300.observables import SimulationData, format_step_log, link_diagonal_energy
from vmc_gb300.operators import transverse_field_ising
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import SampleSpace
from vmc_gb300.tdvp_graph import GraphTDVPDriver

pytestmark = pytest.mark.gpu


def _driver(cls, device, **kw):
    shape, D = (3, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), tensors=uniform_init_tensors(shape, D, seed=3),
                 device=device)
    return cls(model, transverse_field_ising(shape), dt=0.01, time_unit=ImaginaryTimeUnit(),
               preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=1e-2), n_samples=256, n_chains=128,
               sampler_key=5, **kw)


@pytest.mark.parametrize("cls", [TDVPDriver, GraphTDVPDriver], ids=["eager", "graph"])
def test_checkpoint_resumes_bit_identically(cuda_device, tmp_path, cls):
    a = _driver(cls, cuda_device)
    a.run(0.02)
    a.save(tmp_path / "driver.pt")
    a.run(0.02)
    b = _driver(cls, cuda_device)
    b.load(tmp_path / "driver.pt")
    assert b.step_count == 2
    b.run(0.02)
    assert a.step_count == b.step_count == 4 and a.t == b.t
    pa, pb = a.model.packed(), b.model.packed()
    assert torch.equal(pa, pb)
    assert a.energy["mean"] == b.energy["mean"]


def test_lgt_run_log_on_the_gpu(cuda_device, tmp_path):
    shape, dmax, g = (3, 3), 2, 0.4
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax))
    model = GIPEPS(rngs=1, config=cfg, contraction_strategy=ZipUp(4), device=cuda_device)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0, g=g)
    drv = TDVPDriver(model, H, preconditioner=SRPreconditioner(space=SampleSpace(), diag_shift=0.1), dt=0.05,
                     time_unit=ImaginaryTimeUnit(), n_samples=256, n_chains=128, full_gradient=True)
    data = SimulationData(model_type="Z2_pure_gauge", lattice_size=shape, parameters={"g": g, "h": 1.0})
    for step in range(2):
        drv.run(0.05)
        samples = drv._sampler_configuration.reshape(drv.n_chains, -1)
        H_E = GILocalHamiltonian(shape=shape, terms=build_electric_terms(shape, g, 2))
        eng = model.engine(H_E)
        tens = model.packed()
        la, sg, _ = eng.amp_grad(tens, samples, want_O=False)
        e_engine = eng.local_energy(tens, samples, la, sg).double()
        e_link = link_diagonal_energy(H_E, samples)
        assert torch.allclose(e_link, e_engine, rtol=1e-6, atol=1e-6)
        e = drv.energy
        data.add_step(drv.step_count, drv.t, float(e["mean"]), float(e["error_of_mean"]), float(e["variance"]),
                      electric_energy=float(e_link.mean()))
        line = format_step_log(drv.step_count, float(e["mean"]), float(e["error_of_mean"]), float(e["variance"]),
                               time=drv.t, electric_energy=float(e_link.mean()), g=g)
        assert line.startswith(f"Step {drv.step_count:4d}")
    path = tmp_path / "z2.json"
    data.save(path)
    back = SimulationData.load(path)
    assert back.steps == [1, 2] and np.allclose(back.energies, data.energies)
    assert np.all(np.isfinite(back.electric_energies))
