"""The LGT run log (JSON round trip, field names of examples/lgt/observables.py) and the link-diagonal
(electric) energy, checked against the engine's local energy of an electric-only Hamiltonian in the
host-emulation build."""
from __future__ import annotations

import json

import numpy as np
import torch

from oracle import gi as ogi
from vmc_gb300 import ZipUp
from vmc_gb300.gi import GIPEPS, GIPEPSConfig, GILocalHamiltonian, build_electric_terms, z2_pure_gauge_hamiltonian
from vmc_gb300.observables import (SimulationData, compute_energy_derivative, format_step_log,
                                   link_diagonal_energy)

FIELDS = {"model_type", "lattice_size", "parameters", "steps", "times", "energies", "energy_errors",
          "energy_variances", "electric_energies", "plaquette_maps", "vbs_dx", "vbs_dy", "wilson_loops"}


def test_simulation_data_round_trip(tmp_path):
    d = SimulationData(model_type="Z2_pure_gauge", lattice_size=(4, 4), parameters={"g": 0.4, "h": 1.0})
    d.add_step(5, 0.05, -3.25, 0.01, 0.2, electric_energy=1.5)
    d.add_step(10, 0.10, -3.5, 0.02, 0.1)
    d.add_plaquette_map(torch.arange(9, dtype=torch.float64).reshape(3, 3))
    d.add_vbs_order(np.float32(0.25), 0.5)
    d.add_wilson_loops([(1, 0.9), (4, 0.5)])
    path = tmp_path / "run" / "z2.json"
    d.save(path)
    raw = json.loads(path.read_text())
    assert set(raw) == FIELDS
    assert raw["lattice_size"] == [4, 4] and raw["plaquette_maps"][0][2] == [6.0, 7.0, 8.0]
    e = SimulationData.load(path)
    assert e.steps == [5, 10] and e.energies == [-3.25, -3.5] and e.electric_energies == [1.5]
    assert e.wilson_loops == [[[1, 0.9], [4, 0.5]]] and e.vbs_dx == [0.25]


def test_energy_derivative_and_log_line():
    assert compute_energy_derivative(0.5, 2.0) == 4.0
    assert compute_energy_derivative(0.0, 2.0) == 0.0
    line = format_step_log(15, -1.25, 0.01, 0.5, time=0.15, electric_energy=2.0, g=0.5)
    assert line.startswith("Step   15 | t=0.150 | E = -1.250000") and line.endswith("dE/dg = 4.0000")


def test_link_diagonal_energy_matches_the_engine(emu_lib):
    shape, dmax = (3, 4), 2
    ocfg = ogi.GIConfig(shape, 2, dmax)
    T = [[t.astype(np.float32).astype(np.float64) for t in row] for row in ogi.init_tensors(ocfg, seed=5)]
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax))
    model = GIPEPS(config=cfg, contraction_strategy=ZipUp(4), device="cpu", tensors=T, lib=emu_lib)
    samples = torch.from_numpy(ogi.random_physical_configuration(ocfg, 8, seed=6).astype(np.int32))
    # non-uniform couplings, so a wrong link index changes the sum
    terms = tuple(type(t)(t.orientation, t.sites, np.asarray(t.diag) * (1 + 0.1 * i))
                  for i, t in enumerate(build_electric_terms(shape, 0.7, 2)))
    H_E = GILocalHamiltonian(shape=shape, terms=terms)
    eng = model.engine(H_E)
    tens = model.packed()
    la, sg, _ = eng.amp_grad(tens, samples, want_O=False)
    E = eng.local_energy(tens, samples, la, sg)
    ours = link_diagonal_energy(H_E, samples)
    assert torch.allclose(ours, E.double(), rtol=1e-6, atol=1e-6)
    # plaquette terms are skipped
    full = z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.7)
    assert torch.allclose(link_diagonal_energy(full, samples),
                          link_diagonal_energy(GILocalHamiltonian(shape, build_electric_terms(shape, 0.7, 2)), samples))
