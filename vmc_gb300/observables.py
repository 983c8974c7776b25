"""Run logs and host-side observables of lattice-gauge-theory runs (examples/lgt/observables.py).

``SimulationData`` is the JSON log the reference's LGT examples write: the same field names and the same
file layout (one JSON object, the fields as keys), so logs from either implementation read the same way
(examples/lgt/observables.py:25-101).  ``link_diagonal_energy`` evaluates the link-diagonal (electric)
part of a GI Hamiltonian on the device: those terms are diagonal in the sample basis, so a sample's
local value is the sum of its links' diagonal entries and needs no amplitude.  Its mean over samples is
<H_E>, the input of ``compute_energy_derivative``.
"""
from __future__ import annotations

import json
import logging
from dataclasses import asdict, dataclass, field
from pathlib import Path

import numpy as np
import torch

__all__ = ["SimulationData", "compute_energy_derivative", "format_step_log", "link_diagonal_energy"]

logger = logging.getLogger(__name__)


def _plain(x):
    """Nested Python lists/floats of a tensor, array or nested sequence (what json.dump accepts)."""
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    if isinstance(x, np.ndarray):
        return x.tolist()
    if isinstance(x, (list, tuple)):
        return [_plain(v) for v in x]
    if isinstance(x, np.generic):
        return x.item()
    return x


@dataclass
class SimulationData:
    """examples/lgt/observables.py:25-101: metadata plus per-logged-step series."""

    model_type: str = ""
    lattice_size: tuple = (0, 0)
    parameters: dict = field(default_factory=dict)
    steps: list = field(default_factory=list)
    times: list = field(default_factory=list)
    energies: list = field(default_factory=list)
    energy_errors: list = field(default_factory=list)
    energy_variances: list = field(default_factory=list)
    electric_energies: list = field(default_factory=list)
    plaquette_maps: list = field(default_factory=list)
    vbs_dx: list = field(default_factory=list)
    vbs_dy: list = field(default_factory=list)
    wilson_loops: list = field(default_factory=list)

    def add_step(self, step, time, energy, energy_error=0.0, energy_variance=0.0, electric_energy=None):
        self.steps.append(int(step))
        self.times.append(float(time))
        self.energies.append(float(energy))
        self.energy_errors.append(float(energy_error))
        self.energy_variances.append(float(energy_variance))
        if electric_energy is not None:
            self.electric_energies.append(float(electric_energy))

    def add_plaquette_map(self, plaq_map):
        self.plaquette_maps.append(_plain(plaq_map))

    def add_vbs_order(self, dx, dy):
        self.vbs_dx.append(float(dx))
        self.vbs_dy.append(float(dy))

    def add_wilson_loops(self, loops):
        self.wilson_loops.append([(int(a), float(v)) for a, v in loops])

    def save(self, path) -> None:
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        with open(path, "w") as f:
            json.dump({k: _plain(v) for k, v in asdict(self).items()}, f, indent=2)
        logger.info("saved simulation data to %s", path)

    @classmethod
    def load(cls, path) -> "SimulationData":
        with open(path) as f:
            data = json.load(f)
        obj = cls()
        for key, value in data.items():
            setattr(obj, key, value)
        return obj


def compute_energy_derivative(g: float, electric_energy: float) -> float:
    """examples/lgt/observables.py:104-111: dE/dg = <H_E>/g (Hellmann-Feynman for H_E linear in g); 0 at
    |g| < 1e-10."""
    if abs(g) < 1e-10:
        return 0.0
    return electric_energy / g


def format_step_log(step, energy, energy_error, energy_variance, time=None, electric_energy=None, g=None) -> str:
    """examples/lgt/observables.py:114-131: one log line per logged step."""
    parts = [f"Step {step:4d}"]
    if time is not None:
        parts.append(f"t={time:.3f}")
    parts.append(f"E = {energy:.6f} ± {energy_error:.4f} [σ²={energy_variance:.4f}]")
    if electric_energy is not None and g is not None:
        parts.append(f"dE/dg = {compute_energy_derivative(g, electric_energy):.4f}")
    return " | ".join(parts)


def link_diagonal_energy(operator, samples) -> torch.Tensor:
    """Per-sample sum of ``operator``'s link-diagonal terms (gi/local_terms.py:12-39) on GI samples
    (n, R*C + R*(C-1) + (R-1)*C): site values, then horizontal links row-major, then vertical links
    row-major.  Other terms of the operator are skipped.  FP64 on the samples' device."""
    from .gi import LinkDiagonalTerm

    R, C = operator.shape
    s = torch.as_tensor(samples)
    dev = s.device
    s = s.reshape(-1, R * C + R * (C - 1) + (R - 1) * C).long()
    out = torch.zeros(s.shape[0], dtype=torch.float64, device=dev)
    h0, v0 = R * C, R * C + R * (C - 1)
    for t in operator.terms:
        if not isinstance(t, LinkDiagonalTerm):
            continue
        diag = torch.as_tensor(np.asarray(t.diag, dtype=np.float64), device=dev)
        for r, c in t.sites:
            col = h0 + r * (C - 1) + c if t.orientation == "h" else v0 + r * C + c
            out += diag[s[:, col]]
    return out
