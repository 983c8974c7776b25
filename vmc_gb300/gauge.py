"""Gauge-removal configuration (src/vmc/gauge/gauge.py:16-37, weight.py:13-26).

The reference does not implement gauge removal: ``compute_gauge_projection``
raises NotImplementedError for every model.  The same contract holds here.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

__all__ = ["GaugeConfig", "compute_gauge_projection", "WeightConfig", "compute_weight_projection"]


@dataclass(frozen=True)
class GaugeConfig:
    """gauge.py:16-21."""

    rcond: float | None = None
    include_global_scale: bool = True


def compute_gauge_projection(cfg, model, params, *, return_info=False):
    """gauge.py:24-37: not implemented in the PEPS runtime (same as the reference)."""
    raise NotImplementedError("Gauge removal is not implemented in the PEPS-only runtime. Use gauge_config=None.")


@dataclass(frozen=True)
class WeightConfig:
    """weight.py:13-16."""


def compute_weight_projection(cfg, samples, sampler=None):
    """weight.py:19-26: all-ones null vector for the sample-space QGT."""
    return torch.ones(samples.shape[0], dtype=torch.complex128, device=samples.device)
