"""vmc_gb300 -- GB300-native (sm_103a) per-sample PEPS evaluation engine.

Drop-in for the hot path of fliingelephant/VMC: boundary-MPS contraction of a
batch of sampled configurations, sequential row-by-row Metropolis sampling
with environment reuse, O_k = dlog psi/dA, E_loc, and the sliced SR solve.
The compute runs in hand-written CUDA kernels behind the C ABI declared in
include/vmc_gb300.h; this package mirrors the reference's Python surface.
"""
from __future__ import annotations

from .operators import (
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
from .peps import PEPS, ContractionStrategy, DensityMatrix, NoTruncation, Variational, ZipUp

__all__ = [
    "PEPS",
    "ContractionStrategy",
    "NoTruncation",
    "ZipUp",
    "DensityMatrix",
    "Variational",
    "LocalHamiltonian",
    "OneSiteTerm",
    "DiagonalTerm",
    "HorizontalTwoSiteTerm",
    "VerticalTwoSiteTerm",
    "PlaquetteTerm",
    "bucket_terms",
    "heisenberg",
    "transverse_field_ising",
    "build_mc_kernels",
    "make_mc_sampler",
    "GraphTDVPDriver",
]


def __getattr__(name):
    if name == "build_mc_kernels":
        from .kernels import build_mc_kernels

        return build_mc_kernels
    if name == "make_mc_sampler":
        from .sampling import make_mc_sampler

        return make_mc_sampler
    if name == "GraphTDVPDriver":
        from .tdvp_graph import GraphTDVPDriver

        return GraphTDVPDriver
    raise AttributeError(name)
