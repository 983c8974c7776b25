"""Seeded synthetic PEPS workloads (no public dataset exists for this path).

Tensors are i.i.d. N(0,1)/sqrt(d * D^4) drawn from NumPy ``PCG64(seed)``;
initial configurations are uniform in {0..d-1} from ``PCG64(seed + 2)``;
per-site Metropolis uniforms for sweep k come from ``PCG64(seed + 1)``
(one (n_chains, n_sites) block per sweep, in sweep order).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .lowering import site_dims
from .operators import heisenberg, transverse_field_ising

__all__ = ["Workload", "random_tensors", "initial_configs", "uniform_stream", "WORKLOADS"]


def random_tensors(shape, bond_dim, phys_dim=2, seed=0, dtype=np.float64):
    """Entries i.i.d. N(0,1)/sqrt(d D^4); for a complex dtype the real and
    imaginary parts are each i.i.d. N(0,1)/sqrt(2 d D^4)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_rows, n_cols = shape
    cplx = np.issubdtype(np.dtype(dtype), np.complexfloating)
    scale = 1.0 / np.sqrt((2 if cplx else 1) * phys_dim * bond_dim ** 4)
    out = []
    for r in range(n_rows):
        row = []
        for c in range(n_cols):
            dims = (phys_dim,) + site_dims(r, c, n_rows, n_cols, bond_dim)
            t = rng.standard_normal(dims) * scale
            if cplx:
                t = t + 1j * rng.standard_normal(dims) * scale
            row.append(t.astype(dtype))
        out.append(row)
    return out


def initial_configs(n_chains, n_sites, phys_dim=2, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed + 2))
    return rng.integers(0, phys_dim, size=(n_chains, n_sites)).astype(np.int32)


def uniform_stream(n_chains, n_sites, seed=0):
    """Generator of (n_chains, n_sites) float64 uniform blocks, one per sweep."""
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    while True:
        yield rng.random((n_chains, n_sites))


@dataclass(frozen=True)
class Workload:
    name: str
    shape: tuple
    bond_dim: int
    chi: int
    phys_dim: int
    model: str       # "heisenberg" | "tfim"
    n_chains: int
    strategy: str = "ZipUp"
    dtype: str = "float32"   # "float32" | "complex64"

    def operator(self):
        if self.model == "heisenberg":
            return heisenberg(self.shape)
        return transverse_field_ising(self.shape, J=1.0, h=3.0)

    def flops_per_sample(self):
        """Algorithmic real FLOP per sample counted with the reference's einsum orders (SVD/QR excluded;
        oracle/flop_count.py recounts them).  A complex multiply-add is 4 real ones."""
        f = _ALGO_FLOPS.get((self.shape, self.bond_dim, self.chi, self.model, self.strategy))
        return None if f is None else f * (4 if self.dtype == "complex64" else 1)

    def tensors(self, seed=0):
        return random_tensors(self.shape, self.bond_dim, self.phys_dim, seed=seed,
                              dtype=np.complex128 if self.dtype == "complex64" else np.float64)


_ALGO_FLOPS = {
    ((8, 8), 4, 16, "heisenberg", "ZipUp"): 234.9e6,
    ((8, 8), 4, 16, "heisenberg", "Variational"): 370.9e6,
    ((8, 8), 4, 16, "tfim", "ZipUp"): 69.0e6,
    ((10, 10), 4, 16, "tfim", "ZipUp"): 137.0e6,
    ((6, 6), 4, 16, "heisenberg", "ZipUp"): 71.2e6,
    ((8, 8), 5, 25, "heisenberg", "ZipUp"): 1.54e9,
    ((12, 12), 6, 36, "heisenberg", "ZipUp"): 27.1e9,
    ((16, 16), 6, 48, "heisenberg", "ZipUp"): 112.5e9,
}

WORKLOADS = {
    # 4x4 TFIM, J=1 h=3, D=2, ZipUp(4), 256 samples (the CPU-runnable exact case)
    "tfim4x4_D2_chi4": Workload("tfim4x4_D2_chi4", (4, 4), 2, 4, 2, "tfim", 256),
    # 8x8 Heisenberg, D=4, chi=16, 4096 samples per sweep (headline)
    "heis8x8_D4_chi16": Workload("heis8x8_D4_chi16", (8, 8), 4, 16, 2, "heisenberg", 4096),
    # the same lattice with the variational compression, Variational(16) with 2 sweeps
    "heis8x8_D4_chi16_var": Workload("heis8x8_D4_chi16_var", (8, 8), 4, 16, 2, "heisenberg", 4096, "Variational"),
    # the uneven-batch shapes, 4096 samples each (run one shape per launch)
    "heis6x6_D4_chi16": Workload("heis6x6_D4_chi16", (6, 6), 4, 16, 2, "heisenberg", 4096),
    "heis8x8_D5_chi25": Workload("heis8x8_D5_chi25", (8, 8), 5, 25, 2, "heisenberg", 4096),
    "heis12x12_D6_chi36": Workload("heis12x12_D6_chi36", (12, 12), 6, 36, 2, "heisenberg", 4096),
    "heis16x16_D6_chi48": Workload("heis16x16_D6_chi48", (16, 16), 6, 48, 2, "heisenberg", 4096),
    # 10x10 TFIM (J=1, h=3), complex64 PEPS, D=4, chi=16, 8192 samples per step
    "tfim10x10_D4_chi16_c64": Workload("tfim10x10_D4_chi16_c64", (10, 10), 4, 16, 2, "tfim", 8192, "ZipUp",
                                       "complex64"),
}
