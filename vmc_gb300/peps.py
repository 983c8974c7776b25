"""PEPS model container and contraction strategies (API of src/vmc/peps/standard/model.py
and src/vmc/peps/common/strategy.py), backed by the sm_103a engine.

Tensors live on a CUDA device as float32; the packed parameter vector used by
the engine is site-major with each site (d, up, down, left, right) C-order --
the order of the reference's ``ravel_pytree(model.tensors)``.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .lowering import site_dims as _site_dims

__all__ = ["ContractionStrategy", "NoTruncation", "ZipUp", "DensityMatrix", "Variational", "PEPS"]


class ContractionStrategy:
    """strategy.py:25-41."""

    name = "ContractionStrategy"

    def __init__(self, truncate_bond_dimension: int):
        self.truncate_bond_dimension = int(truncate_bond_dimension)

    def __repr__(self):
        return f"{type(self).__name__}({self.truncate_bond_dimension})"


class NoTruncation(ContractionStrategy):
    """strategy.py:44-51: exact boundary application (bonds multiply)."""

    name = "NoTruncation"

    def __init__(self):
        super().__init__(1)


class ZipUp(ContractionStrategy):
    """strategy.py:54-61: on-the-fly SVD truncation to chi."""

    name = "ZipUp"


class DensityMatrix(ContractionStrategy):
    """strategy.py:64-71.  Keeps the top eigenvectors V_k of theta^H theta and
    carries V_k^H (without the singular values) to the next site, so its
    truncations differ from ZipUp's.  The engine does not implement it (the
    plan returns VMC_ERR_UNSUPPORTED)."""

    name = "DensityMatrix"


class Variational(ContractionStrategy):
    """strategy.py:74-92: QR-initialised variational compression with n_sweeps."""

    name = "Variational"

    def __init__(self, truncate_bond_dimension: int, n_sweeps: int = 2):
        super().__init__(truncate_bond_dimension)
        self.n_sweeps = int(n_sweeps)


def _engine_strategy(strategy):
    if isinstance(strategy, Variational):
        return "Variational", strategy.truncate_bond_dimension, strategy.n_sweeps
    if isinstance(strategy, NoTruncation):
        return "NoTruncation", 1 << 20, 2
    return strategy.name, strategy.truncate_bond_dimension, 2


class PEPS:
    """Open-boundary PEPS on a rectangular lattice (model.py:22-98).

    ``rngs`` seeds the reference's initialiser (uniform [0, 1) entries, or
    0.5 (U + iU) for a complex dtype, src/vmc/utils/utils.py:22-47) when
    ``tensors`` is not given.  Real dtypes run the float32 engine, complex
    dtypes the complex64 engine.  ``lib``
    selects an engine library other than the in-tree CUDA build (a ctypes
    handle bound by ``vmc_gb300._abi.bind``); by default the CUDA build is
    required.  ``engine_options``: the plan's launch configuration (a
    vmc_plan_options dict, or "auto" for the autotuner's winner on this GPU);
    None takes the engine's default.
    """

    def __init__(self, *, rngs=0, shape, bond_dim, phys_dim=2, contraction_strategy=None,
                 dtype=torch.float32, device=None, tensors=None, lib=None, engine_options=None):
        self.engine_options = engine_options if engine_options in (None, "auto") else dict(engine_options)
        self.shape = (int(shape[0]), int(shape[1]))
        self.bond_dim = int(bond_dim)
        self.phys_dim = int(phys_dim)
        if dtype in (torch.float32, torch.float64):
            self.dtype = torch.float32
        elif dtype in (torch.complex64, torch.complex128):
            self.dtype = torch.complex64
        else:
            raise NotImplementedError(f"unsupported PEPS dtype {dtype}")
        self.is_complex = self.dtype.is_complex
        if contraction_strategy is None:
            contraction_strategy = Variational(self.bond_dim * self.bond_dim)
        self.strategy = contraction_strategy
        self.device = torch.device(device if device is not None else "cuda")
        n_rows, n_cols = self.shape
        if tensors is None:
            rng = rngs if isinstance(rngs, np.random.Generator) else np.random.default_rng(int(rngs))
            def init(shape):
                if self.is_complex:
                    return 0.5 * (rng.random(shape) + 1j * rng.random(shape))
                return rng.random(shape)

            tensors = [[init((self.phys_dim,) + self.site_dims(r, c, n_rows, n_cols, self.bond_dim))
                        for c in range(n_cols)] for r in range(n_rows)]
        self.tensors = [[torch.as_tensor(np.asarray(t)).to(dtype=self.dtype, device=self.device)
                         for t in row] for row in tensors]
        for r in range(n_rows):
            for c in range(n_cols):
                want = (self.phys_dim,) + self.site_dims(r, c, n_rows, n_cols, self.bond_dim)
                if tuple(self.tensors[r][c].shape) != want:
                    raise ValueError(f"tensor ({r},{c}) has shape {tuple(self.tensors[r][c].shape)}, want {want}")
        self._engines = {}
        self._lib = lib

    site_dims = staticmethod(_site_dims)

    @property
    def n_params(self) -> int:
        return sum(t.numel() for row in self.tensors for t in row)

    def packed(self, tensors=None) -> torch.Tensor:
        tensors = self.tensors if tensors is None else tensors
        if isinstance(tensors, torch.Tensor):
            return tensors.to(self.dtype).contiguous()
        return torch.cat([t.reshape(-1).to(self.dtype) for row in tensors for t in row]).contiguous()

    def unpack(self, flat: torch.Tensor):
        out, off = [], 0
        for row in self.tensors:
            r = []
            for t in row:
                n = t.numel()
                r.append(flat[off:off + n].reshape(t.shape))
                off += n
            out.append(r)
        return out

    def engine(self, operator=None):
        """The engine plan for this model (and operator, if given); cached."""
        from .engine import PEPSEngine

        key = id(operator)
        eng = self._engines.get(key)
        if eng is None:
            sname, chi, n_sweeps = _engine_strategy(self.strategy)
            eng = PEPSEngine(self.shape, self.bond_dim, min(chi, 1 << 20), self.phys_dim, sname, n_sweeps,
                             operator=operator, device=self.device, lib=self._lib,
                             dtype="complex64" if self.is_complex else "float32", options=self.engine_options)
            self._engines[key] = (eng, operator)
            return eng
        return eng[0]

    @staticmethod
    def apply(tensors, sample, shape, strategy):
        from .compat import peps_apply

        return peps_apply(tensors, sample, shape, strategy)

    @staticmethod
    def unflatten_sample(sample, shape):
        return sample.reshape(shape)

    def __call__(self, x):
        """log psi for a batch of samples (complex: log|psi| + i arg psi), as model.py:82-87."""
        from .compat import log_value

        la, sign = log_value(self, x)
        if self.is_complex:
            return torch.complex(la, sign)
        return torch.complex(la, torch.where(sign < 0, torch.full_like(la, math.pi), torch.zeros_like(la)))

    def random_physical_configuration(self, key=0, n_samples=1):
        """model.py:89-98: uniform occupancies, shape (n_samples, n_rows, n_cols), int32."""
        if isinstance(key, torch.Generator):
            return torch.randint(0, self.phys_dim, (n_samples,) + self.shape, generator=key,
                                 device=key.device, dtype=torch.int32)
        rng = np.random.default_rng(int(key))
        cfg = rng.integers(0, self.phys_dim, size=(n_samples,) + self.shape).astype(np.int32)
        return torch.from_numpy(cfg).to(self.device)
