"""Gauge-invariant PEPS for pure Z_N lattice gauge theory on the GB300 engine: the reference's
GIPEPS / GIPEPSConfig (src/vmc/peps/gi/model.py:41-189), its local terms (gi/local_terms.py) and its
Monte-Carlo kernels (gi/kernels.py:17-126), for phys_dim = 1 (no matter) and equal degeneracy per
charge -- the pure-gauge Z2 theory of examples/lgt/z2_pure_gauge.py.

A sample is the reference's flattened (sites, h_links, v_links) (model.py:121-144).  The engine runs a
GI plan (``vmc_gi_plan``): the site tensors (1, nc, up, down, left, right) are packed as standard site
tensors whose "physical" index is the gauge configuration (slice) selected by the links, zero-padded to
the largest nc; sampling is the plaquette Metropolis sweep (model.py:629-703), energies are
link-diagonal plus plaquette terms (model.py:392-617).
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

from . import _abi
from .engine import PEPSEngine
from .kernels import Cache, Context, LocalEstimates
from .operators import PlaquetteTerm

__all__ = ["GIPEPSConfig", "GIPEPS", "GIEngine", "GILocalHamiltonian", "LinkDiagonalTerm", "build_electric_terms",
           "build_gi_mc_kernels", "z2_pure_gauge_hamiltonian"]


@dataclass(frozen=True)
class GIPEPSConfig:
    """model.py:41-64.  Supported: phys_dim = 1 (pure gauge), equal degeneracy per charge."""
    shape: tuple
    N: int
    phys_dim: int
    Qx: int
    degeneracy_per_charge: tuple
    charge_of_site: tuple = (0,)
    dtype: Any = torch.float32

    def __post_init__(self):
        if self.phys_dim != 1:
            raise NotImplementedError("the GB300 GI engine covers pure gauge theory (phys_dim = 1)")
        if len(set(self.degeneracy_per_charge)) != 1:
            raise NotImplementedError("uneven degeneracy per charge (masked sectors) is not implemented")
        if self.Qx % self.N != 0:
            raise NotImplementedError("background charge Qx != 0 needs matter")

    @property
    def dmax(self) -> int:
        return int(max(self.degeneracy_per_charge))


@dataclass(frozen=True)
class LinkDiagonalTerm:
    """gi/local_terms.py:12-39: sum over its links of diag[link value]."""
    orientation: str
    sites: tuple
    diag: Any

    def __post_init__(self):
        if self.orientation not in ("h", "v"):
            raise ValueError("orientation must be 'h' or 'v'")


@dataclass(frozen=True)
class GILocalHamiltonian:
    """gi/local_terms.py:63-77."""
    shape: tuple
    terms: tuple = field(default=())


def build_electric_terms(shape, coeff, N):
    """gi/local_terms.py:80-90: coeff (2 - 2 cos(2 pi E / N)) on every link."""
    R, C = shape
    diag = coeff * (2.0 - 2.0 * np.cos(2.0 * np.pi * np.arange(N) / N))
    terms = [LinkDiagonalTerm("h", ((r, c),), diag) for r in range(R) for c in range(C - 1)]
    terms += [LinkDiagonalTerm("v", ((r, c),), diag) for r in range(R - 1) for c in range(C)]
    return tuple(terms)


def z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.33):
    """examples/lgt/z2_pure_gauge.py:42-76: -h (P + P^dag) per plaquette, g (2 - 2 (-1)^E) per link."""
    R, C = shape
    plaq = tuple(PlaquetteTerm(row=r, col=c, coeff=-h) for r in range(R - 1) for c in range(C - 1))
    return GILocalHamiltonian(shape=tuple(shape), terms=build_electric_terms(shape, g, 2) + plaq)


def _n_configs(shape, N, r, c):
    R, C = shape
    links = int(r > 0) + int(r < R - 1) + int(c > 0) + int(c < C - 1)
    return N ** max(links - 1, 0)


def _bond_dims(shape, dmax, r, c):
    R, C = shape
    return (dmax if r > 0 else 1, dmax if r < R - 1 else 1, dmax if c > 0 else 1, dmax if c < C - 1 else 1)


class GIEngine(PEPSEngine):
    """The engine on a GI plan: configs are (n, n_state) flattened samples, uniforms and flip offsets are
    per plaquette, (n, (R-1)(C-1))."""

    def __init__(self, shape, N, dmax, chi, strategy="ZipUp", n_sweeps=2, operator=None, device=None, lib=None,
                 dtype="float32", options=None):
        self.gi_N = int(N)
        slices = max(_n_configs(shape, N, r, c) for r in range(shape[0]) for c in range(shape[1]))
        super().__init__(shape, dmax, chi, slices, strategy, n_sweeps, operator=None, device=device, lib=lib,
                         dtype=dtype, options=options)
        R, C = self.shape
        self.n_state = R * C + R * (C - 1) + (R - 1) * C
        self.n_draws = (R - 1) * (C - 1)
        self.needs_deltas = self.gi_N > 2
        if operator is not None:
            self.set_operator(operator)

    @property
    def state_limit(self) -> int:
        return self.gi_N  # every entry of a sample is a link value (matter entries are 0)

    def _make_plan(self, lib, shape, dt, sid, n_sweeps, options, plan):
        return lib.vmc_gi_plan(ct.byref(shape), self.gi_N, self.bond_dim, self.chi, dt, sid, n_sweeps,
                               ct.byref(options) if options is not None else None, ct.byref(plan))

    def set_operator(self, operator):
        """Link-diagonal and plaquette terms -> vmc_gi_set_operator tables."""
        R, C = self.shape
        N = self.gi_N
        hdiag = np.zeros((R * (C - 1), N))
        vdiag = np.zeros(((R - 1) * C, N))
        plaq = np.zeros((R - 1) * (C - 1))
        for t in operator.terms:
            if isinstance(t, PlaquetteTerm):
                plaq[t.row * (C - 1) + t.col] += float(np.real(t.coeff))
            elif isinstance(t, LinkDiagonalTerm):
                diag = np.asarray(t.diag, dtype=np.float64).reshape(-1)
                if diag.shape[0] != N:
                    raise ValueError("a link-diagonal table needs N values")
                for r, c in t.sites:
                    if t.orientation == "h":
                        hdiag[r * (C - 1) + c] += diag
                    else:
                        vdiag[r * C + c] += diag
            else:
                raise NotImplementedError(f"{type(t).__name__} is not a pure-gauge term")
        st = self.lib.vmc_gi_set_operator(self._plan, hdiag.ctypes.data_as(ct.c_void_p),
                                          vdiag.ctypes.data_as(ct.c_void_p), plaq.ctypes.data_as(ct.c_void_p))
        _abi.check(self.lib, st, "vmc_gi_set_operator")


# The GI chain is a sequence of small GEMMs on 2-row environments, each ending in a CTA barrier: two warps
# per chain and eight resident chains per SM run it faster than four warps and four chains (on GB300, 9x9
# vertices, D=4, chi=32: 8,843 samples/s at 64 threads, 7,618 at 128, 4,511 at 256).
GI_DEFAULT_OPTIONS = {"threads": 64, "smem_kb": -1, "tile_policy": 0}


class GIPEPS:
    """model.py:67-189 (pure gauge).  ``tensors[r][c]``: (1, nc, mu_u, mu_d, mu_l, mu_r) torch tensors."""

    def __init__(self, *, rngs=0, config: GIPEPSConfig, contraction_strategy, device=None, tensors=None, lib=None,
                 engine_options=None):
        """``engine_options``: the GI plan's launch configuration (vmc_plan_options as a dict); None takes
        ``GI_DEFAULT_OPTIONS``."""
        self.config = config
        self.engine_options = dict(GI_DEFAULT_OPTIONS if engine_options is None else engine_options)
        self.shape = tuple(config.shape)
        self.N = int(config.N)
        self.phys_dim = 1
        self.dmax = config.dmax
        self.bond_dim = config.dmax
        self.strategy = contraction_strategy
        self.dtype = torch.complex64 if torch.empty((), dtype=config.dtype).is_complex() else torch.float32
        self.is_complex = self.dtype.is_complex
        self.device = torch.device(device if device is not None else "cuda")
        R, C = self.shape
        if tensors is None:
            # random_tensor (src/vmc/utils/utils.py:20-45): uniform [0, 1), complex 0.5 (U + iU)
            rng = rngs if isinstance(rngs, np.random.Generator) else np.random.default_rng(int(rngs))
            tensors = []
            for r in range(R):
                row = []
                for c in range(C):
                    shp = (1, _n_configs(self.shape, self.N, r, c)) + _bond_dims(self.shape, self.dmax, r, c)
                    row.append(0.5 * (rng.random(shp) + 1j * rng.random(shp)) if self.is_complex else rng.random(shp))
                tensors.append(row)
        self.tensors = [[torch.as_tensor(np.asarray(t)).to(dtype=self.dtype, device=self.device) for t in row]
                        for row in tensors]
        self._slices = max(_n_configs(self.shape, self.N, r, c) for r in range(R) for c in range(C))
        self._engines = {}
        self._lib = lib

    @property
    def n_state(self) -> int:
        R, C = self.shape
        return R * C + R * (C - 1) + (R - 1) * C

    def packed(self, tensors=None) -> torch.Tensor:
        """Engine layout: per site (slices, up, down, left, right), slices past the site's nc zero."""
        tensors = self.tensors if tensors is None else tensors
        parts = []
        for row in tensors:
            for t in row:
                t = torch.as_tensor(t).to(self.dtype)
                pad = torch.zeros((self._slices,) + tuple(t.shape[2:]), dtype=self.dtype, device=t.device)
                pad[:t.shape[1]] = t[0]
                parts.append(pad.reshape(-1))
        return torch.cat(parts).contiguous()

    def sliced_dims(self) -> tuple:
        """Distinct active slices per site, phys_dim * nc (model.py:1066-1080)."""
        return tuple(int(t.shape[1]) for row in self.tensors for t in row)

    @property
    def n_params(self) -> int:
        return sum(t.numel() for row in self.tensors for t in row)

    def unpack(self, flat: torch.Tensor):
        """A flat vector in the reference's parameter order -> per-site (1, nc, ...) tensors."""
        out, off = [], 0
        for row in self.tensors:
            r = []
            for t in row:
                r.append(flat[off:off + t.numel()].reshape(t.shape))
                off += t.numel()
            out.append(r)
        return out

    def full_gradient(self, o_full: torch.Tensor):
        """The engine's full gradient (per site slices x params) in the reference's layout
        (concatenated (1, nc, ...) per site, gi/kernels.py:80-93)."""
        parts, off = [], 0
        for row in self.tensors:
            for t in row:
                nc, sz = t.shape[1], int(np.prod(t.shape[2:]))
                parts.append(o_full[:, off:off + nc * sz])
                off += self._slices * sz
        return torch.cat(parts, dim=1)

    def engine(self, operator=None):
        from .peps import _engine_strategy

        key = id(operator)
        hit = self._engines.get(key)
        if hit is None:
            sname, chi, n_sweeps = _engine_strategy(self.strategy)
            eng = GIEngine(self.shape, self.N, self.dmax, min(chi, 1 << 20), sname, n_sweeps, operator=operator,
                           device=self.device, lib=self._lib, dtype="complex64" if self.is_complex else "float32",
                           options=self.engine_options)
            self._engines[key] = (eng, operator)
            return eng
        return hit[0]

    @staticmethod
    def flatten_sample(sites, h_links, v_links):
        """model.py:121-129."""
        return torch.cat([sites.reshape(-1), h_links.reshape(-1), v_links.reshape(-1)])

    @staticmethod
    def unflatten_sample(sample, shape):
        """model.py:131-144."""
        R, C = shape
        ns, nh = R * C, R * (C - 1)
        return (sample[:ns].reshape(R, C), sample[ns:ns + nh].reshape(R, C - 1), sample[ns + nh:].reshape(R - 1, C))

    def gi_config_states(self, gen: torch.Generator, n: int) -> torch.Tensor:
        """Initial chains for a driver: random plaquette charges from the driver's generator."""
        seed = int(torch.randint(0, 2 ** 31 - 1, (1,), generator=gen, device=gen.device).item())
        return self.random_physical_configuration(seed, n)

    def random_physical_configuration(self, key=0, n_samples=1):
        """model.py:146-189 for pure gauge: random plaquette charges on the zero configuration."""
        rng = key if isinstance(key, np.random.Generator) else np.random.default_rng(int(key))
        R, C = self.shape
        n = int(n_samples)
        h = np.zeros((n, R, C - 1), dtype=np.int64)
        v = np.zeros((n, R - 1, C), dtype=np.int64)
        d = rng.integers(0, self.N, (n, R - 1, C - 1))
        h[:, :R - 1, :] += d
        h[:, 1:, :] -= d
        v[:, :, :C - 1] += d
        v[:, :, 1:] -= d
        out = np.concatenate([np.zeros((n, R * C), dtype=np.int64), (h % self.N).reshape(n, -1),
                              (v % self.N).reshape(n, -1)], axis=1)
        return torch.from_numpy(out.astype(np.int32)).to(self.device)


def build_gi_mc_kernels(model: GIPEPS, operator: GILocalHamiltonian, *, full_gradient: bool = False):
    """gi/kernels.py:17-126 on the engine: batched init_cache / transition / estimate."""
    eng = model.engine(operator)
    n_state, n_plaq = eng.n_state, eng.n_draws

    def init_cache(tensors, config_states) -> Cache:
        cfg = config_states.reshape(-1, n_state).to(device=eng.device, dtype=torch.int32).contiguous()
        return Cache(bottom_envs=eng.init_cache(model.packed(tensors), cfg))

    def transition(tensors, config_state, key, cache: Cache, deltas=None):
        cfg = config_state.reshape(-1, n_state).to(device=eng.device, dtype=torch.int32).contiguous().clone()
        n = cfg.shape[0]
        if isinstance(key, torch.Tensor):
            u = key.to(device=eng.device, dtype=torch.float64).reshape(n, n_plaq).contiguous()
            gen = None
        else:
            gen = key
            u = torch.rand((n, n_plaq), generator=gen, dtype=torch.float64, device=eng.device)
        if eng.needs_deltas and deltas is None:
            deltas = torch.randint(1, model.N, (n, n_plaq), generator=gen, device=eng.device, dtype=torch.int32)
        res = eng.sweep(model.packed(tensors), cfg, u, cache.bottom_envs, deltas=deltas, full_gradient=full_gradient)
        amp = eng.amplitude(res.logamp, res.sign)
        o = model.full_gradient(res.O) if full_gradient else res.O
        est = LocalEstimates(local_log_derivatives=o, local_estimate=res.E,
                             active_slice_indices=None if full_gradient else res.p, amp=amp, log_amp=res.logamp,
                             sign=res.sign, margin=res.margin)
        return res.configs, key, Context(amp=amp, estimates=est, cache_next=cache)

    def estimate(tensors, config_state_next, context: Context):
        return Cache(bottom_envs=context.cache_next.bottom_envs), context.estimates

    return init_cache, transition, estimate
