"""build_mc_kernels: init_cache / transition / estimate over a batch of chains
(API of src/vmc/peps/standard/kernels.py:32-247), backed by one fused launch.

The reference's kernels are per-chain functions that ``make_mc_sampler``
vmaps; here they take the whole batch (n_chains, n_sites) at once.  The
engine runs transition and estimate in one kernel: ``transition`` launches
the fused sweep and returns its estimate in the Context; ``estimate`` hands
it back with the next Cache, so the call pattern and pytrees stay the same.

Randomness: ``key`` is either a ``torch.Generator`` on the engine device
(per-site uniforms are drawn from it) or an explicit float64 tensor of
uniforms shaped (n_chains, n_sites) -- the reference's per-site
``uniform(accept_key)`` draws (kernels.py:189-190).
"""
from __future__ import annotations

from typing import Any, NamedTuple

import torch

__all__ = ["Cache", "Context", "LocalEstimates", "build_mc_kernels"]


class Cache(NamedTuple):
    """kernels.py:32-35: per-chain bottom environments (engine-owned bytes)."""
    bottom_envs: Any


class Context(NamedTuple):
    """kernels.py:38-42.  top_envs stay inside the fused launch (None here)."""
    amp: torch.Tensor
    top_envs: Any = None
    estimates: Any = None
    cache_next: Any = None


class LocalEstimates(NamedTuple):
    """kernels.py:45-51 plus log|psi| and sign (amp underflows float64 on big lattices)."""
    local_log_derivatives: torch.Tensor
    local_estimate: torch.Tensor
    active_slice_indices: torch.Tensor | None
    amp: torch.Tensor | None = None
    log_amp: torch.Tensor | None = None
    sign: torch.Tensor | None = None
    margin: torch.Tensor | None = None


def _uniforms(key, n, n_sites, device):
    if isinstance(key, torch.Tensor):
        u = key.to(device=device, dtype=torch.float64).reshape(n, n_sites).contiguous()
        return u, key
    if isinstance(key, torch.Generator):
        return torch.rand((n, n_sites), generator=key, dtype=torch.float64, device=device), key
    raise TypeError("key must be a torch.Generator or a float64 tensor of per-site uniforms")


# Bottom-environment caches larger than this are not kept between sweeps: each sweep recomputes its
# chains' bottom rows in the launch instead (one cache entry per resident CTA), the same results for one
# extra bottom-up pass.  4096 chains of a 16x16 D=6 chi=48 PEPS would hold 58 GB.
DEFAULT_CACHE_BUDGET_BYTES = 16 << 30


def build_mc_kernels(model, operator, *, full_gradient: bool = False, cache_budget_bytes: int | None = None):
    """kernels.py:91-247 for the standard PEPS on the GB300 engine; a GIPEPS model gets the
    gauge-invariant kernels (src/vmc/peps/gi/kernels.py:17-126, dispatched on the model type there).

    ``cache_budget_bytes`` (default ``DEFAULT_CACHE_BUDGET_BYTES``): when the chains' bottom-environment
    cache would exceed it, ``init_cache`` keeps none (``Cache.bottom_envs`` is None) and every sweep
    recomputes the bottom rows inside its launch."""
    from .gi import GIPEPS, build_gi_mc_kernels

    if isinstance(model, GIPEPS):
        return build_gi_mc_kernels(model, operator, full_gradient=full_gradient)
    engine = model.engine(operator)
    n_sites = model.shape[0] * model.shape[1]
    d = model.phys_dim

    budget = DEFAULT_CACHE_BUDGET_BYTES if cache_budget_bytes is None else int(cache_budget_bytes)

    def init_cache(tensors, config_states) -> Cache:
        cfg = config_states.reshape(-1, n_sites).to(device=engine.device, dtype=torch.int32).contiguous()
        if engine.cache_bytes(cfg.shape[0]) > budget:
            return Cache(bottom_envs=None)  # over budget: the sweeps recompute the bottom rows
        return Cache(bottom_envs=engine.init_cache(model.packed(tensors), cfg))

    def transition(tensors, config_state, key, cache: Cache, deltas=None):
        cfg = config_state.reshape(-1, n_sites).to(device=engine.device, dtype=torch.int32).contiguous().clone()
        n = cfg.shape[0]
        u, key_next = _uniforms(key, n, n_sites, engine.device)
        if d > 2 and deltas is None:
            gen = key if isinstance(key, torch.Generator) else None
            deltas = torch.randint(1, d, (n, n_sites), generator=gen, device=engine.device, dtype=torch.int32)
        res = engine.sweep(model.packed(tensors), cfg, u, cache.bottom_envs, deltas=deltas,
                           full_gradient=full_gradient)
        amp = engine.amplitude(res.logamp, res.sign)
        est = LocalEstimates(
            local_log_derivatives=res.O,
            local_estimate=res.E,
            active_slice_indices=None if full_gradient else res.p,
            amp=amp, log_amp=res.logamp, sign=res.sign, margin=res.margin)
        return res.configs, key_next, Context(amp=amp, estimates=est, cache_next=cache)

    def estimate(tensors, config_state_next, context: Context):
        return Cache(bottom_envs=context.cache_next.bottom_envs), context.estimates

    return init_cache, transition, estimate
