"""make_mc_sampler (src/vmc/core/sampling.py:22-82) for batched engine kernels."""
from __future__ import annotations

import math

import torch

from .kernels import LocalEstimates

__all__ = ["make_mc_sampler", "_sample_counts", "_trim_samples"]


def make_mc_sampler(transition, estimate):
    """Returns mc_sampler(tensors, config_states, chain_keys, cache, *, n_steps).

    ``chain_keys`` is a torch.Generator (or a float64 tensor of uniforms of
    shape (n_steps, n_chains, n_sites)).  The result mirrors the reference's
    ``lax.scan`` output: ((configs, keys, cache), (config_hist, estimates))
    with a leading n_steps axis on the history.
    """

    def mc_sampler(tensors, config_states, chain_keys, cache, *, n_steps: int):
        configs = config_states
        hist_cfg, hist = [], []
        for step in range(n_steps):
            key = chain_keys[step] if isinstance(chain_keys, torch.Tensor) else chain_keys
            configs, key_next, ctx = transition(tensors, configs, key, cache)
            cache, est = estimate(tensors, configs, ctx)
            hist_cfg.append(configs.clone() if n_steps > 1 else configs)
            hist.append(est)
        stacked = LocalEstimates(*[
            None if getattr(hist[0], f) is None else torch.stack([getattr(e, f) for e in hist])
            for f in LocalEstimates._fields])
        keys_out = chain_keys
        return (configs, keys_out, cache), (torch.stack(hist_cfg), stacked)

    return mc_sampler


def _sample_counts(n_samples: int, n_chains: int):
    chain_length = math.ceil(n_samples / n_chains)
    return n_samples, n_chains, chain_length, chain_length * n_chains


def _trim_samples(samples, total_samples: int, num_samples: int):
    return samples.reshape((total_samples,) + tuple(samples.shape[2:]))[:num_samples]
