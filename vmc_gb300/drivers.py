"""TDVP / VMC driver with Euler and RK4 integrators
(API of src/vmc/drivers/tdvp.py:54-249 and integrators.py:45-144).

State is the list-of-lists of site tensors; the derivative is the SR update
computed from one engine sampling run (init_cache + n_steps fused sweeps).
Real-time evolution (grad factor -i) needs complex parameters: it runs on a
complex PEPS and raises NotImplementedError for a real one.

With ``process_group`` (one process per GPU, e.g. ``torch.distributed.group.WORLD``)
the chains are sharded contiguously across the group's ranks (``shard_chains``):
each rank sweeps its shard, drawing the same uniform stream as one process would
and keeping its rows; the step's histories are all-gathered along the chain axis,
and every rank runs the same SR solve on the single-process arrays, so the
parameters stay identical on all ranks and equal to a one-process run's.
"""
from __future__ import annotations

import logging
import math

import torch

from . import distributed as _dist
from .kernels import build_mc_kernels
from .preconditioners import SRPreconditioner
from .sampling import _sample_counts, _trim_samples, make_mc_sampler

logger = logging.getLogger(__name__)

__all__ = ["TDVPDriver", "Integrator", "Euler", "RK4", "TimeUnit", "RealTimeUnit", "ImaginaryTimeUnit", "EnergyStats"]


def _add_scaled(base, delta, scale):
    """src/vmc/utils/utils.py:60-65."""
    return [[b + scale * d for b, d in zip(rb, rd)] for rb, rd in zip(base, delta)]


class EnergyStats(dict):
    """Statistics of the last step's local energies (tdvp.py:226, netket.stats.statistics): ``mean``,
    ``variance`` and ``error_of_mean``, read as attributes (``driver.energy.mean.real``, as the
    reference's examples do) or as keys."""

    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError:
            raise AttributeError(name) from None

    @classmethod
    def of(cls, e: torch.Tensor) -> "EnergyStats":
        mean = e.mean()
        var = float((e - mean).abs().pow(2).mean())
        return cls(mean=mean.item(), variance=var, error_of_mean=math.sqrt(var / e.numel()))


class Integrator:
    """integrators.py:21-42."""

    @staticmethod
    def step(derivative_fn, state, t, dt, carry):  # pragma: no cover - abstract
        raise NotImplementedError


class Euler(Integrator):
    """integrators.py:45-63."""

    @staticmethod
    def step(derivative_fn, state, t, dt, carry):
        k, carry_next, aux = derivative_fn(state, t, carry)
        return _add_scaled(state, k, dt), t + dt, carry_next, aux


class RK4(Integrator):
    """integrators.py:66-109."""

    @staticmethod
    def step(derivative_fn, state, t, dt, carry):
        k1, c1, _ = derivative_fn(state, t, carry)
        k2, c2, _ = derivative_fn(_add_scaled(state, k1, 0.5 * dt), t + 0.5 * dt, c1)
        k3, c3, _ = derivative_fn(_add_scaled(state, k2, 0.5 * dt), t + 0.5 * dt, c2)
        k4, c4, aux = derivative_fn(_add_scaled(state, k3, dt), t + dt, c3)
        incr = [[(a + 2.0 * b + 2.0 * c + d) / 6.0 for a, b, c, d in zip(ra, rb, rc, rd)]
                for ra, rb, rc, rd in zip(k1, k2, k3, k4)]
        return _add_scaled(state, incr, dt), t + dt, c4, aux


class TimeUnit:
    """integrators.py:112-122."""

    grad_factor = 1.0

    def default_integrator(self):  # pragma: no cover - abstract
        raise NotImplementedError


class RealTimeUnit(TimeUnit):
    """integrators.py:125-133: i d/dt psi = H psi."""

    grad_factor = -1.0j

    def default_integrator(self):
        return RK4()


class ImaginaryTimeUnit(TimeUnit):
    """integrators.py:136-144: d/dt psi = -H psi."""

    grad_factor = -1.0

    def default_integrator(self):
        return Euler()


class TDVPDriver:
    """tdvp.py:54-249 on the GB300 engine."""

    def __init__(self, model, operator, *, preconditioner: SRPreconditioner, dt: float, t0: float = 0.0,
                 time_unit: TimeUnit = RealTimeUnit(), integrator: Integrator | None = None, sampler_key=0,
                 n_samples: int = 1, n_chains: int = 1, full_gradient: bool = False, process_group=None):
        if isinstance(time_unit.grad_factor, complex) and not getattr(model, "is_complex", False):
            raise NotImplementedError("real-time TDVP needs complex parameters: use a complex PEPS")
        self._group = process_group
        self._rank, self._world = _dist.group_rank_size(process_group) if process_group is not None else (0, 1)
        if self._world > 1 and hasattr(model, "gi_config_states"):
            raise NotImplementedError("chain sharding runs standard PEPS; a gauge-invariant PEPS runs on one rank")
        self._model = model
        self.operator = operator
        self.preconditioner = preconditioner
        self.dt = float(dt)
        self.t = float(t0)
        self.step_count = 0
        self.n_samples = int(n_samples)
        self.n_chains = int(n_chains)
        self.full_gradient = bool(full_gradient)
        self.time_unit = time_unit
        self.integrator = integrator or time_unit.default_integrator()
        dev = model.device
        self._gen = torch.Generator(device=dev)
        self._gen.manual_seed(int(sampler_key))
        self._tensors = [[t.clone() for t in row] for row in model.tensors]
        if hasattr(model, "gi_config_states"):  # a gauge-invariant PEPS: Gauss-law configurations
            self._sampler_configuration = model.gi_config_states(self._gen, self.n_chains)
        else:
            self._sampler_configuration = torch.randint(0, model.phys_dim, (self.n_chains,) + model.shape,
                                                        generator=self._gen, device=dev, dtype=torch.int32)
        # this rank's chains [start, start + count); the whole range on one process
        self._shard = _dist.shard_chains(self.n_chains, self._world, self._rank)
        if self._world > 1:
            start, count = self._shard
            self._sampler_configuration = self._sampler_configuration[start:start + count].clone()
        init_cache, transition, estimate = build_mc_kernels(model, operator, full_gradient=self.full_gradient)
        self._init_cache = init_cache
        self._transition, self._estimate = transition, estimate
        self._mc_sampler = make_mc_sampler(transition, estimate)
        self.residual_error = None
        self.diag_shift_error = None
        self.solve_time = None
        self._loss_stats = None

    def _sharded_sampling(self, tensors, configs, gen, chain_length):
        """This rank's sweeps over its chain shard with the uniforms (and flip offsets) one process
        would draw for those chains; the histories gathered over the group along the chain axis."""
        start, count = self._shard
        n_sites = configs.shape[-1]
        dev = self._model.device
        d = self._model.phys_dim
        cache = self._init_cache(tensors, configs)
        hist_cfg, ests = [], []
        for _ in range(chain_length):
            # the draws of kernels.transition with a generator key, for all chains; this rank's rows kept
            u = torch.rand((self.n_chains, n_sites), generator=gen, dtype=torch.float64, device=dev)
            deltas = None
            if d > 2:
                deltas = torch.randint(1, d, (self.n_chains, n_sites), generator=gen, device=dev,
                                       dtype=torch.int32)[start:start + count].contiguous()
            configs, _, ctx = self._transition(tensors, configs, u[start:start + count].contiguous(), cache,
                                               deltas=deltas)
            cache, est = self._estimate(tensors, configs, ctx)
            hist_cfg.append(configs.clone())
            ests.append(est)

        def gathered(field):
            if getattr(ests[0], field) is None:
                return None
            return _dist.gather_chain_axis(torch.stack([getattr(e, field) for e in ests]), self.n_chains,
                                           self._group)

        hist = _dist.gather_chain_axis(torch.stack(hist_cfg), self.n_chains, self._group)
        return configs, hist, gathered("local_log_derivatives"), gathered("local_estimate"), \
            gathered("active_slice_indices")

    def _time_derivative(self, tensors, t, carry):
        """tdvp.py:113-163."""
        gen, configs = carry
        _, num_chains, chain_length, total = _sample_counts(self.n_samples, self.n_chains)
        if self._world > 1:
            configs, hist, o_h, e_h, p_h = self._sharded_sampling(tensors, configs, gen, chain_length)
            samples = _trim_samples(hist, total, self.n_samples)
            o = _trim_samples(o_h, total, self.n_samples)
            e = _trim_samples(e_h, total, self.n_samples)
            p = None if self.full_gradient else _trim_samples(p_h, total, self.n_samples)
            self._model.tensors = tensors
            updates, metrics = self.preconditioner.apply(self._model, tensors, samples, o, p, e,
                                                         grad_factor=self.time_unit.grad_factor)
            return updates, (gen, configs), (e, metrics)
        cache = self._init_cache(tensors, configs)
        (configs, _, _), (hist, est) = self._mc_sampler(tensors, configs.reshape(num_chains, -1), gen, cache,
                                                          n_steps=chain_length)
        samples = _trim_samples(hist, total, self.n_samples)
        o = _trim_samples(est.local_log_derivatives, total, self.n_samples)
        e = _trim_samples(est.local_estimate, total, self.n_samples)
        p = None if self.full_gradient else _trim_samples(est.active_slice_indices, total, self.n_samples)
        self._model.tensors = tensors
        updates, metrics = self.preconditioner.apply(self._model, tensors, samples, o, p, e,
                                                     grad_factor=self.time_unit.grad_factor)
        return updates, (gen, configs), (e, metrics)

    def run(self, T: float) -> None:
        """tdvp.py:205-237."""
        duration = float(T)
        assert duration > 0.0, f"T must be positive, got {duration}"
        n_steps = int(round(duration / self.dt))
        eps = 1e-12 * max(1.0, abs(duration), abs(self.dt))
        assert abs(duration - n_steps * self.dt) <= eps, f"T={duration} must be an integer multiple of dt={self.dt}"
        assert n_steps > 0
        carry = (self._gen, self._sampler_configuration.reshape(self._shard[1], -1))
        e = None
        metrics = {}
        for _ in range(n_steps):
            self._tensors, self.t, carry, (e, metrics) = self.integrator.step(
                self._time_derivative, self._tensors, self.t, self.dt, carry)
            logger.debug("E_mean=%s", e.mean().item())
        self._sampler_configuration = carry[1]
        self._model.tensors = self._tensors
        self.step_count += n_steps
        self._loss_stats = EnergyStats.of(e)
        self.residual_error = metrics.get("residual_error")

    # ------------------------------------------------------------ checkpoint
    def state_dict(self) -> dict:
        """Everything a run carries between ``run`` calls (the attributes tdvp.py:76-93 sets up):
        parameters, time, step count, sampler configurations and the sampler's RNG state, so a
        resumed run draws the same uniforms and reaches bit-identical parameters."""
        return {
            "format": "vmc_gb300.TDVPDriver/1",
            "t": self.t,
            "dt": self.dt,
            "step_count": self.step_count,
            "n_samples": self.n_samples,
            "n_chains": self.n_chains,
            "full_gradient": self.full_gradient,
            "tensors": [[t.detach().to("cpu").clone() for t in row] for row in self._tensors],
            "sampler_configuration": self._sampler_configuration.detach().to("cpu").clone(),
            "generator_state": self._gen.get_state(),
            "loss_stats": None if self._loss_stats is None else dict(self._loss_stats),
        }

    def load_state_dict(self, state: dict) -> None:
        if state.get("format") != "vmc_gb300.TDVPDriver/1":
            raise ValueError("not a TDVPDriver checkpoint")
        for key in ("n_samples", "n_chains", "full_gradient"):
            if state[key] != getattr(self, key):
                raise ValueError(f"checkpoint {key}={state[key]} does not match this driver ({getattr(self, key)})")
        shapes = [[tuple(t.shape) for t in row] for row in self._tensors]
        if [[tuple(t.shape) for t in row] for row in state["tensors"]] != shapes:
            raise ValueError("checkpoint tensors do not match the model's shapes")
        dev = self._model.device
        self.t = float(state["t"])
        self.dt = float(state["dt"])
        self.step_count = int(state["step_count"])
        self._tensors = [[t.to(dev, self._model.dtype).clone() for t in row] for row in state["tensors"]]
        self._model.tensors = self._tensors
        self._sampler_configuration = state["sampler_configuration"].to(dev, torch.int32).clone()
        self._gen.set_state(state["generator_state"])
        self._loss_stats = None if state["loss_stats"] is None else EnergyStats(state["loss_stats"])

    def save(self, path) -> None:
        torch.save(self.state_dict(), path)

    def load(self, path) -> None:
        self.load_state_dict(torch.load(path, map_location="cpu", weights_only=True))

    @property
    def energy(self):
        return self._loss_stats

    @property
    def model(self):
        return self._model
