"""A TDVP step -- sampling, SR solve and parameter update -- as ONE CUDA graph
(tdvp.py:113-237, integrators.py:45-109).

``GraphTDVPDriver`` keeps every quantity of a step in device buffers at fixed
addresses: the packed parameters, the chains' configurations and bottom cache,
the uniforms, the sweep outputs and the integrator stages.  One step is:

    for each derivative call of the integrator (4 for RK4, 1 for Euler):
        uniforms <- vmc_uniforms(seed, device counter)
        init_cache; n_steps fused sweeps (vmc_peps_sweep)
        SR solve in FP64 (DirectSolve, Cholesky without a host check), reorder, 2 Re
    parameters <- the integrator's combination of the stages

The first step runs eagerly (it also warms cuBLAS/cuSOLVER and the allocator);
it is then captured once and every later step is a single graph replay with no
host round trip.  Uniforms come from a counter in device memory, so a replayed
step draws exactly what the eager step with the same counter draws, and the
two give the same bits.
"""
from __future__ import annotations

import ctypes as ct

import torch

from . import _abi
from .drivers import EnergyStats, Euler, RealTimeUnit, RK4, TimeUnit
from .engine import SweepResult
from .lowering import params_per_site
from .preconditioners import DirectSolve, SRPreconditioner, _direct_solve, reorder_updates
from .qgt import Jacobian, SlicedJacobian, solve_cholesky
from .sampling import _sample_counts

__all__ = ["GraphTDVPDriver"]


class GraphTDVPDriver:
    """TDVPDriver's run / energy / checkpoint surface with every step replayed from one CUDA graph.

    Supported: Euler or RK4, SRPreconditioner with DirectSolve(solve_cholesky) in either space, no
    gauge projection -- the configurations whose step reads nothing from the host.  The sampler
    key seeds the device uniform stream (vmc_uniforms) instead of a torch.Generator."""

    def __init__(self, model, operator, *, preconditioner: SRPreconditioner, dt: float, t0: float = 0.0,
                 time_unit: TimeUnit = RealTimeUnit(), integrator=None, sampler_key=0, n_samples: int = 1,
                 n_chains: int = 1, full_gradient: bool = False, use_graph: bool = True):
        if isinstance(time_unit.grad_factor, complex) and not getattr(model, "is_complex", False):
            raise NotImplementedError("real-time TDVP needs complex parameters: use a complex PEPS")
        strat = preconditioner.strategy
        if not isinstance(strat, DirectSolve) or strat.solver is not solve_cholesky:
            raise NotImplementedError("a graph step needs DirectSolve(solve_cholesky): the QR solve's rank "
                                      "and the SVD/CG solvers read the host")
        if preconditioner.gauge_config is not None:
            raise NotImplementedError("gauge projection is not part of a graph step")
        if model.phys_dim > 2:
            raise NotImplementedError("graph steps draw accept uniforms only; d > 2 also needs flip offsets")
        if hasattr(model, "sliced_dims"):
            raise NotImplementedError("graph steps run standard PEPS; a gauge-invariant PEPS runs in TDVPDriver")
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
        if not isinstance(self.integrator, (Euler, RK4)):
            raise NotImplementedError("graph steps exist for Euler and RK4")
        self.use_graph = bool(use_graph)
        self.seed = int(sampler_key) & ((1 << 64) - 1)
        eng = model.engine(operator)
        self._eng = eng
        dev = eng.device
        self._dev = dev
        _, _, self._chain_length, self._total = _sample_counts(self.n_samples, self.n_chains)
        n_sites = model.shape[0] * model.shape[1]
        self._n_sites = n_sites
        gen = torch.Generator(device=dev)
        gen.manual_seed(self.seed)
        self._configs = torch.randint(0, model.phys_dim, (self.n_chains, n_sites), generator=gen, device=dev,
                                      dtype=torch.int32)
        self._counter = torch.zeros(1, dtype=torch.int64, device=dev)
        self._theta = model.packed().clone()
        self._stage = torch.empty_like(self._theta)
        self._k = [torch.empty_like(self._theta) for _ in range(4 if isinstance(self.integrator, RK4) else 1)]
        self._cache = eng.new_cache(self.n_chains)
        L, n = self._chain_length, self.n_chains
        self._u = torch.empty((L, n, n_sites), dtype=torch.float64, device=dev)
        np_ = eng.n_params_full if self.full_gradient else eng.n_params_sliced
        self._O = torch.empty((L, n, np_), dtype=eng.param_dtype, device=dev)
        self._p = None if self.full_gradient else torch.empty((L, n, eng.n_params_sliced), dtype=torch.int8,
                                                              device=dev)
        self._E = torch.empty((L, n), dtype=eng.energy_dtype, device=dev)
        self._la = torch.empty((L, n), dtype=torch.float64, device=dev)
        self._sg = torch.empty((L, n), dtype=torch.float64, device=dev)
        self._outs = [SweepResult(configs=self._configs, O=self._O[s], p=None if self._p is None else self._p[s],
                                  E=self._E[s], logamp=self._la[s], sign=self._sg[s], margin=None, gap=None)
                      for s in range(L)]
        self._pps = tuple(params_per_site(model.shape, model.bond_dim))
        self._sd = (model.phys_dim,) * n_sites
        self._residual = torch.zeros((), dtype=torch.float64, device=dev)
        self._graph = None
        self._loss_stats = None

    # ------------------------------------------------------------------ one derivative call
    def _derivative(self, theta, k_out):
        """tdvp.py:113-163 on device buffers: k_out <- the SR update at parameters theta."""
        eng = self._eng
        u = self._u
        st = eng.lib.vmc_uniforms(eng._stream(), ct.c_void_p(u.data_ptr()), u.numel(), self.seed,
                                  ct.c_void_p(self._counter.data_ptr()))
        _abi.check(eng.lib, st, "vmc_uniforms")
        eng.init_cache(theta, self._configs, cache=self._cache)
        for s in range(self._chain_length):
            eng.sweep(theta, self._configs, u[s], self._cache, full_gradient=self.full_gradient,
                      out=self._outs[s])
        N = self.n_samples
        o = self._O.reshape(self._total, -1)[:N]
        p = None if self._p is None else self._p.reshape(self._total, -1)[:N]
        e = self._E.reshape(-1)[:N]
        # SRPreconditioner.apply (preconditioners.py:265-330) without host reads
        e = e.to(torch.complex128 if e.is_complex() else torch.float64)
        dv = (e - e.mean()) / N
        gf = self.time_unit.grad_factor
        complex_factor = isinstance(gf, complex) and gf.imag != 0
        dv = dv.to(torch.complex128) * gf if complex_factor else dv * float(getattr(gf, "real", gf))
        pre = self.preconditioner
        jac = Jacobian(o) if p is None else SlicedJacobian(o, p, self._sd, pre.ordering)
        x, metrics = _direct_solve(pre.space, jac, dv, pre.diag_shift, pre.strategy.solver)
        if p is not None:
            x = reorder_updates(pre.ordering, x, self._pps, self._sd)
        if not complex_factor and not self._theta.is_complex():
            x = 2.0 * x.real
        k_out.copy_(x.to(k_out.dtype))
        self._residual.copy_(metrics["residual_error"])

    def _step(self):
        """integrators.py:45-109 on flat parameter vectors."""
        th, dt, k = self._theta, self.dt, self._k
        if isinstance(self.integrator, Euler):
            self._derivative(th, k[0])
            th.add_(k[0], alpha=dt)
            return
        self._derivative(th, k[0])
        torch.add(th, k[0], alpha=0.5 * dt, out=self._stage)
        self._derivative(self._stage, k[1])
        torch.add(th, k[1], alpha=0.5 * dt, out=self._stage)
        self._derivative(self._stage, k[2])
        torch.add(th, k[2], alpha=dt, out=self._stage)
        self._derivative(self._stage, k[3])
        k[1].mul_(2.0).add_(k[2], alpha=2.0).add_(k[0]).add_(k[3])
        th.add_(k[1], alpha=dt / 6.0)

    def step(self):
        """One integrator step: eager the first time, then a replay of the captured graph."""
        if not self.use_graph or self._dev.type != "cuda":
            self._step()
        elif self._graph is None:
            self._step()
            torch.cuda.synchronize(self._dev)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._step()
            self._graph = g
        else:
            self._graph.replay()
        self.t += self.dt
        self.step_count += 1

    def run(self, T: float) -> None:
        """tdvp.py:205-237."""
        duration = float(T)
        assert duration > 0.0, f"T must be positive, got {duration}"
        n_steps = int(round(duration / self.dt))
        eps = 1e-12 * max(1.0, abs(duration), abs(self.dt))
        assert abs(duration - n_steps * self.dt) <= eps, f"T={duration} must be an integer multiple of dt={self.dt}"
        assert n_steps > 0
        if self._dev.type == "cuda":
            with torch.cuda.device(self._dev):
                for _ in range(n_steps):
                    self.step()
        else:  # the host-emulation build of the kernels (CPU tests): eager steps only
            for _ in range(n_steps):
                self.step()
        self._eng.raise_on_status()
        self._model.tensors = self._model.unpack(self._theta.clone())
        e = self._E.reshape(-1)[:self.n_samples]
        self._loss_stats = EnergyStats.of(e)

    # ------------------------------------------------------------------ state
    @property
    def residual_error(self):
        return float(self._residual.item())

    @property
    def energy(self):
        return self._loss_stats

    @property
    def model(self):
        return self._model

    @property
    def parameters(self) -> torch.Tensor:
        """The packed parameter vector (device buffer; a view, not a copy)."""
        return self._theta

    def state_dict(self) -> dict:
        return {
            "format": "vmc_gb300.GraphTDVPDriver/1",
            "t": self.t, "dt": self.dt, "step_count": self.step_count, "seed": self.seed,
            "n_samples": self.n_samples, "n_chains": self.n_chains, "full_gradient": self.full_gradient,
            "theta": self._theta.detach().cpu().clone(),
            "sampler_configuration": self._configs.detach().cpu().clone(),
            "counter": int(self._counter.item()),
            "loss_stats": None if self._loss_stats is None else dict(self._loss_stats),
        }

    def load_state_dict(self, state: dict) -> None:
        """Copies into the existing device buffers, so a captured graph stays valid."""
        if state.get("format") != "vmc_gb300.GraphTDVPDriver/1":
            raise ValueError("not a GraphTDVPDriver checkpoint")
        for key in ("n_samples", "n_chains", "full_gradient", "seed"):
            if state[key] != getattr(self, key):
                raise ValueError(f"checkpoint {key}={state[key]} does not match this driver ({getattr(self, key)})")
        if tuple(state["theta"].shape) != tuple(self._theta.shape):
            raise ValueError("checkpoint parameters do not match the model")
        self.t = float(state["t"])
        self.dt = float(state["dt"])
        self.step_count = int(state["step_count"])
        self._theta.copy_(state["theta"].to(self._dev))
        self._configs.copy_(state["sampler_configuration"].to(self._dev))
        self._counter.fill_(int(state["counter"]))
        self._loss_stats = None if state["loss_stats"] is None else EnergyStats(state["loss_stats"])
        self._model.tensors = self._model.unpack(self._theta.clone())

    def save(self, path) -> None:
        torch.save(self.state_dict(), path)

    def load(self, path) -> None:
        self.load_state_dict(torch.load(path, map_location="cpu", weights_only=True))
