"""Python handle on the C-ABI engine: plan, workspace, cache and calls.

``PEPSEngine`` owns one ``vmc_plan`` and a device workspace; every call is
issued on torch's current CUDA stream and takes/returns torch tensors that
live on that device.  Nothing here computes on the CPU: if the CUDA library
or the GPU is missing, construction raises ``EngineUnavailable``.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np
import torch

from . import _abi
from ._lib import EngineUnavailable
from .lowering import lower_operator

__all__ = ["BatchJob", "PEPSBatch", "PEPSEngine", "SweepResult", "STRATEGY_IDS"]

STRATEGY_IDS = {
    "NoTruncation": _abi.VMC_STRATEGY_NO_TRUNCATION,
    "ZipUp": _abi.VMC_STRATEGY_ZIP_UP,
    "DensityMatrix": _abi.VMC_STRATEGY_DENSITY_MATRIX,
    "Variational": _abi.VMC_STRATEGY_VARIATIONAL,
}


def _vp(t):
    if t is None:
        return None
    return ct.c_void_p(t.data_ptr())


def _np_vp(a):
    return a.ctypes.data_as(ct.c_void_p) if a is not None else None


@dataclass
class SweepResult:
    configs: torch.Tensor        # (n, n_sites) int32, updated in place
    O: torch.Tensor | None       # (n, n_params) float32
    p: torch.Tensor | None       # (n, n_params_sliced) int8
    E: torch.Tensor | None       # (n,) float64, complex128 for a complex engine
    logamp: torch.Tensor | None  # (n,) float64 log|psi|
    sign: torch.Tensor | None    # (n,) float64 sign of psi, or its phase in radians for a complex engine
    margin: torch.Tensor | None  # (n,) float32
    gap: torch.Tensor | None = None  # (n,) float32 smallest relative eigen-gap at a cut


class PEPSEngine:
    """Plan + workspace for one (shape, D, chi, d, strategy, operator)."""

    def __init__(self, shape, bond_dim, chi, phys_dim=2, strategy="ZipUp", n_sweeps=2, operator=None,
                 device=None, lib=None, dtype="float32", options=None, precision=None):
        """``options``: the plan's launch configuration -- None (defaults), a dict with keys threads /
        smem_kb / tile_policy / precision / trunc_method / vchunk / vert_smem (vmc_plan_options), or
        "auto" for the autotuned choice of this (lattice, D, chi, dtype, strategy, precision) from
        vmc_gb300.autotune.  ``precision``: "fp32" (default) or "mixed" -- the boundary-MPS chain in
        double-float (FP64 eigenvalues), everything else FP32 (overrides the options' precision)."""
        self.shape = (int(shape[0]), int(shape[1]))
        self.complex = str(dtype).replace("torch.", "") in ("complex64", "complex128")
        # dtypes of this engine's parameters / O_k and of E_loc
        self.param_dtype = torch.complex64 if self.complex else torch.float32
        self.energy_dtype = torch.complex128 if self.complex else torch.float64
        self.bond_dim, self.chi, self.phys_dim = int(bond_dim), int(chi), int(phys_dim)
        self.strategy = strategy
        self.n_sites = self.shape[0] * self.shape[1]
        if lib is None:
            if not torch.cuda.is_available():
                raise EngineUnavailable("vmc_gb300 needs a CUDA GPU; no CPU fallback exists")
            from ._lib import lib as _load
            lib = _load()
            self.device = torch.device(device if device is not None else "cuda")
            if self.device.type != "cuda":
                raise EngineUnavailable("vmc_gb300 engine tensors must live on a CUDA device")
            if self.device.index is None:  # tensors report their index: compare like with like
                self.device = torch.device("cuda", torch.cuda.current_device())
        else:
            self.device = torch.device(device if device is not None else "cpu")
        self.lib = lib
        plan = ct.c_void_p()
        sid = STRATEGY_IDS[strategy] if isinstance(strategy, str) else int(strategy)
        if isinstance(options, str):
            if options != "auto":
                raise ValueError("options must be None, a dict or 'auto'")
        if isinstance(options, str):
            from .autotune import tuned_options

            prec = "mixed" if precision in ("mixed", _abi.VMC_PRECISION_MIXED) else "fp32"
            options = tuned_options(self.shape, self.bond_dim, self.chi, self.phys_dim, strategy, n_sweeps,
                                    "complex64" if self.complex else "float32", operator=operator,
                                    device=self.device, lib=lib, precision=prec)
        if precision is not None:
            options = dict(options or {})
            options["precision"] = precision
        self.options = None if options is None else dict(options)
        dt = _abi.VMC_DTYPE_C64 if self.complex else _abi.VMC_DTYPE_F32
        o = None if options is None else _abi.plan_options(options)
        with torch.cuda.device(self.device) if self.device.type == "cuda" else _null():
            st = self._make_plan(lib, _abi.VmcShape(*self.shape), dt, sid, int(n_sweeps), o, plan)
        _abi.check(lib, st, "vmc_peps_plan")
        self.resident_chains = int(lib.vmc_plan_resident_ctas(plan))
        self._plan = plan
        # ints of state per chain, accept draws per chain (and flip offsets, if needed) per sweep
        self.n_state = self.n_sites
        self.n_draws = self.n_sites
        self.needs_deltas = self.phys_dim > 2
        self.n_params_sliced = int(lib.vmc_peps_n_params_sliced(plan))
        self.n_params_full = int(lib.vmc_peps_n_params_full(plan))
        self._ws = None
        self._ws_n = -1
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        if operator is not None:
            self.set_operator(operator)

    def _make_plan(self, lib, shape, dt, sid, n_sweeps, options, plan):
        if options is None:
            return lib.vmc_peps_plan(ct.byref(shape), self.bond_dim, self.chi, self.phys_dim, dt, sid, n_sweeps,
                                     ct.byref(plan))
        return lib.vmc_peps_plan_ex(ct.byref(shape), self.bond_dim, self.chi, self.phys_dim, dt, sid, n_sweeps,
                                    ct.byref(options), ct.byref(plan))

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                self.lib.vmc_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    # ------------------------------------------------------------------ setup
    def set_operator(self, operator):
        lo = lower_operator(operator, self.shape, self.phys_dim, complex_elements=self.complex)
        onesite, horiz, vert = (np.ascontiguousarray(a) for a in (lo.onesite, lo.horiz, lo.vert))
        st = self.lib.vmc_peps_plan_set_operator(
            self._plan, _np_vp(onesite), _np_vp(lo.onesite_mask), _np_vp(horiz), _np_vp(lo.horiz_mask),
            _np_vp(vert), _np_vp(lo.vert_mask), lo.n_diag,
            _np_vp(lo.diag_nsites) if lo.n_diag else None, _np_vp(lo.diag_site_off) if lo.n_diag else None,
            _np_vp(lo.diag_sites) if lo.n_diag else None, _np_vp(lo.diag_value_off) if lo.n_diag else None,
            _np_vp(lo.diag_values) if lo.n_diag else None)
        _abi.check(self.lib, st, "vmc_peps_plan_set_operator")

    def cache_bytes(self, n):
        return int(self.lib.vmc_cache_size(self._plan, int(n)))

    def workspace(self, n, recompute=False):
        size = self.lib.vmc_sweep_recompute_workspace_size if recompute else self.lib.vmc_workspace_size
        need = int(size(self._plan, int(n)))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._ws

    def new_cache(self, n):
        return torch.empty(self.cache_bytes(n), dtype=torch.uint8, device=self.device)

    def _stream(self):
        if self.device.type == "cuda":
            return ct.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        return None

    def _check_tensors(self, tensors):
        if tensors.dtype != self.param_dtype or tensors.device != self.device or not tensors.is_contiguous():
            raise ValueError(f"packed tensors must be a contiguous {self.param_dtype} vector on the engine device")
        if tensors.numel() != self.n_params_full:
            raise ValueError(f"expected {self.n_params_full} packed parameters, got {tensors.numel()}")

    # configuration values lie in [0, state_limit): spins below phys_dim (gauge links below N on a GI plan)
    @property
    def state_limit(self) -> int:
        return self.phys_dim

    def _configs(self, configs):
        c = configs.reshape(-1, self.n_state)
        if c.dtype != torch.int32 or c.device != self.device or not c.is_contiguous():
            raise ValueError("configs must be a contiguous int32 (n, n_state) tensor on the engine device")
        self._check_range(c)
        return c

    def _check_range(self, c):
        """The kernels index the site tensors with the configuration values unchecked, so a value outside
        [0, state_limit) is refused here, before any launch: one min/max reduction and a host read.  Skipped
        inside a CUDA-graph capture, whose configurations are the engine's own sweep outputs."""
        if c.numel() == 0 or (c.device.type == "cuda" and torch.cuda.is_current_stream_capturing()):
            return
        lo, hi = torch.stack([c.min(), c.max()]).tolist()
        if lo < 0 or hi >= self.state_limit:
            raise ValueError(f"configuration values must lie in [0, {self.state_limit}); got [{lo}, {hi}]")

    def status(self, reset=True) -> int:
        v = int(self._status.item())
        if reset and v:
            self._status.zero_()
        return v

    def raise_on_status(self):
        v = self.status()
        if v & _abi.VMC_DEV_NONFINITE:
            raise FloatingPointError("engine reported a non-finite amplitude or energy")
        if v & _abi.VMC_DEV_TIMEOUT:
            raise TimeoutError("engine reported a device-side timeout")

    def amplitude(self, logamp, sign):
        """psi from (log|psi|, sign) -- or (log|psi|, phase) for a complex engine."""
        if self.complex:
            return torch.exp(torch.complex(logamp, sign))
        return sign * torch.exp(logamp)

    def log_sign(self, amps):
        """(log|psi|, sign or phase) of given amplitudes, the inverse of ``amplitude``."""
        a = torch.as_tensor(amps, device=self.device)
        if self.complex:
            a = a.to(torch.complex128)
            return torch.log(torch.abs(a)), torch.angle(a)
        a = a.to(torch.float64)
        return torch.log(torch.abs(a)), torch.sign(a)

    # ------------------------------------------------------------------ calls
    def init_cache(self, tensors, configs, cache=None):
        self._check_tensors(tensors)
        c = self._configs(configs)
        n = c.shape[0]
        if cache is None:
            cache = self.new_cache(n)
        ws = self.workspace(n)
        st = self.lib.vmc_peps_init_cache(self._plan, self._stream(), _vp(tensors), _vp(c), n, _vp(cache),
                                          _vp(ws), ws.numel(), _vp(self._status))
        _abi.check(self.lib, st, "vmc_peps_init_cache")
        return cache

    def _sweep_io(self, tensors, configs, uniforms, deltas, full_gradient, want_O, want_p, want_margin, out):
        self._check_tensors(tensors)
        c = self._configs(configs)
        n = c.shape[0]
        u = uniforms.reshape(n, self.n_draws)
        if u.dtype != torch.float64 or u.device != self.device or not u.is_contiguous():
            raise ValueError("uniforms must be a contiguous float64 (n, n_draws) tensor on the engine device")
        if self.needs_deltas:
            if deltas is None:
                raise ValueError("this plan needs explicit flip offsets (deltas)")
            deltas = deltas.reshape(n, self.n_draws).to(torch.int32).contiguous()
        else:
            deltas = None
        np_ = self.n_params_full if full_gradient else self.n_params_sliced
        dev = self.device
        if out is None:
            out = SweepResult(
                configs=c,
                O=torch.empty((n, np_), dtype=self.param_dtype, device=dev) if want_O else None,
                p=torch.empty((n, self.n_params_sliced), dtype=torch.int8, device=dev) if want_p else None,
                E=torch.empty(n, dtype=self.energy_dtype, device=dev),
                logamp=torch.empty(n, dtype=torch.float64, device=dev),
                sign=torch.empty(n, dtype=torch.float64, device=dev),
                margin=torch.empty(n, dtype=torch.float32, device=dev) if want_margin else None,
                gap=torch.empty(n, dtype=torch.float32, device=dev) if want_margin else None,
            )
        return c, u, deltas, out

    def sweep(self, tensors, configs, uniforms, cache=None, deltas=None, full_gradient=False, want_O=True,
              want_p=True, want_margin=True, out=None):
        """One sweep of every chain.  ``cache``: the bottom-environment cache from ``init_cache`` (read and
        rewritten); None recomputes the environments inside the launch instead (the same results as
        init_cache + sweep, memory per resident CTA rather than per chain)."""
        c, u, deltas, out = self._sweep_io(tensors, configs, uniforms, deltas, full_gradient, want_O, want_p,
                                           want_margin, out)
        n = c.shape[0]
        if cache is None:
            # no per-chain cache: the bottom environments are recomputed inside the launch
            ws = self.workspace(n, recompute=True)
            st = self.lib.vmc_peps_sweep_recompute(
                self._plan, self._stream(), _vp(tensors), _vp(c), _vp(u), _vp(deltas), n, int(bool(full_gradient)),
                _vp(out.O), _vp(out.p), _vp(out.E), _vp(out.logamp), _vp(out.sign), _vp(out.margin), _vp(out.gap),
                _vp(ws), ws.numel(), _vp(self._status))
            _abi.check(self.lib, st, "vmc_peps_sweep_recompute")
            return out
        ws = self.workspace(n)
        st = self.lib.vmc_peps_sweep(self._plan, self._stream(), _vp(tensors), _vp(c), _vp(u), _vp(deltas), n,
                                     _vp(cache), int(bool(full_gradient)), _vp(out.O), _vp(out.p), _vp(out.E),
                                     _vp(out.logamp), _vp(out.sign), _vp(out.margin), _vp(out.gap), _vp(ws),
                                     ws.numel(), _vp(self._status))
        _abi.check(self.lib, st, "vmc_peps_sweep")
        return out

    def amp_grad(self, tensors, samples, full_gradient=False, want_O=True, want_gap=False):
        self._check_tensors(tensors)
        c = self._configs(samples)
        n = c.shape[0]
        dev = self.device
        np_ = self.n_params_full if full_gradient else self.n_params_sliced
        O = torch.empty((n, np_), dtype=self.param_dtype, device=dev) if want_O else None
        logamp = torch.empty(n, dtype=torch.float64, device=dev)
        sign = torch.empty(n, dtype=torch.float64, device=dev)
        gap = torch.empty(n, dtype=torch.float32, device=dev) if want_gap else None
        ws = self.workspace(n)
        st = self.lib.vmc_peps_amp_grad(self._plan, self._stream(), _vp(tensors), _vp(c), n,
                                        int(bool(full_gradient)), _vp(O), _vp(logamp), _vp(sign), _vp(gap),
                                        _vp(ws), ws.numel(), _vp(self._status))
        _abi.check(self.lib, st, "vmc_peps_amp_grad")
        if want_gap:
            return logamp, sign, O, gap
        return logamp, sign, O

    def vjp(self, tensors, samples, weights):
        """sum_i w_i O_i over the full parameter layout (``vmc_peps_vjp``), FP64 (complex128 for a complex
        engine): the adjoint of the amplitudes without an (n, n_params) O matrix."""
        self._check_tensors(tensors)
        c = self._configs(samples)
        n = c.shape[0]
        w = weights.to(torch.complex128 if self.complex else torch.float64).contiguous()
        if self.complex:
            w = torch.view_as_real(w).contiguous()
        grad = torch.empty(self.n_params_full * (2 if self.complex else 1), dtype=torch.float64, device=self.device)
        ws = self.workspace(n)
        st = self.lib.vmc_peps_vjp(self._plan, self._stream(), _vp(tensors), _vp(c), n, _vp(w), _vp(grad), _vp(ws),
                                   ws.numel(), _vp(self._status))
        _abi.check(self.lib, st, "vmc_peps_vjp")
        return torch.view_as_complex(grad.view(-1, 2)) if self.complex else grad

    def local_energy(self, tensors, samples, logamp, sign):
        self._check_tensors(tensors)
        c = self._configs(samples)
        n = c.shape[0]
        E = torch.empty(n, dtype=self.energy_dtype, device=self.device)
        ws = self.workspace(n)
        la = logamp.to(torch.float64).contiguous()
        sg = sign.to(torch.float64).contiguous()
        st = self.lib.vmc_peps_local_energy(self._plan, self._stream(), _vp(tensors), _vp(c), n, _vp(la),
                                            _vp(sg), _vp(E), _vp(ws), ws.numel(), _vp(self._status))
        _abi.check(self.lib, st, "vmc_peps_local_energy")
        return E


    # ------------------------------------------------------- batch jobs
    # The same calls as jobs of an uneven batch (PEPSBatch.run): arguments are
    # checked and outputs allocated here, and the launch happens in the batch.
    def init_cache_job(self, tensors, configs, cache=None):
        self._check_tensors(tensors)
        c = self._configs(configs)
        cache = self.new_cache(c.shape[0]) if cache is None else cache
        out = SweepResult(configs=c, O=None, p=None, E=None, logamp=None, sign=None, margin=None)
        return BatchJob(self, _abi.VMC_JOB_INIT_CACHE, tensors, out, cache=cache)

    def sweep_job(self, tensors, configs, uniforms, cache=None, deltas=None, full_gradient=False, want_O=True,
                  want_p=True, want_margin=True, out=None):
        c, u, deltas, out = self._sweep_io(tensors, configs, uniforms, deltas, full_gradient, want_O, want_p,
                                           want_margin, out)
        return BatchJob(self, _abi.VMC_JOB_SWEEP, tensors, out, uniforms=u, deltas=deltas, cache=cache,
                        full_gradient=full_gradient)

    def amp_grad_job(self, tensors, samples, full_gradient=False, want_O=True, want_gap=False):
        self._check_tensors(tensors)
        c = self._configs(samples)
        n, dev = c.shape[0], self.device
        np_ = self.n_params_full if full_gradient else self.n_params_sliced
        out = SweepResult(configs=c, O=torch.empty((n, np_), dtype=self.param_dtype, device=dev) if want_O else None,
                          p=None, E=None, logamp=torch.empty(n, dtype=torch.float64, device=dev),
                          sign=torch.empty(n, dtype=torch.float64, device=dev), margin=None,
                          gap=torch.empty(n, dtype=torch.float32, device=dev) if want_gap else None)
        return BatchJob(self, _abi.VMC_JOB_AMP_GRAD, tensors, out, full_gradient=full_gradient)

    def local_energy_job(self, tensors, samples, logamp, sign):
        self._check_tensors(tensors)
        c = self._configs(samples)
        out = SweepResult(configs=c, O=None, p=None, E=torch.empty(c.shape[0], dtype=self.energy_dtype,
                                                                     device=self.device),
                          logamp=logamp.to(torch.float64).contiguous(), sign=sign.to(torch.float64).contiguous(),
                          margin=None)
        return BatchJob(self, _abi.VMC_JOB_LOCAL_ENERGY, tensors, out)


@dataclass
class BatchJob:
    """One call of an uneven batch: the engine (plan) it runs on, its inputs, and
    ``out``, whose tensors the launch writes (for a local-energy job, ``out.logamp``
    and ``out.sign`` are the given denominators; an init-cache job writes ``cache``)."""
    engine: PEPSEngine
    kind: int
    tensors: torch.Tensor
    out: SweepResult
    uniforms: torch.Tensor | None = None
    deltas: torch.Tensor | None = None
    cache: torch.Tensor | None = None
    full_gradient: bool = False

    def c_struct(self) -> _abi.VmcPepsJob:
        o = self.out

        def ptr(t):
            return None if t is None else t.data_ptr()

        return _abi.VmcPepsJob(self.engine._plan, self.kind, o.configs.shape[0], int(bool(self.full_gradient)),
                               ptr(self.tensors), ptr(o.configs), ptr(self.uniforms), ptr(self.deltas),
                               ptr(self.cache), ptr(o.O), ptr(o.p), ptr(o.E), ptr(o.logamp), ptr(o.sign),
                               ptr(o.margin), ptr(o.gap))


class PEPSBatch:
    """Uneven batches: jobs on several engines -- lattices, bond dimensions,
    strategies, operators of one element type -- in one persistent launch
    (``vmc_peps_batch``) on torch's current stream.  Each chain's results are
    bit-identical to the engine's single call.  ``run`` allocates only when its
    workspace must grow, so after one warm-up call it can be captured in a CUDA
    graph (the graph replays on the jobs' tensors)."""

    def __init__(self, device=None):
        self.device = None if device is None else torch.device(device)
        self._ws = None
        self._status = None

    def _setup(self, jobs):
        if not jobs:
            raise ValueError("a batch needs at least one job")
        if len(jobs) > _abi.VMC_MAX_BATCH_JOBS:
            raise ValueError(f"at most {_abi.VMC_MAX_BATCH_JOBS} jobs per batch")
        eng0 = jobs[0].engine
        for j in jobs:
            if j.engine.lib is not eng0.lib or j.engine.device != eng0.device:
                raise ValueError("all jobs of a batch run on one library and device")
            if j.engine.complex != eng0.complex:
                raise ValueError("all jobs of a batch have one element type")
        if self.device is None:
            self.device = eng0.device
        elif self.device != eng0.device:
            raise ValueError("jobs on another device than this batch's")
        if self._status is None:
            self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        return eng0.lib, eng0

    LAYOUTS = {None: _abi.VMC_BATCH_LAYOUT_AUTO, "auto": _abi.VMC_BATCH_LAYOUT_AUTO,
               "plan": _abi.VMC_BATCH_LAYOUT_PLAN, "shared": _abi.VMC_BATCH_LAYOUT_PLAN,
               "slot": _abi.VMC_BATCH_LAYOUT_SLOT}

    def run(self, jobs, layout=None):
        """``layout``: buffer placement of the launch -- None / "auto" (by cost share), "plan" (each
        plan's shared-memory placement) or "slot" (every buffer in the CTA's workspace slot)."""
        lib, eng0 = self._setup(jobs)
        lay = self.LAYOUTS[layout]
        arr = (_abi.VmcPepsJob * len(jobs))(*[j.c_struct() for j in jobs])
        need = int(lib.vmc_batch_workspace_size_ex(arr, len(jobs), lay))
        if need == 0:
            raise ValueError("invalid batch (missing buffers, or plans of different element type or CTA size)")
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        st = lib.vmc_peps_batch_ex(arr, len(jobs), lay, eng0._stream(), _vp(self._ws), self._ws.numel(),
                                   _vp(self._status))
        _abi.check(lib, st, "vmc_peps_batch")
        return [j.out for j in jobs]

    def status(self, reset=True) -> int:
        if self._status is None:
            return 0
        v = int(self._status.item())
        if reset and v:
            self._status.zero_()
        return v

    def raise_on_status(self):
        v = self.status()
        if v & _abi.VMC_DEV_NONFINITE:
            raise FloatingPointError("engine reported a non-finite amplitude or energy")
        if v & _abi.VMC_DEV_TIMEOUT:
            raise TimeoutError("engine reported a device-side timeout")


class _null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
