"""PyTorch operators over the engine's C ABI (``torch.ops.vmc_gb300.*``, registered with torch.library).

Each operator takes an engine handle (``register_engine``), the packed FP32 / complex64 parameters and
int32 samples, and launches the engine's kernels on torch's current stream.  Every operator has a fake
(meta) implementation, so they trace under FakeTensor / torch.compile graph capture with the output
shapes the engine would produce.

    amp_grad(engine, packed, samples, full_gradient)  -> (log|psi|, sign or phase, O)   vmc_peps_amp_grad
    vjp(engine, packed, samples, weights)             -> sum_i w_i O_i (full layout)    vmc_peps_vjp
    local_energy(engine, packed, samples, logamp, sign) -> E_loc                         vmc_peps_local_energy
    sweep(engine, packed, configs!, uniforms, cache!, deltas?, full_gradient)
                                                      -> (O, p, E, log|psi|, sign)      vmc_peps_sweep
    peps_amplitude(engine, packed, samples)           -> psi, differentiable in packed

``peps_amplitude`` is the torch counterpart of the reference's ``peps_apply`` custom VJP
(src/vmc/peps/standard/compat.py:31-64): its backward is ``vjp`` with w_i = g_i psi_i, which rebuilds the
environments in the kernel and accumulates the gradient there, so no (n, n_params) matrix is stored
between forward and backward.
"""
from __future__ import annotations

import weakref
from typing import Optional

import torch
from torch import Tensor

__all__ = ["register_engine", "engine_of", "amp_grad", "vjp", "local_energy", "sweep", "peps_amplitude"]

_ENGINES: "weakref.WeakValueDictionary[int, object]" = weakref.WeakValueDictionary()


def register_engine(engine) -> int:
    """The integer handle the operators take for `engine` (kept while the engine lives)."""
    key = id(engine)
    _ENGINES[key] = engine
    return key


def engine_of(handle: int):
    eng = _ENGINES.get(int(handle))
    if eng is None:
        raise KeyError(f"no live vmc_gb300 engine with handle {handle}")
    return eng


def _energy_dtype(eng):
    return torch.complex128 if eng.complex else torch.float64


@torch.library.custom_op("vmc_gb300::amp_grad", mutates_args=())
def amp_grad(engine: int, packed: Tensor, samples: Tensor, full_gradient: bool) -> tuple[Tensor, Tensor, Tensor]:
    eng = engine_of(engine)
    la, sg, O = eng.amp_grad(packed.contiguous(), samples, full_gradient=full_gradient, want_O=True)
    return la, sg, O


@amp_grad.register_fake
def _(engine, packed, samples, full_gradient):
    eng = engine_of(engine)
    n = samples.shape[0]
    np_ = eng.n_params_full if full_gradient else eng.n_params_sliced
    return (packed.new_empty(n, dtype=torch.float64), packed.new_empty(n, dtype=torch.float64),
            packed.new_empty((n, np_), dtype=eng.param_dtype))


@torch.library.custom_op("vmc_gb300::vjp", mutates_args=())
def vjp(engine: int, packed: Tensor, samples: Tensor, weights: Tensor) -> Tensor:
    return engine_of(engine).vjp(packed.contiguous(), samples, weights)


@vjp.register_fake
def _(engine, packed, samples, weights):
    eng = engine_of(engine)
    return packed.new_empty(eng.n_params_full, dtype=_energy_dtype(eng))


@torch.library.custom_op("vmc_gb300::local_energy", mutates_args=())
def local_energy(engine: int, packed: Tensor, samples: Tensor, logamp: Tensor, sign: Tensor) -> Tensor:
    return engine_of(engine).local_energy(packed.contiguous(), samples, logamp, sign)


@local_energy.register_fake
def _(engine, packed, samples, logamp, sign):
    return packed.new_empty(samples.shape[0], dtype=_energy_dtype(engine_of(engine)))


@torch.library.custom_op("vmc_gb300::sweep", mutates_args=("configs", "cache"))
def sweep(engine: int, packed: Tensor, configs: Tensor, uniforms: Tensor, cache: Tensor, deltas: Optional[Tensor],
          full_gradient: bool) -> tuple[Tensor, Tensor, Tensor, Tensor, Tensor]:
    res = engine_of(engine).sweep(packed.contiguous(), configs, uniforms, cache, deltas=deltas,
                                  full_gradient=full_gradient)
    return res.O, res.p, res.E, res.logamp, res.sign


@sweep.register_fake
def _(engine, packed, configs, uniforms, cache, deltas, full_gradient):
    eng = engine_of(engine)
    n = configs.shape[0]
    np_ = eng.n_params_full if full_gradient else eng.n_params_sliced
    return (packed.new_empty((n, np_), dtype=eng.param_dtype),
            packed.new_empty((n, eng.n_params_sliced), dtype=torch.int8),
            packed.new_empty(n, dtype=_energy_dtype(eng)), packed.new_empty(n, dtype=torch.float64),
            packed.new_empty(n, dtype=torch.float64))


@torch.library.custom_op("vmc_gb300::peps_amplitude", mutates_args=())
def peps_amplitude(engine: int, packed: Tensor, samples: Tensor) -> Tensor:
    eng = engine_of(engine)
    la, sg, _ = eng.amp_grad(packed.contiguous(), samples, want_O=False)
    return eng.amplitude(la, sg)


@peps_amplitude.register_fake
def _(engine, packed, samples):
    return packed.new_empty(samples.shape[0], dtype=_energy_dtype(engine_of(engine)))


def _amp_setup(ctx, inputs, output):
    engine, packed, samples = inputs
    ctx.engine = engine
    ctx.param_dtype = packed.dtype
    ctx.save_for_backward(packed, samples, output)


def _amp_backward(ctx, g):
    packed, samples, amp = ctx.saved_tensors
    # d psi_i / d theta = psi_i O_i and psi is holomorphic in theta: torch's gradient is
    # sum_i g_i conj(psi_i O_i) = conj(sum_i conj(g_i) psi_i O_i); real: sum_i g_i psi_i O_i
    if amp.is_complex():
        grad = torch.conj(vjp(ctx.engine, packed, samples, torch.conj(g) * amp))
    else:
        grad = vjp(ctx.engine, packed, samples, g * amp)
    return None, grad.to(ctx.param_dtype), None


peps_amplitude.register_autograd(_amp_backward, setup_context=_amp_setup)
