"""Evaluation surfaces of src/vmc/peps/standard/compat.py on the engine.

* ``peps_apply``: amplitude with a hand-written adjoint (compat.py:31-64), the
  ``vmc_gb300::peps_amplitude`` operator: its backward is the engine's
  vector-Jacobian product (``vmc_peps_vjp``), which rebuilds the environments
  and accumulates sum_i g_i dpsi_i/dtheta in the kernel -- nothing per sample
  is stored between forward and backward.
* ``_value`` / ``_grad`` / ``_value_and_grad`` (compat.py:67-133).
* ``local_estimate`` (compat.py:136-194).

For d = 2, samples may be 0/1 occupancies or +-1 spins, mapped by the reference's
``spin_to_occupancy`` (src/vmc/utils/utils.py:55-57).  For d > 2 they are occupancies 0..d-1 taken as
given, the sampler kernels' convention: the reference's (s + 1) // 2 would send occupancy 2 to 1.
"""
from __future__ import annotations

import torch

from . import ops
from .lowering import params_per_site

__all__ = ["peps_apply", "log_value", "_value", "_grad", "_value_and_grad", "local_estimate",
           "spin_to_occupancy", "occupancy_to_spin"]


def spin_to_occupancy(spins):
    """src/vmc/utils/utils.py:55-57 (idempotent on 0/1 occupancies)."""
    return torch.div(spins + 1, 2, rounding_mode="floor").to(torch.int32)


def occupancy_to_spin(occ):
    """src/vmc/utils/utils.py:50-52."""
    return (2 * occ - 1).to(torch.int32)


def _samples(model, samples):
    s = torch.as_tensor(samples, device=model.device)
    if s.ndim == 1:
        s = s[None]
    n_sites = model.shape[0] * model.shape[1]
    s = s.reshape(-1, n_sites)
    if model.phys_dim == 2:
        s = spin_to_occupancy(s)
    return s.to(torch.int32).contiguous()


def peps_apply(tensors, sample, shape, strategy, model=None):
    """compat.py:31-40: amplitude(s) of `sample` (n, n_sites) or (n_sites,)."""
    from .peps import PEPS

    if model is None:
        if isinstance(tensors, PEPS):
            model = tensors
        else:
            raise TypeError("peps_apply needs the PEPS model (it carries the engine plan)")
    packed = model.packed(tensors if not isinstance(tensors, PEPS) else None)
    s = _samples(model, sample)
    amp = ops.peps_amplitude(ops.register_engine(model.engine()), packed, s)
    return amp if torch.as_tensor(sample).ndim > 1 else amp[0]


def log_value(model, samples, tensors=None):
    """(log|psi|, sign) for a batch -- (log|psi|, phase) for a complex model; never underflows."""
    eng = model.engine()
    logamp, sign, _ = eng.amp_grad(model.packed(tensors), _samples(model, samples), want_O=False)
    return logamp, sign


def _value(model, sample):
    """compat.py:67-78 (float64 / complex128 amplitudes)."""
    la, sg = log_value(model, sample)
    amp = model.engine().amplitude(la, sg)
    return amp if torch.as_tensor(sample).ndim > 1 else amp[0]


def _value_and_grad(model, sample, *, full_gradient=False):
    """compat.py:94-133: (amp, dpsi/dA, p) with the sliced or full layout."""
    eng = model.engine()
    s = _samples(model, sample)
    logamp, sign, O = eng.amp_grad(model.packed(), s, full_gradient=full_gradient, want_O=True)
    amp = eng.amplitude(logamp, sign)
    grads = O.to(amp.dtype) * amp[:, None]
    p = None
    if not full_gradient:
        pps = torch.as_tensor(params_per_site(model.shape, model.bond_dim), device=s.device)
        p = torch.repeat_interleave(s.to(torch.int8), pps, dim=1)
    if torch.as_tensor(sample).ndim == 1:
        return amp[0], grads[0], None if p is None else p[0]
    return amp, grads, p


def _grad(model, sample, *, full_gradient=False):
    """compat.py:81-91."""
    _, g, p = _value_and_grad(model, sample, full_gradient=full_gradient)
    return g, p


def local_estimate(model, samples, operator, amps):
    """compat.py:136-194: E_loc with the caller's amplitudes as denominators.

    ``amps`` is a tensor of amplitudes or a (log|psi|, sign-or-phase) pair."""
    eng = model.engine(operator)
    s = _samples(model, samples)
    if isinstance(amps, tuple):
        logamp, sign = amps
    else:
        logamp, sign = eng.log_sign(amps)
    return eng.local_energy(model.packed(), s, logamp, sign)
