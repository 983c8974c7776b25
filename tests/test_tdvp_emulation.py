"""One Euler and one RK4 step of TDVPDriver (integrators.py:45-109) on the host emulation of the kernels,
in both SR spaces and in imaginary and real time: every stage's SR solve is re-solved by the oracle
(oracle/sr.py) from the stage's recorded inputs, and the step's parameter change is the integrator's
combination of those stages.  The same check runs on the GPU at a larger size."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import sr as osr
from tests.helpers import complex_tensors, hamiltonian
from vmc_gb300 import PEPS, ZipUp
from vmc_gb300.drivers import RK4, Euler, ImaginaryTimeUnit, RealTimeUnit, TDVPDriver
from vmc_gb300.lowering import params_per_site
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import ParameterSpace, SampleSpace


class _Recording(SRPreconditioner):
    """SRPreconditioner that keeps every stage's inputs and flat update."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.stages = []

    def apply(self, model, params, samples, o, p, local_energies, *, grad_factor=1.0):
        upd, metrics = super().apply(model, params, samples, o, p, local_energies, grad_factor=grad_factor)
        self.stages.append((o.clone(), None if p is None else p.clone(), local_energies.clone(), grad_factor,
                            model.packed(upd).to(torch.complex128).numpy()))
        return upd, metrics


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("integrator,space,real_time", [
    (Euler(), SampleSpace(), False), (RK4(), SampleSpace(), False), (RK4(), ParameterSpace(), False),
    (RK4(), SampleSpace(), True)], ids=["euler", "rk4", "rk4-param", "rk4-real-time"])
def test_tdvp_step_matches_oracle_stages(emu_lib, integrator, space, real_time):
    shape, D, chi = (3, 3), 2, 4
    H = hamiltonian("tfim" if real_time else "heisenberg", shape)
    if real_time:
        model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device="cpu", lib=emu_lib,
                     dtype=torch.complex64, tensors=complex_tensors(shape, D, seed=3))
    else:
        model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device="cpu", lib=emu_lib, rngs=5)
    theta0 = model.packed().to(torch.complex128).numpy()
    shift, dt = 1e-3, 0.02
    pre = _Recording(space=space, diag_shift=shift)
    drv = TDVPDriver(model, H, preconditioner=pre, dt=dt, time_unit=RealTimeUnit() if real_time else ImaginaryTimeUnit(),
                     integrator=integrator, n_samples=64, n_chains=32, sampler_key=9)
    drv.run(dt)
    ks = []
    for o, p, e, gf, x in pre.stages:
        x_ref, _ = osr.sr_apply(o.numpy().astype(np.complex128 if o.is_complex() else np.float64),
                                None if p is None else p.numpy(),
                                e.numpy().astype(np.complex128 if e.is_complex() else np.float64),
                                pps=params_per_site(shape, D), sliced_dims=(2,) * (shape[0] * shape[1]),
                                n_samples=o.shape[0],
                                space=osr.SampleSpace() if isinstance(space, SampleSpace) else osr.ParameterSpace(),
                                strategy=osr.DirectSolve(), diag_shift=shift, ordering=osr.SliceOrdering(),
                                grad_factor=gf, real_params=not real_time)
        assert _rel(x, x_ref) < 1e-6, _rel(x, x_ref)
        ks.append(x_ref)
    if isinstance(integrator, Euler):
        assert len(ks) == 1
        want = theta0 + dt * ks[0]
    else:
        assert len(ks) == 4
        want = theta0 + dt * (ks[0] + 2 * ks[1] + 2 * ks[2] + ks[3]) / 6.0
    got = drv.model.packed().to(torch.complex128).numpy()
    assert _rel(got - theta0, want - theta0) < 1e-5, _rel(got - theta0, want - theta0)
    assert drv.step_count == 1 and abs(drv.t - dt) < 1e-12
