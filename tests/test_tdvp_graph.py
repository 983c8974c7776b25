"""The graph TDVP driver's building blocks on CPU: the device uniform stream (vmc_uniforms) in the
host-emulation build against a NumPy restatement of SplitMix64, and one eager Euler step of
GraphTDVPDriver against SRPreconditioner.apply on the same sweep outputs."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from tests.helpers import hamiltonian
from vmc_gb300 import PEPS, ZipUp
from vmc_gb300.drivers import Euler, ImaginaryTimeUnit
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import ParameterSpace, SampleSpace
from vmc_gb300.tdvp_graph import GraphTDVPDriver

GAMMA = np.uint64(0x9E3779B97F4A7C15)


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def splitmix_uniforms(n, seed, counter):
    with np.errstate(over="ignore"):
        key = _mix(np.array([seed], dtype=np.uint64) + np.uint64(counter + 1) * GAMMA)[0]
        z = _mix(key + (np.arange(1, n + 1, dtype=np.uint64) * GAMMA))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def test_uniform_stream_matches_splitmix64(emu_lib):
    out = torch.empty(1000, dtype=torch.float64)
    counter = torch.tensor([5], dtype=torch.int64)
    for c in (5, 6):
        assert emu_lib.vmc_uniforms(None, ct.c_void_p(out.data_ptr()), out.numel(), 12345,
                                    ct.c_void_p(counter.data_ptr())) == 0
        assert np.array_equal(out.numpy(), splitmix_uniforms(1000, 12345, c))
    assert int(counter.item()) == 7
    u = splitmix_uniforms(200000, 1, 0)
    assert 0.0 <= u.min() and u.max() < 1.0 and abs(u.mean() - 0.5) < 3e-3


def _model(emu_lib, dtype=torch.float32):
    shape, D = (3, 3), 2
    return PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), device="cpu", lib=emu_lib, rngs=3,
                dtype=dtype)


@pytest.mark.parametrize("space", [ParameterSpace(), SampleSpace()])
def test_eager_euler_step_is_the_sr_update(emu_lib, space):
    model = _model(emu_lib)
    H = hamiltonian("heisenberg", model.shape)
    pre = SRPreconditioner(space=space, diag_shift=1e-2)
    drv = GraphTDVPDriver(model, H, preconditioner=pre, dt=0.05, time_unit=ImaginaryTimeUnit(),
                          integrator=Euler(), n_samples=24, n_chains=8, sampler_key=4)
    theta0 = drv.parameters.clone()
    drv.run(0.05)
    assert drv.step_count == 1 and int(drv._counter.item()) == 1
    # the SR update recomputed from the step's own sweep outputs
    N = drv.n_samples
    o = drv._O.reshape(drv._total, -1)[:N]
    p = drv._p.reshape(drv._total, -1)[:N]
    e = drv._E.reshape(-1)[:N]
    samples = torch.zeros((N, 9), dtype=torch.int32)
    upd, _ = SRPreconditioner(space=space, diag_shift=1e-2).apply(model, model.unpack(theta0), samples, o, p, e,
                                                                  grad_factor=-1.0)
    ref = theta0 + 0.05 * torch.cat([t.reshape(-1) for row in upd for t in row])
    assert torch.allclose(drv.parameters, ref, rtol=1e-6, atol=1e-7)
    assert np.isfinite(drv.energy["mean"])


def test_checkpoint_round_trip_reproduces_the_run(emu_lib):
    H = hamiltonian("tfim", (3, 3))
    pre = SRPreconditioner(space=SampleSpace(), diag_shift=1e-2)

    def make():
        return GraphTDVPDriver(_model(emu_lib), H, preconditioner=pre, dt=0.02, time_unit=ImaginaryTimeUnit(),
                               n_samples=16, n_chains=16, sampler_key=9)

    a = make()
    a.run(0.02)
    state = a.state_dict()
    a.run(0.04)
    b = make()
    b.load_state_dict(state)
    b.run(0.04)
    assert torch.equal(a.parameters, b.parameters) and b.step_count == 3


def test_unsupported_configurations_are_refused(emu_lib):
    from vmc_gb300.preconditioners import QRSolve

    model = _model(emu_lib)
    H = hamiltonian("heisenberg", model.shape)
    with pytest.raises(NotImplementedError):
        GraphTDVPDriver(model, H, preconditioner=SRPreconditioner(strategy=QRSolve()), dt=0.1,
                        time_unit=ImaginaryTimeUnit())
    with pytest.raises(NotImplementedError):
        GraphTDVPDriver(model, H, preconditioner=SRPreconditioner(), dt=0.1)  # real time on a real PEPS
