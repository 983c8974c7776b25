"""The FP64 SR / TDVP layer on the GPU against the FP64 oracle (oracle/sr.py) on the same inputs.

The inputs are the engine's own sweep outputs -- O_k, active slice indices and E_loc of sampled
chains -- so the solves see the rank structure and scales of a real run:

- 8x8 Heisenberg, D=4, chi=16, 4096 samples: the sliced Jacobian (4096 x 10,816, two slices), SampleSpace
  DirectSolve with diagonal shift 1e-4, Gram built in 16 column blocks (the reference's sliced
  DirectSolve, preconditioners.py:117-152 and qgt.py:173-223);
- 6x6 Heisenberg, D=4, chi=16, 512 samples: the same in ParameterSpace (a 10,368^2 FP64 S);
- one Euler and one RK4 step of TDVPDriver (integrators.py:45-109): every stage's SR solve is
  re-solved by the oracle from the stage's recorded inputs, and the step's update is the
  integrator's combination of those stages.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import sr as osr
from tests.helpers import hamiltonian, make_case
from vmc_gb300 import PEPS, ZipUp
from vmc_gb300.drivers import RK4, Euler, ImaginaryTimeUnit, TDVPDriver
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors, params_per_site
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import ParameterSpace, SampleSpace

pytestmark = pytest.mark.gpu

N_SAMPLES, N_CHAINS = 1024, 512


def _sweep_outputs(device, shape, D, chi, n):
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, n, seed=3)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=device, precision="mixed")
    tens = torch.from_numpy(pack_tensors(T)).to(device)
    c = torch.from_numpy(cfg).to(device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(device), cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=device,
                 tensors=T)
    return model, res


def _oracle_update(o, p, e, shape, D, space, shift, grad_factor=1.0):
    n = o.shape[0]
    x, _ = osr.sr_apply(o.cpu().numpy().astype(np.float64), None if p is None else p.cpu().numpy(),
                        e.cpu().numpy().astype(np.float64), pps=params_per_site(shape, D),
                        sliced_dims=(2,) * (shape[0] * shape[1]), n_samples=n, space=space,
                        strategy=osr.DirectSolve(), diag_shift=shift, ordering=osr.SliceOrdering(),
                        grad_factor=grad_factor, real_params=True)
    return x


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_config2_sliced_direct_solve_sample_space(cuda_device):
    shape, D, chi, n = (8, 8), 4, 16, 4096
    model, res = _sweep_outputs(cuda_device, shape, D, chi, n)
    assert res.O.shape == (n, 10816)
    pre = SRPreconditioner(space=SampleSpace(), diag_shift=1e-4)
    upd, metrics = pre.apply(model, model.tensors, res.configs, res.O, res.p, res.E)
    x = model.packed(upd).double().cpu().numpy()
    x_ref = _oracle_update(res.O, res.p, res.E, shape, D, osr.SampleSpace(), 1e-4)
    assert x.shape == x_ref.shape == (2 * 10816,)
    # FP64 solves on both sides; the update is returned in the parameters' FP32
    assert _rel(x, x_ref) < 1e-6, _rel(x, x_ref)
    assert np.isfinite(float(metrics["residual_error"]))


def test_parameter_space_sliced_direct_solve(cuda_device):
    shape, D, chi, n = (6, 6), 4, 16, 512
    model, res = _sweep_outputs(cuda_device, shape, D, chi, n)
    pre = SRPreconditioner(space=ParameterSpace(), diag_shift=1e-4)
    upd, _ = pre.apply(model, model.tensors, res.configs, res.O, res.p, res.E)
    x = model.packed(upd).double().cpu().numpy()
    x_ref = _oracle_update(res.O, res.p, res.E, shape, D, osr.ParameterSpace(), 1e-4)
    assert _rel(x, x_ref) < 1e-6, _rel(x, x_ref)


class _Recording(SRPreconditioner):
    """SRPreconditioner that keeps every stage's inputs and flat update."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.stages = []

    def apply(self, model, params, samples, o, p, local_energies, *, grad_factor=1.0):
        upd, metrics = super().apply(model, params, samples, o, p, local_energies, grad_factor=grad_factor)
        self.stages.append((o.clone(), None if p is None else p.clone(), local_energies.clone(), grad_factor,
                            model.packed(upd).double().cpu().numpy()))
        return upd, metrics


@pytest.mark.parametrize("integrator,space", [(Euler(), SampleSpace()), (RK4(), SampleSpace()),
                                              (RK4(), ParameterSpace())], ids=["euler", "rk4", "rk4-param"])
def test_tdvp_step_matches_oracle_stages(cuda_device, integrator, space):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, rngs=5)
    theta0 = model.packed().double().cpu().numpy()
    pre = _Recording(space=space, diag_shift=1e-3)
    dt = 0.02
    drv = TDVPDriver(model, H, preconditioner=pre, dt=dt, time_unit=ImaginaryTimeUnit(), integrator=integrator,
                     n_samples=N_SAMPLES, n_chains=N_CHAINS, sampler_key=9)
    drv.run(dt)
    ks = []
    for o, p, e, gf, x in pre.stages:
        x_ref = _oracle_update(o, p, e, shape, D, osr.SampleSpace() if isinstance(space, SampleSpace)
                               else osr.ParameterSpace(), 1e-3, grad_factor=gf)
        assert _rel(x, x_ref) < 1e-6, _rel(x, x_ref)
        ks.append(x_ref)
    if isinstance(integrator, Euler):
        assert len(ks) == 1
        want = theta0 + dt * ks[0]
    else:
        assert len(ks) == 4
        want = theta0 + dt * (ks[0] + 2 * ks[1] + 2 * ks[2] + ks[3]) / 6.0
    got = drv.model.packed().double().cpu().numpy()
    assert _rel(got - theta0, want - theta0) < 1e-5, _rel(got - theta0, want - theta0)


@pytest.mark.parametrize("space,qr", [(SampleSpace(), False), (ParameterSpace(), False), (ParameterSpace(), True)],
                         ids=["sample-direct", "parameter-direct", "parameter-qr"])
def test_gauge_removed_solve_matches_the_dense_formulation(cuda_device, space, qr):
    """Gauge removal on the GPU (6x6 D4 chi16, 512 samples, full gradient): the update against the
    reference's formulation (solve with O Q, return Q y) evaluated with an explicit Q in FP64."""
    from vmc_gb300.gauge import GaugeConfig, compute_gauge_projection
    from vmc_gb300.preconditioners import QRSolve

    shape, D, chi, n = (6, 6), 4, 16, 512
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, n, seed=3)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device=cuda_device, precision="mixed")
    tens = torch.from_numpy(pack_tensors(T)).to(cuda_device)
    c = torch.from_numpy(cfg).to(cuda_device)
    cache = eng.init_cache(tens, c)
    res = eng.sweep(tens, c, torch.from_numpy(u).to(cuda_device), cache, full_gradient=True)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, tensors=T)
    pre = SRPreconditioner(space=space, diag_shift=1e-3, gauge_config=GaugeConfig(),
                           strategy=QRSolve() if qr else SRPreconditioner().strategy)
    upd, metrics = pre.apply(model, model.tensors, res.configs, res.O, None, res.E)
    x = model.packed(upd).double()
    Q = compute_gauge_projection(GaugeConfig(), model, model.tensors).dense()
    oc = res.O.double() @ Q
    oc = oc - oc.mean(0)
    e = res.E.double()
    dv = (e - e.mean()) / n
    if qr:
        red = torch.linalg.lstsq(oc.cpu(), dv.cpu(), driver="gelsd", rcond=1e-12).solution.to(cuda_device)
    elif isinstance(space, SampleSpace):
        red = oc.T @ torch.linalg.solve(oc @ oc.T / n + 1e-3 * torch.eye(n, dtype=torch.float64, device=cuda_device),
                                        dv)
    else:
        red = torch.linalg.solve(oc.T @ oc / n + 1e-3 * torch.eye(Q.shape[1], dtype=torch.float64,
                                                                  device=cuda_device), oc.T @ dv)
    want = 2.0 * (Q @ red)
    assert torch.linalg.norm(x - want) / torch.linalg.norm(want) < 1e-5
    # 60 bonds x D^2 generators and the global scale, less one dependency per plaquette: the scalar
    # (T = 1) gauges span the lattice graph's cut space, of dimension n_sites - 1 = 35, not 60
    assert metrics["gauge_rank"] == 60 * 16 - 25 + 1


@pytest.mark.parametrize("space", [SampleSpace(), ParameterSpace()], ids=["sample", "parameter"])
def test_graph_tdvp_step_matches_oracle(cuda_device, space):
    """A replayed GraphTDVPDriver Euler step: the parameter change over the replay is dt times the
    oracle's SR update (oracle/sr.py) of the sweep outputs the replay left in the driver's buffers."""
    from vmc_gb300.tdvp_graph import GraphTDVPDriver

    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, rngs=5)
    dt = 0.02
    drv = GraphTDVPDriver(model, H, preconditioner=SRPreconditioner(space=space, diag_shift=1e-3), dt=dt,
                          time_unit=ImaginaryTimeUnit(), integrator=Euler(), n_samples=N_SAMPLES,
                          n_chains=N_CHAINS, sampler_key=9)
    drv.run(2 * dt)  # the eager step, then the capture
    assert drv._graph is not None
    theta0 = drv.parameters.double().cpu().numpy()
    drv.run(dt)      # one replay
    theta1 = drv.parameters.double().cpu().numpy()
    n = N_SAMPLES
    o = drv._O.reshape(-1, drv._O.shape[-1])[:n]
    p = drv._p.reshape(-1, drv._p.shape[-1])[:n]
    e = drv._E.reshape(-1)[:n]
    x_ref = _oracle_update(o, p, e, shape, D, osr.SampleSpace() if isinstance(space, SampleSpace)
                           else osr.ParameterSpace(), 1e-3, grad_factor=drv.time_unit.grad_factor)
    assert _rel(theta1 - theta0, dt * x_ref) < 1e-5, _rel(theta1 - theta0, dt * x_ref)
