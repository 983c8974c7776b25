"""A whole TDVP step (sampling, FP64 SR solve, RK4 update) replayed from one CUDA graph gives the
bits of the same steps run eagerly: same configurations, same parameters, same energies."""
from __future__ import annotations

import pytest
import torch

from tests.helpers import complex_tensors, hamiltonian
from vmc_gb300 import PEPS, ZipUp
from vmc_gb300.drivers import RK4, ImaginaryTimeUnit, RealTimeUnit
from vmc_gb300.preconditioners import SRPreconditioner
from vmc_gb300.qgt import ParameterSpace, SampleSpace
from vmc_gb300.tdvp_graph import GraphTDVPDriver

pytestmark = pytest.mark.gpu


def _pair(cuda_device, shape, D, chi, model_name, dtype, time_unit, space, n_samples, n_chains):
    H = hamiltonian(model_name, shape)
    out = []
    for graph in (False, True):
        tensors = complex_tensors(shape, D, seed=2) if dtype == torch.complex64 else None
        model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(chi), device=cuda_device, rngs=2,
                     dtype=dtype, tensors=tensors)
        out.append(GraphTDVPDriver(model, H, preconditioner=SRPreconditioner(space=space, diag_shift=1e-2),
                                   dt=0.01, time_unit=time_unit, integrator=RK4(), n_samples=n_samples,
                                   n_chains=n_chains, sampler_key=11, use_graph=graph))
    return out


@pytest.mark.parametrize("space", [SampleSpace(), ParameterSpace()])
def test_graph_steps_equal_eager_steps_real_imaginary_time(cuda_device, space):
    eager, graph = _pair(cuda_device, (4, 4), 2, 4, "heisenberg", torch.float32, ImaginaryTimeUnit(), space,
                         512, 256)
    eager.run(0.03)
    graph.run(0.03)  # one eager step, the capture, two replays
    assert graph._graph is not None
    assert torch.equal(eager._configs, graph._configs)
    assert torch.equal(eager.parameters, graph.parameters)
    assert eager.energy["mean"] == graph.energy["mean"]


def test_graph_steps_equal_eager_steps_complex_real_time(cuda_device):
    eager, graph = _pair(cuda_device, (4, 4), 3, 9, "tfim", torch.complex64, RealTimeUnit(), SampleSpace(),
                         256, 256)
    eager.run(0.02)
    graph.run(0.02)
    assert torch.equal(eager._configs, graph._configs)
    assert torch.equal(torch.view_as_real(eager.parameters), torch.view_as_real(graph.parameters))
