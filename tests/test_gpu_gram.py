"""vmc_sliced_gram on the GPU against the expanded-block product in FP64 (cuBLAS), and its use in the
SampleSpace solve (the config-2 solve against the oracle runs in tests/test_gpu_sr.py)."""
from __future__ import annotations

import pytest
import torch

from vmc_gb300 import qgt as gq
from vmc_gb300.linalg import sliced_gram

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,ncols,d", [(1000, 3000, 2), (64, 31, 3), (130, 257, 2), (1, 5, 2)])
def test_sliced_gram_matches_fp64_expanded_product(cuda_device, n, ncols, d):
    g = torch.Generator(device=cuda_device)
    g.manual_seed(n + ncols)
    o = torch.randn((n, ncols), generator=g, device=cuda_device, dtype=torch.float32)
    p = torch.randint(0, d, (n, ncols), generator=g, device=cuda_device, dtype=torch.int8)
    T = sliced_gram(o, p)
    jac = gq.SlicedJacobian(o, p, (d,) * ncols)
    ref = sum(ob @ ob.T for ob in gq.iter_sliced_blocks(jac))
    assert torch.equal(T, T.T)
    # exact FP32 products summed in double-float, flushed to FP64 every 256 columns
    scale = torch.sqrt(torch.outer(torch.diagonal(ref), torch.diagonal(ref))).clamp_min(1e-300)
    assert float(((T - ref).abs() / scale).max()) < 1e-12
    assert float(torch.linalg.norm(T - ref) / torch.linalg.norm(ref)) < 1e-13


def test_sample_space_dense_uses_the_kernel_and_agrees(cuda_device):
    g = torch.Generator(device=cuda_device)
    g.manual_seed(3)
    o = torch.randn((300, 700), generator=g, device=cuda_device, dtype=torch.float32)
    p = torch.randint(0, 2, (300, 700), generator=g, device=cuda_device, dtype=torch.int8)
    jac = gq.SlicedJacobian(o, p, (2,) * 700)
    assert gq._kernel_gram(jac)
    T = gq.QGT(jac, gq.SampleSpace()).to_dense()
    dense = torch.cat(list(gq.iter_sliced_blocks(jac)), dim=1)
    oc = dense - dense.mean(0)
    ref = oc @ oc.T / 300
    assert float(torch.linalg.norm(T - ref) / torch.linalg.norm(ref)) < 1e-12


@pytest.mark.parametrize("n,ncols", [(700, 300), (64, 31), (1, 5), (33, 64)])
def test_sliced_gram_params_matches_fp64_expanded_product(cuda_device, n, ncols):
    from vmc_gb300.linalg import sliced_gram_params

    g = torch.Generator(device=cuda_device)
    g.manual_seed(n + 7 * ncols)
    o = torch.randn((n, ncols), generator=g, device=cuda_device, dtype=torch.float32)
    p = torch.randint(0, 2, (n, ncols), generator=g, device=cuda_device, dtype=torch.int8)
    S = sliced_gram_params(o, p)
    jac = gq.SlicedJacobian(o, p, (2,) * ncols)
    E = torch.cat(list(gq.iter_sliced_blocks(jac)), dim=1)
    ref = E.T @ E
    assert torch.equal(S, S.T)
    scale = torch.sqrt(torch.outer(torch.diagonal(ref), torch.diagonal(ref))).clamp_min(1e-300)
    assert float(((S - ref).abs() / scale).max()) < 1e-12
    assert float(torch.linalg.norm(S - ref) / torch.linalg.norm(ref)) < 1e-13


def test_parameter_space_dense_uses_the_kernel_and_agrees(cuda_device):
    g = torch.Generator(device=cuda_device)
    g.manual_seed(5)
    o = torch.randn((300, 200), generator=g, device=cuda_device, dtype=torch.float32)
    p = torch.randint(0, 2, (300, 200), generator=g, device=cuda_device, dtype=torch.int8)
    jac = gq.SlicedJacobian(o, p, (2,) * 200)
    S = gq.QGT(jac, gq.ParameterSpace()).to_dense()
    E = torch.cat(list(gq.iter_sliced_blocks(jac)), dim=1)
    m = E.mean(0)
    ref = E.T @ E / 300 - m[:, None] * m[None, :]
    assert float(torch.linalg.norm(S - ref) / torch.linalg.norm(ref)) < 1e-12


def test_parameter_space_dense_site_ordering_uses_the_kernel(cuda_device):
    g = torch.Generator(device=cuda_device)
    g.manual_seed(9)
    pps = (40, 70, 25, 65)
    ncols = sum(pps)
    o = torch.randn((257, ncols), generator=g, device=cuda_device, dtype=torch.float32)
    p = torch.randint(0, 2, (257, ncols), generator=g, device=cuda_device, dtype=torch.int8)
    jac = gq.SlicedJacobian(o, p, (2,) * len(pps), gq.SiteOrdering(pps))
    assert gq._kernel_gram(jac) and gq._site_from_slice_order(jac) is not None
    S = gq.QGT(jac, gq.ParameterSpace()).to_dense()
    E = torch.cat(list(gq.iter_sliced_blocks(jac)), dim=1)
    m = E.mean(0)
    ref = E.T @ E / 257 - m[:, None] * m[None, :]
    assert float(torch.linalg.norm(S - ref) / torch.linalg.norm(ref)) < 1e-12
