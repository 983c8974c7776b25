"""vmc_sliced_gram (the SampleSpace Gram of a sliced Jacobian) through the host-emulation library, and
the centring terms computed from the sliced rows, against the expanded-block formulation
(src/vmc/qgt/qgt.py:173-223)."""
from __future__ import annotations

import ctypes as ct

import numpy as np
import pytest
import torch

from vmc_gb300 import _abi
from vmc_gb300 import qgt as gq


def _expanded_gram(o, p, d):
    o = o.astype(np.float64)
    return sum((np.where(p == k, o, 0.0)) @ (np.where(p == k, o, 0.0)).T for k in range(d))


def _call(lib, o, p, ld=None):
    n, ncols = o.shape
    ld = ncols if ld is None else ld
    ob = np.zeros((n, ld), np.float32)
    pb = np.zeros((n, ld), np.int8)
    ob[:, :ncols] = o
    pb[:, :ncols] = p
    out = np.full((n, n), np.nan)
    st = lib.vmc_sliced_gram(None, ob.ctypes.data_as(ct.c_void_p), pb.ctypes.data_as(ct.c_void_p), n, ncols, ld,
                             out.ctypes.data_as(ct.c_void_p))
    return st, out


@pytest.mark.parametrize("n,ncols,d,ld", [(70, 45, 2, None), (5, 33, 3, 40), (1, 1, 2, None)])
def test_sliced_gram_equals_the_expanded_product(emu_lib, n, ncols, d, ld):
    rng = np.random.default_rng(n + ncols)
    o = rng.standard_normal((n, ncols)).astype(np.float32)
    p = rng.integers(0, d, (n, ncols)).astype(np.int8)
    st, out = _call(emu_lib, o, p, ld)
    assert st == _abi.VMC_OK
    ref = _expanded_gram(o, p, d)
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-12)
    assert np.array_equal(out, out.T)


def test_sliced_gram_rejects_bad_arguments(emu_lib):
    o = np.zeros((4, 8), np.float32)
    p = np.zeros((4, 8), np.int8)
    out = np.zeros((4, 4))
    args = (o.ctypes.data_as(ct.c_void_p), p.ctypes.data_as(ct.c_void_p))
    assert emu_lib.vmc_sliced_gram(None, *args, 4, 8, 7, out.ctypes.data_as(ct.c_void_p)) == _abi.VMC_ERR_INVALID
    assert emu_lib.vmc_sliced_gram(None, *args, -1, 8, 8, out.ctypes.data_as(ct.c_void_p)) == _abi.VMC_ERR_INVALID
    assert emu_lib.vmc_sliced_gram(None, None, None, 4, 8, 8, None) == _abi.VMC_ERR_INVALID
    assert emu_lib.vmc_sliced_gram(None, None, None, 0, 8, 8, None) == _abi.VMC_OK


@pytest.mark.parametrize("d", [2, 3])
def test_sliced_centring_equals_the_block_terms(d):
    rng = np.random.default_rng(d)
    o = torch.from_numpy(rng.standard_normal((37, 29)).astype(np.float32))
    p = torch.from_numpy(rng.integers(0, d, (37, 29)).astype(np.int8))
    jac = gq.SlicedJacobian(o, p, (d,) * 29)
    w, msq = gq.sliced_centring(jac)
    w_ref = torch.zeros(37, dtype=torch.float64)
    msq_ref = torch.zeros((), dtype=torch.float64)
    for ob in gq.iter_sliced_blocks(jac):
        mb = ob.mean(dim=0)
        w_ref += ob @ mb
        msq_ref += mb @ mb
    assert torch.allclose(w, w_ref, rtol=1e-12, atol=1e-14)
    assert torch.allclose(msq, msq_ref, rtol=1e-12)


def _expanded_params(o, p, d):
    o = o.astype(np.float64)
    E = np.concatenate([np.where(p == k, o, 0.0) for k in range(d)], axis=1)
    return E.T @ E


@pytest.mark.parametrize("n,ncols,ld", [(37, 45, None), (5, 33, 40), (1, 1, None)])
def test_sliced_gram_params_equals_the_expanded_product(emu_lib, n, ncols, ld):
    rng = np.random.default_rng(n * ncols)
    o = rng.standard_normal((n, ncols)).astype(np.float32)
    p = rng.integers(0, 2, (n, ncols)).astype(np.int8)
    ld = ncols if ld is None else ld
    ob = np.zeros((n, ld), np.float32)
    pb = np.zeros((n, ld), np.int8)
    ob[:, :ncols] = o
    pb[:, :ncols] = p
    out = np.full((2 * ncols, 2 * ncols), np.nan)
    st = emu_lib.vmc_sliced_gram_params(None, ob.ctypes.data_as(ct.c_void_p), pb.ctypes.data_as(ct.c_void_p), n,
                                        ncols, ld, 2, out.ctypes.data_as(ct.c_void_p))
    assert st == _abi.VMC_OK
    assert np.allclose(out, _expanded_params(o, p, 2), rtol=1e-12, atol=1e-12)


def test_sliced_gram_params_rejects_bad_arguments(emu_lib):
    o = np.zeros((4, 8), np.float32)
    p = np.zeros((4, 8), np.int8)
    out = np.zeros((16, 16))
    args = (o.ctypes.data_as(ct.c_void_p), p.ctypes.data_as(ct.c_void_p))
    assert emu_lib.vmc_sliced_gram_params(None, *args, 4, 8, 8, 3, out.ctypes.data_as(ct.c_void_p)) == \
        _abi.VMC_ERR_UNSUPPORTED
    assert emu_lib.vmc_sliced_gram_params(None, *args, 4, 8, 7, 2, out.ctypes.data_as(ct.c_void_p)) == \
        _abi.VMC_ERR_INVALID
    assert emu_lib.vmc_sliced_gram_params(None, None, None, 4, 8, 8, 2, None) == _abi.VMC_ERR_INVALID
    assert emu_lib.vmc_sliced_gram_params(None, None, None, 0, 0, 1, 2, None) == _abi.VMC_OK


def test_site_order_is_the_slice_order_permuted():
    """The ParameterSpace S of a site-ordered sliced Jacobian (jacobian.py:36-46) is the slice-ordered S
    with rows and columns permuted by qgt._site_from_slice_order (how the GPU path reuses its kernel)."""
    rng = np.random.default_rng(3)
    pps = (3, 5, 2, 4)
    ncols = sum(pps)
    o = torch.from_numpy(rng.standard_normal((9, ncols)).astype(np.float32))
    p = torch.from_numpy(rng.integers(0, 2, (9, ncols)).astype(np.int8))
    sd = (2,) * len(pps)
    site = gq.SlicedJacobian(o, p, sd, gq.SiteOrdering(pps))
    slc = gq.SlicedJacobian(o, p, sd, gq.SliceOrdering())
    S_site = gq.QGT(site, gq.ParameterSpace()).to_dense()
    S_slice = gq.QGT(slc, gq.ParameterSpace()).to_dense()
    idx = gq._site_from_slice_order(site)
    assert torch.allclose(S_slice.index_select(0, idx).index_select(1, idx), S_site, rtol=1e-12, atol=1e-14)
    assert gq._site_from_slice_order(slc) is None
