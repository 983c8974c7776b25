"""FP64 factorisations and Gram matrices of the SR solve on the GPU.

``qr_pivoted`` is the column-pivoted QR of src/vmc/preconditioners/preconditioners.py:178-180
(``jax.lax.linalg.qr(o_centered, full_matrices=False, pivoting=True)``, LAPACK/MAGMA xGEQP3),
run by the engine library's ``vmc_qr_pivoted`` kernels in FP64 or complex128.  ``sliced_gram``
is the sample-space Gram matrix of a real sliced Jacobian (``vmc_sliced_gram``), the FP64 matrix
of the SampleSpace solve (src/vmc/qgt/qgt.py:173-223).  Nothing here computes on the CPU: without
the CUDA library and a GPU it raises ``EngineUnavailable``.
"""
from __future__ import annotations

import ctypes as ct

import torch

from . import _abi
from ._lib import EngineUnavailable

__all__ = ["qr_pivoted", "sliced_gram", "sliced_gram_params"]


def _resolve_lib(lib, device):
    if lib is not None:
        return lib
    if device.type != "cuda":
        raise EngineUnavailable("the pivoted QR runs on a CUDA device; no CPU fallback exists")
    from ._lib import lib as _load

    return _load()


def sliced_gram(o: torch.Tensor, p: torch.Tensor, lib=None) -> torch.Tensor:
    """T[i, j] = sum_c [p[i, c] == p[j, c]] o[i, c] o[j, c] in FP64 for FP32 o and int8 p of shape
    (n, ncols): the sum over slices k of (o masked to slice k) (o masked to slice k)^T."""
    if o.dim() != 2 or p.shape != o.shape or o.dtype != torch.float32 or p.dtype != torch.int8:
        raise ValueError("sliced_gram takes FP32 o and int8 p of the same (n, ncols) shape")
    lib = _resolve_lib(lib, o.device)
    o = o.contiguous()
    p = p.contiguous()
    n, ncols = o.shape
    out = torch.empty((n, n), dtype=torch.float64, device=o.device)
    stream = ct.c_void_p(torch.cuda.current_stream(o.device).cuda_stream) if o.device.type == "cuda" else None
    st = lib.vmc_sliced_gram(stream, ct.c_void_p(o.data_ptr()), ct.c_void_p(p.data_ptr()), n, ncols,
                             max(ncols, 1), ct.c_void_p(out.data_ptr()))
    _abi.check(lib, st, "vmc_sliced_gram")
    return out


def sliced_gram_params(o: torch.Tensor, p: torch.Tensor, d: int = 2, lib=None) -> torch.Tensor:
    """S = O_exp^T O_exp in FP64 for FP32 o and int8 p of shape (n, ncols), O_exp the expanded Jacobian in
    slice order (column k * ncols + c is o[:, c] masked to slice k); d = 2 slices."""
    if o.dim() != 2 or p.shape != o.shape or o.dtype != torch.float32 or p.dtype != torch.int8:
        raise ValueError("sliced_gram_params takes FP32 o and int8 p of the same (n, ncols) shape")
    lib = _resolve_lib(lib, o.device)
    o = o.contiguous()
    p = p.contiguous()
    n, ncols = o.shape
    out = torch.empty((d * ncols, d * ncols), dtype=torch.float64, device=o.device)
    stream = ct.c_void_p(torch.cuda.current_stream(o.device).cuda_stream) if o.device.type == "cuda" else None
    st = lib.vmc_sliced_gram_params(stream, ct.c_void_p(o.data_ptr()), ct.c_void_p(p.data_ptr()), n, ncols,
                                    max(ncols, 1), int(d), ct.c_void_p(out.data_ptr()))
    _abi.check(lib, st, "vmc_sliced_gram_params")
    return out


def qr_pivoted(a: torch.Tensor, rhs: torch.Tensor | None = None, lib=None):
    """A P = Q R for a (m, n) matrix, in FP64 (complex128 for complex input).

    Returns ``(r, piv, qhb)``: ``r`` (k, n) upper trapezoidal with k = min(m, n) and R's
    diagonal following xLARFG's sign convention; ``piv`` (n,) int64, the original column of
    each column of R (so ``a[:, piv] = Q r``); ``qhb`` (k, nrhs) = the first k rows of Q^H rhs
    (None without ``rhs``; a 1-D rhs is one column).  Pivots follow xLAQP2, the unblocked
    xGEQP3: largest partial column norm first, the first column on ties.
    """
    if a.dim() != 2:
        raise ValueError("qr_pivoted factorises a 2-D matrix")
    lib = _resolve_lib(lib, a.device)
    m, n = a.shape
    cplx = a.is_complex() or (rhs is not None and rhs.is_complex())
    dt = torch.complex128 if cplx else torch.float64
    nrhs = 0 if rhs is None else (1 if rhs.dim() == 1 else int(rhs.shape[1]))
    k = min(m, n)
    dev = a.device
    # column-major m x (n + nrhs): row c of buf is column c of [a | rhs]
    buf = torch.empty((n + nrhs, max(m, 1)), dtype=dt, device=dev)
    buf[:n, :m] = a.to(dt).t()
    if nrhs:
        buf[n:, :m] = rhs.to(dt).reshape(m, nrhs).t()
    tau = torch.empty(max(k, 1), dtype=dt, device=dev)
    jpvt = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    ws = torch.empty(max(int(lib.vmc_qr_pivoted_workspace_size(n)), 8), dtype=torch.uint8, device=dev)
    stream = ct.c_void_p(torch.cuda.current_stream(dev).cuda_stream) if dev.type == "cuda" else None
    st = lib.vmc_qr_pivoted(stream, int(cplx), ct.c_void_p(buf.data_ptr()), max(m, 1), m, n, nrhs,
                            ct.c_void_p(tau.data_ptr()), ct.c_void_p(jpvt.data_ptr()), ct.c_void_p(ws.data_ptr()),
                            ws.numel())
    _abi.check(lib, st, "vmc_qr_pivoted")
    r = buf[:n, :k].t().triu()
    piv = jpvt[:n].long()
    qhb = buf[n:, :k].t() if nrhs else None
    return r, piv, qhb
