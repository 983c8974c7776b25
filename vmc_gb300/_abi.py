"""ctypes declarations of the C ABI in include/vmc_gb300.h.

``bind(path)`` loads a shared library exporting that ABI and attaches the
argument/return types of every entry point.  The package binds the CUDA
build (``vmc_gb300/_native/libvmc_gb300.so``) through ``vmc_gb300._lib``.
"""
from __future__ import annotations

import ctypes as ct

VMC_OK = 0
VMC_ERR_INVALID = 1
VMC_ERR_UNSUPPORTED = 2
VMC_ERR_WORKSPACE = 3
VMC_ERR_CUDA = 4
VMC_ERR_NONFINITE = 5
VMC_ERR_TIMEOUT = 6
VMC_ERR_SCRATCH = 7

VMC_DTYPE_F32 = 0
VMC_DTYPE_C64 = 1

VMC_PRECISION_FP32 = 0
VMC_PRECISION_MIXED = 1

VMC_STRATEGY_NO_TRUNCATION = 0
VMC_STRATEGY_ZIP_UP = 1
VMC_STRATEGY_DENSITY_MATRIX = 2
VMC_STRATEGY_VARIATIONAL = 3

VMC_DEV_NONFINITE = 1
VMC_DEV_TIMEOUT = 2

VMC_JOB_INIT_CACHE = 0
VMC_JOB_SWEEP = 1
VMC_JOB_AMP_GRAD = 2
VMC_JOB_LOCAL_ENERGY = 3
VMC_MAX_BATCH_JOBS = 16
VMC_BATCH_LAYOUT_AUTO = -1
VMC_BATCH_LAYOUT_PLAN = 0
VMC_BATCH_LAYOUT_SLOT = 1


class VmcShape(ct.Structure):
    _fields_ = [("n_rows", ct.c_int), ("n_cols", ct.c_int)]


_P = ct.c_void_p
_I = ct.c_int
_SZ = ct.c_size_t


class VmcPlanOptions(ct.Structure):
    """vmc_plan_options: a plan's launch configuration and arithmetic."""
    _fields_ = [("threads", _I), ("smem_kb", _I), ("tile_policy", _I), ("precision", _I), ("trunc_method", _I),
                ("vchunk", _I), ("vert_smem", _I)]


PRECISIONS = {"fp32": VMC_PRECISION_FP32, "mixed": VMC_PRECISION_MIXED}
TRUNC_METHODS = {"gram": 0, "jacobi": 1}


def plan_options(options) -> VmcPlanOptions:
    """A vmc_plan_options from a dict (threads, smem_kb, tile_policy, precision, trunc_method, vchunk,
    vert_smem); precision is "fp32" / "mixed" (or 0 / 1), trunc_method "gram" / "jacobi" (or 0 / 1)."""
    o = dict(options)
    prec = o.get("precision", VMC_PRECISION_FP32)
    prec = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
    tm = o.get("trunc_method", 0)
    tm = TRUNC_METHODS[tm] if isinstance(tm, str) else int(tm)
    return VmcPlanOptions(int(o.get("threads", 0)), int(o.get("smem_kb", -1)), int(o.get("tile_policy", 0)), prec,
                          tm, int(o.get("vchunk", 0)), int(o.get("vert_smem", 0)))


class VmcPepsJob(ct.Structure):
    """vmc_peps_job: one call of an uneven batch."""
    _fields_ = [("plan", _P), ("kind", _I), ("n_chains", _I), ("full_gradient", _I), ("tensors", _P),
                ("configs", _P), ("uniforms", _P), ("deltas", _P), ("cache", _P), ("out_O", _P), ("out_p", _P),
                ("out_E", _P), ("logamp", _P), ("sign", _P), ("out_margin", _P), ("out_gap", _P)]


# name -> (restype, argtypes)
SIGNATURES = {
    "vmc_version": (ct.c_char_p, []),
    "vmc_status_string": (ct.c_char_p, [_I]),
    "vmc_peps_plan": (_I, [ct.POINTER(VmcShape), _I, _I, _I, _I, _I, _I, ct.POINTER(_P)]),
    "vmc_peps_plan_ex": (_I, [ct.POINTER(VmcShape), _I, _I, _I, _I, _I, _I, ct.POINTER(VmcPlanOptions), ct.POINTER(_P)]),
    "vmc_gi_plan": (_I, [ct.POINTER(VmcShape), _I, _I, _I, _I, _I, _I, ct.POINTER(VmcPlanOptions), ct.POINTER(_P)]),
    "vmc_gi_set_operator": (_I, [_P, _P, _P, _P]),
    "vmc_peps_plan_set_operator": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _P]),
    "vmc_plan_destroy": (None, [_P]),
    "vmc_peps_n_params_sliced": (ct.c_int64, [_P]),
    "vmc_peps_n_params_full": (ct.c_int64, [_P]),
    "vmc_plan_resident_ctas": (_I, [_P]),
    "vmc_cache_size": (_SZ, [_P, _I]),
    "vmc_workspace_size": (_SZ, [_P, _I]),
    "vmc_peps_init_cache": (_I, [_P, _P, _P, _P, _I, _P, _P, _SZ, _P]),
    "vmc_peps_sweep": (_I, [_P, _P, _P, _P, _P, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "vmc_sweep_recompute_workspace_size": (_SZ, [_P, _I]),
    "vmc_peps_sweep_recompute": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "vmc_peps_amp_grad": (_I, [_P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _SZ, _P]),
    "vmc_peps_amp_grad_noalloc": (_I, [_P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P]),
    "vmc_peps_vjp": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _SZ, _P]),
    "vmc_peps_local_energy": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _P, _SZ, _P]),
    "vmc_batch_workspace_size": (_SZ, [ct.POINTER(VmcPepsJob), _I]),
    "vmc_peps_batch": (_I, [ct.POINTER(VmcPepsJob), _I, _P, _P, _SZ, _P]),
    "vmc_batch_workspace_size_ex": (_SZ, [ct.POINTER(VmcPepsJob), _I, _I]),
    "vmc_peps_batch_ex": (_I, [ct.POINTER(VmcPepsJob), _I, _I, _P, _P, _SZ, _P]),
    "vmc_uniforms": (_I, [_P, _P, ct.c_int64, ct.c_uint64, _P]),
    "vmc_qr_pivoted_workspace_size": (_SZ, [_I]),
    "vmc_qr_pivoted": (_I, [_P, _I, _P, ct.c_int64, _I, _I, _I, _P, _P, _P, _SZ]),
    "vmc_sliced_gram": (_I, [_P, _P, _P, _I, _I, ct.c_int64, _P]),
    "vmc_sliced_gram_params": (_I, [_P, _P, _P, _I, _I, ct.c_int64, _I, _P]),
}


def bind(path: str) -> ct.CDLL:
    lib = ct.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class VmcError(RuntimeError):
    """A C-ABI call returned a non-zero vmc_status."""

    def __init__(self, status: int, where: str, lib=None):
        msg = lib.vmc_status_string(status).decode() if lib is not None else str(status)
        super().__init__(f"{where}: vmc_status {status} ({msg})")
        self.status = status


def check(lib, status: int, where: str) -> None:
    if status != VMC_OK:
        raise VmcError(status, where, lib)
