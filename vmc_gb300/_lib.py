"""Loads the sm_103a engine library.  There is no CPU fallback: if the CUDA
build is missing or no GPU is visible, every engine call raises."""
from __future__ import annotations

import threading

from . import _abi
from .build import LIB_NAME, NATIVE

_lock = threading.Lock()
_lib = None


class EngineUnavailable(RuntimeError):
    pass


def lib():
    """The bound CUDA library (built by ``vmc_gb300.build.build_native``)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = NATIVE / LIB_NAME
            if not path.exists():
                raise EngineUnavailable(
                    f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                    "(or vmc_gb300.build.build_native()) on a machine with nvcc")
            _lib = _abi.bind(str(path))
    return _lib


def library_path() -> str:
    return str(NATIVE / LIB_NAME)
