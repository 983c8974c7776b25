"""The C ABI as declared in include/vmc_gb300.h: every declared function is exported by the sm_103a
library (built here by cross-compilation; loading it needs no GPU and nothing is called) and by the
host-emulation build, and has a ctypes prototype in vmc_gb300._abi."""
from __future__ import annotations

import ctypes as ct
import re
import shutil
from pathlib import Path

import pytest

from vmc_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "vmc_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(vmc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_documented_entry_points():
    names = declared_functions()
    for must in ("vmc_peps_plan", "vmc_peps_plan_set_operator", "vmc_plan_destroy", "vmc_workspace_size",
                 "vmc_cache_size", "vmc_peps_init_cache", "vmc_peps_sweep", "vmc_peps_amp_grad",
                 "vmc_peps_local_energy", "vmc_status_string"):
        assert must in names


def test_every_declared_function_has_a_ctypes_prototype():
    missing = [n for n in declared_functions() if n not in _abi.SIGNATURES]
    assert not missing, missing


def test_emulation_build_exports_every_declared_function(emu_lib):
    for name in declared_functions():
        assert hasattr(emu_lib, name), name


def test_cuda_library_loads_and_exports_every_declared_function():
    from vmc_gb300._lib import library_path
    from vmc_gb300.build import build_native

    path = Path(library_path())
    if not path.exists():
        if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
            pytest.skip("no nvcc to build the sm_103a library")
        build_native()
    lib = ct.CDLL(str(path))
    for name in declared_functions():
        assert hasattr(lib, name), name
