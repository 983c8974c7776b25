"""Shared fixtures for the vmc_gb300 test suite.

Markers:
  gpu  -- needs a CUDA GPU and the sm_103a library (run with -m gpu);
  slow -- long CPU tests (deselect with -m "not slow").

The CPU suite also checks the engine's device code through its host-emulation
build (tests/_emu/libvmc_emu.so, compiled here with g++ from
vmc_gb300/csrc/*.cu with -DVMC_HOST_EMULATION: every CTA runs with
one thread).  That library is test infrastructure only; the package never
loads it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

EMU_DIR = Path(__file__).resolve().parent / "_emu"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU with the sm_103a engine library")
    config.addinivalue_line("markers", "slow: long-running test")


def _newest(paths):
    return max(p.stat().st_mtime for p in paths)


def build_emulation_library() -> Path:
    srcs = sorted((ROOT / "vmc_gb300" / "csrc").glob("*.cu"))
    deps = list((ROOT / "vmc_gb300" / "csrc").glob("*.cuh")) + srcs + [ROOT / "include" / "vmc_gb300.h"]
    EMU_DIR.mkdir(exist_ok=True)
    out = EMU_DIR / "libvmc_emu.so"
    if not out.exists() or out.stat().st_mtime < _newest(deps):
        tmp = out.with_suffix(f".{os.getpid()}.tmp")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DVMC_HOST_EMULATION", "-x", "c++", *map(str, srcs),
               "-o", str(tmp)]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        tmp.replace(out)
    return out


@pytest.fixture(scope="session")
def emu_lib():
    from vmc_gb300 import _abi

    return _abi.bind(str(build_emulation_library()))


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
