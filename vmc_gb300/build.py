"""Build recipe for the sm_103a engine library (in-tree, no cmake).

``build_native()`` compiles ``vmc_gb300/csrc/*.cu`` with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` into
``vmc_gb300/_native/libvmc_gb300.so``.  Translation units compile in
parallel; a unit is skipped when its object is newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
NATIVE = PKG / "_native"
INCLUDE = PKG.parent / "include"
LIB_NAME = "libvmc_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the vmc_gb300 engine needs the CUDA 13 toolkit to build")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _compile(nvcc: str, src: Path, obj: Path, extra) -> None:
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-I", str(INCLUDE), "-c", str(src), "-o", str(obj), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")


def build_native(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    nvcc = nvcc_path()
    NATIVE.mkdir(exist_ok=True)
    lib = NATIVE / LIB_NAME
    srcs = _sources()
    hdr_time = _newest(_headers())
    jobs = []
    for src in srcs:
        obj = NATIVE / (src.stem + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_time):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            list(ex.map(lambda j: _compile(nvcc, j[0], j[1], list(extra_flags)), jobs))
    objs = [NATIVE / (s.stem + ".o") for s in srcs]
    if force or jobs or not lib.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build_native(verbose=True)
