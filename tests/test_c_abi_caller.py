"""The C ABI from plain C: tests/c_abi_caller.c is compiled as C99 against include/vmc_gb300.h (the header
is self-contained C) and linked with the host-emulation build of the library, which exports the same
symbols.  It creates a plan, attaches a Heisenberg operator, sizes its own workspace and evaluates
amplitudes, log-derivatives and local energies; the results equal the Python engine's bit for bit."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

from tests.conftest import build_emulation_library
from tests.helpers import hamiltonian, make_case
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_plain_c_caller_matches_the_python_engine(emu_lib, tmp_path):
    lib = build_emulation_library()
    exe = tmp_path / "c_abi_caller"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_abi_caller.c"), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True, capture_output=True, text=True)
    shape, D, chi, n = (4, 4), 3, 6, 5
    T, cfg, _ = make_case(shape, D, n, seed=12)
    packed = pack_tensors(T).astype(np.float32)
    packed.tofile(tmp_path / "tensors.f32")
    cfg.astype(np.int32).tofile(tmp_path / "configs.i32")
    res = subprocess.run([str(exe), *map(str, (shape[0], shape[1], D, chi, n)), str(tmp_path / "tensors.f32"),
                          str(tmp_path / "configs.i32"), str(tmp_path) + "/"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    np_sliced, ws_bytes = map(int, res.stdout.split())

    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device="cpu",
                     lib=emu_lib)
    tens, c = torch.from_numpy(packed), torch.from_numpy(cfg.astype(np.int32))
    la, sg, O = eng.amp_grad(tens, c)
    E = eng.local_energy(tens, c, la, sg)
    assert np_sliced == eng.n_params_sliced and ws_bytes == int(emu_lib.vmc_workspace_size(eng._plan, n))
    assert np.array_equal(np.fromfile(tmp_path / "logamp.f64"), la.numpy())
    assert np.array_equal(np.fromfile(tmp_path / "sign.f64"), sg.numpy())
    assert np.array_equal(np.fromfile(tmp_path / "O.f32", dtype=np.float32).reshape(n, -1), O.numpy())
    assert np.array_equal(np.fromfile(tmp_path / "E.f64"), E.numpy())
