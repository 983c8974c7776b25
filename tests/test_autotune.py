"""Launch options and the autotuner on the host-emulation build: explicit options build plans,
invalid ones are refused, and tune / tuned_options time the candidates and keep the winner in the
cache file (the emulation's times mean nothing for a GPU; the code path is what is checked)."""
from __future__ import annotations

import ctypes as ct
import json

import numpy as np
import pytest
import torch

from oracle import peps as oracle
from tests.helpers import assert_parity, fp32, hamiltonian, make_case, oracle_sweep
from vmc_gb300 import _abi
from vmc_gb300.autotune import CANDIDATES, tune, tuned_options
from vmc_gb300.operators import transverse_field_ising
from vmc_gb300.engine import PEPSEngine
from vmc_gb300.lowering import pack_tensors


@pytest.mark.parametrize("options", CANDIDATES)
def test_every_candidate_matches_the_oracle(emu_lib, options):
    shape, D, chi = (4, 4), 3, 6
    H = hamiltonian("heisenberg", shape)
    T, cfg, u = make_case(shape, D, 4, seed=5)
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=H, device="cpu", lib=emu_lib, options=options)
    assert eng.options == options and eng.resident_chains > 0
    tens = torch.from_numpy(pack_tensors(T))
    c = torch.from_numpy(cfg.copy())
    res = eng.sweep(tens, c, torch.from_numpy(u), eng.init_cache(tens, c))
    c2, ctx, le = oracle_sweep(fp32(T), shape, D, "ZipUp", chi, H, cfg, u)
    assert np.array_equal(res.configs.numpy(), c2)
    e_ref = le.local_estimate
    assert_parity(np.abs(res.E.numpy() - e_ref) / np.maximum(1.0, np.abs(e_ref)), True)


def test_invalid_options_are_refused(emu_lib):
    shape = _abi.VmcShape(3, 3)
    plan = ct.c_void_p()
    for bad in [(48, -1, 0), (300, -1, 0), (128, -2, 0), (128, -1, 5), (128, -1, -1)]:
        o = _abi.VmcPlanOptions(*bad)
        assert emu_lib.vmc_peps_plan_ex(ct.byref(shape), 2, 4, 2, 0, 1, 2, ct.byref(o), ct.byref(plan)) == \
            _abi.VMC_ERR_INVALID
    with pytest.raises(ValueError):
        PEPSEngine((3, 3), 2, 4, device="cpu", lib=emu_lib, options="fastest")


def test_tune_and_cache(emu_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("VMC_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    entry = tune((3, 3), 2, 4, lib=emu_lib, candidates=CANDIDATES[:2])
    assert entry["options"] in CANDIDATES[:2] and len(entry["candidates"]) == 2
    data = json.loads((tmp_path / "tune.json").read_text())
    (key,) = data
    assert "3x3|D2|chi4" in key and data[key]["options"] == entry["options"]
    # a cached problem is not re-timed: the stored winner comes back
    data[key]["options"] = CANDIDATES[5]
    (tmp_path / "tune.json").write_text(json.dumps(data))
    assert tuned_options((3, 3), 2, 4, lib=emu_lib) == CANDIDATES[5]
    eng = PEPSEngine((3, 3), 2, 4, device="cpu", lib=emu_lib, options="auto")
    assert eng.options == CANDIDATES[5]


def test_mixed_tier_is_tuned_under_its_own_key(emu_lib, tmp_path, monkeypatch):
    from vmc_gb300.autotune import MIXED_CANDIDATES

    monkeypatch.setenv("VMC_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    entry = tune((3, 3), 2, 4, lib=emu_lib, candidates=MIXED_CANDIDATES[:2], precision="mixed")
    data = json.loads((tmp_path / "tune.json").read_text())
    (key,) = data
    assert key.endswith("|mixed") and data[key]["options"] == entry["options"]
    data[key]["options"] = MIXED_CANDIDATES[3]
    (tmp_path / "tune.json").write_text(json.dumps(data))
    eng = PEPSEngine((3, 3), 2, 4, device="cpu", lib=emu_lib, options="auto", precision="mixed")
    assert eng.options == dict(MIXED_CANDIDATES[3], precision="mixed")
    # the FP32 entry of the same problem is a different key: tuning it leaves the mixed one alone
    tune((3, 3), 2, 4, lib=emu_lib, candidates=CANDIDATES[:1])
    assert len(json.loads((tmp_path / "tune.json").read_text())) == 2


def test_shipped_table_is_the_fallback(emu_lib, tmp_path, monkeypatch):
    import vmc_gb300.autotune as at

    monkeypatch.setenv("VMC_AUTOTUNE_CACHE", str(tmp_path / "empty.json"))
    key = at._key(torch.device("cpu"), (3, 3), 2, 4, 2, "ZipUp", 2, "float32")
    shipped = tmp_path / "shipped.json"
    shipped.write_text(json.dumps({key: {"options": CANDIDATES[4], "samples_per_s": 1.0, "candidates": []}}))
    monkeypatch.setattr(at, "SHIPPED", shipped)
    assert tuned_options((3, 3), 2, 4, lib=emu_lib) == CANDIDATES[4]
    assert not (tmp_path / "empty.json").exists()  # nothing was tuned


def test_shipped_table_entries_are_valid_candidates(emu_lib):
    """Every winner in the shipped GB300 table is one of the candidates, and each candidate it lists was a
    valid plan configuration (vmc_peps_plan_ex accepts it)."""
    from vmc_gb300.autotune import SHIPPED

    from vmc_gb300.autotune import MIXED_CANDIDATES

    table = json.loads(SHIPPED.read_text())
    assert table
    shape = _abi.VmcShape(3, 3)
    for key, entry in table.items():
        mixed = key.endswith("|mixed")
        assert entry["options"] in (MIXED_CANDIDATES if mixed else CANDIDATES), key
        assert entry["samples_per_s"] == max(c["samples_per_s"] for c in entry["candidates"]), key
        for cand in entry["candidates"]:
            o = _abi.plan_options(dict(cand["options"], precision="mixed" if mixed else "fp32"))
            plan = ct.c_void_p()
            assert emu_lib.vmc_peps_plan_ex(ct.byref(shape), 2, 4, 2, 0, 1, 2, ct.byref(o), ct.byref(plan)) == \
                _abi.VMC_OK, (key, cand)
            emu_lib.vmc_plan_destroy(plan)


def test_shipped_options_lookup(monkeypatch):
    from vmc_gb300 import autotune

    assert autotune.shipped_options((8, 8), 4, 16, device="cpu") is None  # no table for the host build
    monkeypatch.setattr(autotune, "_device_name", lambda device: "NVIDIA GB300")
    table = json.loads(autotune.SHIPPED.read_text())
    key = autotune._key(torch.device("cpu"), (16, 16), 6, 48, 2, "ZipUp", 2, "float32")
    assert key.startswith("NVIDIA GB300|16x16|D6|chi48|d2|ZipUp|sweeps2|float32|H") and key.endswith("|fp32")
    want = table[key]["options"]
    assert autotune.shipped_options((16, 16), 6, 48, device="cpu") == want
    assert autotune.shipped_options((5, 7), 3, 9, device="cpu") is None


def test_the_cache_key_tells_hamiltonians_apart():
    """E_loc forms only the amplitudes a term's nonzero elements need, so a Heisenberg winner is not
    reused for a TFIM plan of the same lattice (and neither for another precision)."""
    from vmc_gb300 import autotune
    from vmc_gb300.operators import heisenberg, transverse_field_ising

    dev = torch.device("cpu")
    kh = autotune._key(dev, (4, 4), 3, 6, 2, "ZipUp", 2, "float32", heisenberg((4, 4)))
    kt = autotune._key(dev, (4, 4), 3, 6, 2, "ZipUp", 2, "float32", transverse_field_ising((4, 4)))
    assert kh != kt
    assert kh == autotune._key(dev, (4, 4), 3, 6, 2, "ZipUp", 2, "float32", None)  # default: Heisenberg
    assert kh != autotune._key(dev, (4, 4), 3, 6, 2, "ZipUp", 2, "float32", None, precision="mixed")


def test_unsupported_candidates_are_skipped(emu_lib, tmp_path, monkeypatch):
    """The tcgen05 tile policy exists for real FP32 plans only: tuning a complex plan skips it and says so."""
    monkeypatch.setenv("VMC_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    cands = [{"threads": 128, "smem_kb": -1, "tile_policy": 0}, {"threads": 128, "smem_kb": -1, "tile_policy": 4}]
    entry = tune((3, 3), 2, 4, dtype="complex64", operator=transverse_field_ising((3, 3)), lib=emu_lib,
                 candidates=cands, store=False)
    assert entry["options"] == cands[0] and entry["unsupported"] == [cands[1]]
    assert len(entry["candidates"]) == 1
