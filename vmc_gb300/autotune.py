"""Launch-configuration autotuner: per (lattice, D, chi, d, dtype, strategy, Hamiltonian structure), the CTA
size, shared-memory budget and GEMM register-tile policy of the fused FP32 kernel that give the most samples/s
on this GPU.

``tune`` builds one plan per candidate (``vmc_peps_plan_ex``), times full sweeps on seeded synthetic
inputs -- whole waves of chains, after a warm-up sweep -- and records every candidate's rate with the
winner in a JSON cache keyed by GPU name and problem (``$VMC_AUTOTUNE_CACHE``, default
``~/.cache/vmc_gb300/autotune.json``).  ``tuned_options`` returns the cached winner -- from that cache, else
from the table this package ships (``tuned_gb300.json``, made by ``python -m vmc_gb300.autotune`` on a
GB300 for the standard workloads) -- tuning first when the problem is in neither.  All candidates compute the same quantities and differ only in FP32 rounding
order; each is covered by the parity tests.  The cache is the only process-wide mutable state of the
package and is guarded by a lock.
"""
from __future__ import annotations

import hashlib
import json
import os
import threading
from pathlib import Path

import numpy as np
import torch

from . import _abi

__all__ = ["CANDIDATES", "MIXED_CANDIDATES", "cache_path", "shipped_options", "tune", "tuned_options"]

# (threads, smem_kb, tile_policy); smem_kb -1 = the 52 KB default, 0 = all buffers in the slot
CANDIDATES = [
    {"threads": 128, "smem_kb": -1, "tile_policy": 0},
    {"threads": 128, "smem_kb": -1, "tile_policy": 1},
    {"threads": 128, "smem_kb": -1, "tile_policy": 2},
    {"threads": 128, "smem_kb": 0, "tile_policy": 0},
    {"threads": 256, "smem_kb": -1, "tile_policy": 0},
    {"threads": 256, "smem_kb": -1, "tile_policy": 2},
    {"threads": 64, "smem_kb": -1, "tile_policy": 0},
    {"threads": 64, "smem_kb": 0, "tile_policy": 0},
    {"threads": 64, "smem_kb": 0, "tile_policy": 2},
    {"threads": 64, "smem_kb": 20, "tile_policy": 0},
    {"threads": 128, "smem_kb": -1, "tile_policy": 3},
    {"threads": 256, "smem_kb": -1, "tile_policy": 3},
    {"threads": 128, "smem_kb": -1, "tile_policy": 4},
    {"threads": 256, "smem_kb": -1, "tile_policy": 4},
]

# the mixed-precision tier (FFMA tiles and the Gram eigensolver only); its FP64 arena is twice the FP32
# one, smem_kb -1 = its 52 KB default (the eigensolver's working set at 8x8 D4), up to 200 KB
MIXED_CANDIDATES = [
    {"threads": 128, "smem_kb": -1, "tile_policy": 0},
    {"threads": 128, "smem_kb": 0, "tile_policy": 0},
    {"threads": 128, "smem_kb": 110, "tile_policy": 0},
    {"threads": 128, "smem_kb": 200, "tile_policy": 0},
    {"threads": 128, "smem_kb": -1, "tile_policy": 1},
    {"threads": 128, "smem_kb": -1, "tile_policy": 2},
    {"threads": 256, "smem_kb": -1, "tile_policy": 0},
    {"threads": 256, "smem_kb": 110, "tile_policy": 0},
    {"threads": 64, "smem_kb": -1, "tile_policy": 0},
    {"threads": 64, "smem_kb": 0, "tile_policy": 0},
]

_LOCK = threading.Lock()


def cache_path() -> Path:
    p = os.environ.get("VMC_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "vmc_gb300" / "autotune.json"


def _device_name(device) -> str:
    device = torch.device(device)
    if device.type == "cuda":
        return torch.cuda.get_device_name(device)
    return "host-emulation"


def operator_tag(operator, shape, phys_dim=2, complex_elements=False) -> str:
    """Fingerprint of a Hamiltonian's nonzero structure on this lattice: which sites and bonds carry
    terms and which operator elements are nonzero.  The estimate forms only the amplitudes a term's
    nonzero elements need, so its cost -- and the launch configuration that wins -- depends on it."""
    from .lowering import lower_operator
    from .operators import heisenberg

    op = operator if operator is not None else heisenberg(shape)
    lo = lower_operator(op, shape, phys_dim, complex_elements=complex_elements)
    h = hashlib.sha1()
    for a in (lo.onesite, lo.horiz, lo.vert):
        h.update(np.ascontiguousarray(np.asarray(a) != 0).tobytes())
    for a in (lo.onesite_mask, lo.horiz_mask, lo.vert_mask):
        h.update(np.ascontiguousarray(np.asarray(a, dtype=np.int32)).tobytes())
    h.update(str(int(lo.n_diag)).encode())
    return h.hexdigest()[:10]


def _key(device, shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, operator=None, precision="fp32") -> str:
    tag = operator_tag(operator, shape, phys_dim, dtype == "complex64")
    return (f"{_device_name(device)}|{shape[0]}x{shape[1]}|D{bond_dim}|chi{chi}|d{phys_dim}|{strategy}"
            f"|sweeps{n_sweeps}|{dtype}|H{tag}|{precision}")


SHIPPED = Path(__file__).resolve().parent / "tuned_gb300.json"


def _load(path=None) -> dict:
    p = cache_path() if path is None else Path(path)
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, entry: dict) -> None:
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    data = _load()
    data[key] = entry
    tmp = p.with_suffix(f".{os.getpid()}.tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    tmp.replace(p)


def _time_candidate(options, shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, operator, device, lib,
                    waves, reps, seed=0, n_chains=None, precision="fp32"):
    from .engine import PEPSEngine
    from .lowering import pack_tensors
    from .synthetic import initial_configs, random_tensors

    eng = PEPSEngine(shape, bond_dim, chi, phys_dim, strategy, n_sweeps, operator=operator, device=device,
                     lib=lib, dtype=dtype, options=options, precision=precision)
    n = int(n_chains) if n_chains else max(1, waves * eng.resident_chains)
    n_sites = shape[0] * shape[1]
    T = random_tensors(shape, bond_dim, phys_dim=phys_dim, seed=seed,
                       dtype=np.complex128 if dtype == "complex64" else np.float64)
    dev = eng.device
    tens = torch.from_numpy(pack_tensors(T)).to(dev)
    cfg = torch.from_numpy(initial_configs(n, n_sites, phys_dim, seed=seed)).to(dev)
    rng = np.random.default_rng(seed + 1)
    u = [torch.from_numpy(rng.random((n, n_sites))).to(dev) for _ in range(reps + 1)]
    deltas = None
    if phys_dim > 2:
        deltas = torch.from_numpy(rng.integers(1, phys_dim, (n, n_sites)).astype(np.int32)).to(dev)
    cache = eng.init_cache(tens, cfg)
    out = eng.sweep(tens, cfg, u[0], cache, deltas=deltas)
    if dev.type == "cuda":
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for i in range(reps):
            out = eng.sweep(tens, cfg, u[i + 1], cache, deltas=deltas, out=out)
        b.record()
        torch.cuda.synchronize(dev)
        seconds = a.elapsed_time(b) / 1e3
    else:  # host-emulation build: exercises the code path; its times mean nothing for a GPU
        import time

        t0 = time.perf_counter()
        for i in range(reps):
            out = eng.sweep(tens, cfg, u[i + 1], cache, deltas=deltas, out=out)
        seconds = time.perf_counter() - t0
    eng.raise_on_status()
    return n * reps / seconds


def tune(shape, bond_dim, chi, phys_dim=2, strategy="ZipUp", n_sweeps=2, dtype="float32", operator=None,
         device=None, lib=None, candidates=None, waves=1, reps=1, store=True, n_chains=None,
         precision="fp32") -> dict:
    """Time every candidate on this problem; returns {"options", "samples_per_s", "candidates"}.
    ``precision``: "fp32" or "mixed" (the candidates default to ``MIXED_CANDIDATES`` for the latter).
    ``n_chains``: chains per timed sweep (the run's own count); None times ``waves`` full waves of each
    candidate's resident chains.  One wave favours configurations whose extra resident chains only pay
    off within a wave, so a table meant for a given run size is best tuned at that size."""
    from .operators import heisenberg

    shape = (int(shape[0]), int(shape[1]))
    device = torch.device(device if device is not None else ("cuda" if lib is None else "cpu"))
    if operator is None and phys_dim != 2:
        raise ValueError("tuning a d != 2 plan needs its operator")
    op = operator if operator is not None else heisenberg(shape)
    results, skipped = [], []
    for cand in candidates or (MIXED_CANDIDATES if precision == "mixed" else CANDIDATES):
        try:
            rate = _time_candidate(cand, shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, op, device,
                                   lib, waves, reps, n_chains=n_chains, precision=precision)
        except _abi.VmcError as e:
            # a configuration the plan does not support for this problem (the tcgen05 tiles on complex
            # elements, say) is not a candidate here
            if e.status != _abi.VMC_ERR_UNSUPPORTED:
                raise
            skipped.append(dict(cand))
            continue
        results.append({"options": dict(cand), "samples_per_s": rate})
    if not results:
        raise ValueError("no launch configuration supports this problem")
    best = max(results, key=lambda r: r["samples_per_s"])
    entry = {"options": best["options"], "samples_per_s": best["samples_per_s"], "candidates": results}
    if skipped:
        entry["unsupported"] = skipped
    if store:
        with _LOCK:
            _store(_key(device, shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, op, precision), entry)
    return entry


def shipped_options(shape, bond_dim, chi, phys_dim=2, strategy="ZipUp", n_sweeps=2, dtype="float32",
                    device=None, operator=None, precision="fp32"):
    """The winner the shipped table holds for this problem on this GPU, or None (no tuning, no local cache)."""
    device = torch.device(device if device is not None else "cuda")
    hit = _load(SHIPPED).get(_key(device, (int(shape[0]), int(shape[1])), bond_dim, chi, phys_dim, strategy, n_sweeps,
                                  dtype, operator, precision))
    return dict(hit["options"]) if hit else None


def tuned_options(shape, bond_dim, chi, phys_dim=2, strategy="ZipUp", n_sweeps=2, dtype="float32", operator=None,
                  device=None, lib=None, precision="fp32") -> dict:
    """The cached winner for this problem on this GPU, tuning it first when it is not cached."""
    shape = (int(shape[0]), int(shape[1]))
    device = torch.device(device if device is not None else ("cuda" if lib is None else "cpu"))
    key = _key(device, shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, operator, precision)
    with _LOCK:
        hit = _load().get(key)
        if hit is None:
            hit = _load(SHIPPED).get(key)
    if hit is not None:
        return dict(hit["options"])
    return dict(tune(shape, bond_dim, chi, phys_dim, strategy, n_sweeps, dtype, operator, device, lib,
                     precision=precision)["options"])


def main(argv=None) -> None:
    """Tune the standard workloads on this GPU and write their entries to a JSON table."""
    import argparse

    from .synthetic import WORKLOADS

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--workloads", nargs="*", default=["heis6x6_D4_chi16", "heis8x8_D4_chi16", "heis8x8_D4_chi16_var",
                                                       "heis8x8_D5_chi25", "tfim10x10_D4_chi16_c64",
                                                       "heis12x12_D6_chi36", "heis16x16_D6_chi48"])
    ap.add_argument("--out", default=str(SHIPPED))
    ap.add_argument("--precision", choices=["fp32", "mixed"], default="fp32")
    ap.add_argument("--chains", type=int, default=-1,
                    help="chains per timed sweep: -1 the workload's own count when one sweep of it stays under "
                         "about 20 s, else one wave; 0 one wave; N > 0 exactly N")
    args = ap.parse_args(argv)
    table = _load(args.out)
    dev = torch.device("cuda")
    for name in args.workloads:
        w = WORKLOADS[name]
        n = args.chains
        if n < 0:
            # about 2.4 TFLOP/s of algorithmic work is what one GB300 sustains on these plans
            n = w.n_chains if (w.flops_per_sample() or 0) * w.n_chains < 20 * 2.4e12 else 0
        entry = tune(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, 2, w.dtype, w.operator(), dev, store=False,
                     n_chains=n or None, precision=args.precision)
        entry["chains"] = n or "one wave"
        table[_key(dev, w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, 2, w.dtype, w.operator(),
                   args.precision)] = entry
        print(json.dumps({"workload": name, **entry}), flush=True)
        Path(args.out).write_text(json.dumps(table, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
