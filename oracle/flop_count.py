"""Algorithmic FLOP per sample of the PEPS evaluation path, counted on the oracle (test and
measurement infrastructure only).

Every einsum of one Monte-Carlo sweep (transition + estimate, one chain) is charged the FLOP count
numpy reports for the contraction path the call specifies (2 x multiply-adds), which is the
reference's own contraction order wherever it gives one.  SVD / QR / eigen-decompositions are not
counted.  Run from the repository root:

    python oracle/flop_count.py heis8x8_D4_chi16 heis8x8_D4_chi16_var
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from oracle import peps as oracle  # noqa: E402
from vmc_gb300.synthetic import WORKLOADS, initial_configs, random_tensors, uniform_stream  # noqa: E402


def sweep_flops(w) -> tuple[float, float]:
    orig = np.einsum
    total = [0.0]

    def counting(subscripts, *ops, optimize=False, **kw):
        _, info = np.einsum_path(subscripts, *ops, optimize=optimize if optimize else True)
        total[0] += float(re.search(r"Optimized FLOP count:\s*([0-9.eE+]+)", info).group(1))
        return orig(subscripts, *ops, optimize=optimize, **kw)

    T = [[t.astype(np.float32).astype(np.float64) for t in row]
         for row in random_tensors(w.shape, w.bond_dim, w.phys_dim, seed=0)]
    n_sites = w.shape[0] * w.shape[1]
    cfg = initial_configs(1, n_sites, w.phys_dim, seed=0).astype(np.int64)
    u = next(uniform_stream(1, n_sites, seed=0))
    strat = oracle.Variational(w.chi, 2) if w.strategy == "Variational" else oracle.ZipUp(w.chi)
    model = oracle.PEPS(T, w.shape, w.bond_dim, w.phys_dim, strategy=strat)
    init, trans, est = oracle.build_mc_kernels(model, w.operator())
    cache = init(T, cfg)
    np.einsum = counting
    try:
        c2, ctx = trans(T, cfg, u, cache)
        t_trans = total[0]
        est(T, c2, ctx)
    finally:
        np.einsum = orig
    return t_trans, total[0]


if __name__ == "__main__":
    for name in sys.argv[1:] or ["heis8x8_D4_chi16"]:
        t, tot = sweep_flops(WORKLOADS[name])
        print(f"{name}: transition {t / 1e6:.1f} MFLOP, estimate {(tot - t) / 1e6:.1f} MFLOP, "
              f"sweep {tot / 1e6:.1f} MFLOP")
