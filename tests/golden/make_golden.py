"""Generates tests/golden/*.npz from the FP64 oracle (run from the repository root:
``python tests/golden/make_golden.py``).

Inputs are the seeded synthetic workloads of vmc_gb300.synthetic (tensors
N(0,1)/sqrt(d D^4) from PCG64(seed), configurations from PCG64(seed+2),
uniforms from PCG64(seed+1)); each fixture stores those inputs and the
oracle's outputs of one Monte-Carlo sweep (transition + estimate).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import exact  # noqa: E402
from oracle import peps as oracle  # noqa: E402
from vmc_gb300.lowering import pack_tensors  # noqa: E402
from vmc_gb300.operators import heisenberg, transverse_field_ising  # noqa: E402
from vmc_gb300.synthetic import initial_configs, random_tensors, uniform_stream  # noqa: E402

CASES = {
    "heis3x3_D2_exact": dict(shape=(3, 3), D=2, chi=0, strategy="NoTruncation", model="heisenberg", n=8, seed=0),
    "tfim4x4_D2_chi4": dict(shape=(4, 4), D=2, chi=4, strategy="ZipUp", model="tfim", n=16, seed=0),
    "heis8x8_D4_chi16": dict(shape=(8, 8), D=4, chi=16, strategy="ZipUp", model="heisenberg", n=4, seed=0),
}


def make(name, shape, D, chi, strategy, model, n, seed):
    T = random_tensors(shape, D, seed=seed)
    T32 = [[t.astype(np.float32).astype(np.float64) for t in row] for row in T]  # the engine's input precision
    n_sites = shape[0] * shape[1]
    cfg = initial_configs(n, n_sites, seed=seed)
    u = next(uniform_stream(n, n_sites, seed=seed))
    H = heisenberg(shape) if model == "heisenberg" else transverse_field_ising(shape)
    strat = oracle.NoTruncation() if strategy == "NoTruncation" else oracle.ZipUp(chi)
    om = oracle.PEPS(T32, shape, D, strategy=strat)
    init, trans, est = oracle.build_mc_kernels(om, H)
    c2, ctx = trans(T32, cfg.astype(np.int64), u, init(T32, cfg.astype(np.int64)))
    _, le = est(T32, c2, ctx)
    out = dict(tensors=pack_tensors(T), configs_in=cfg, uniforms=u, configs_out=c2.astype(np.int32),
               amp=ctx.amp, margin=ctx.margins.min(axis=1), local_energy=le.local_estimate,
               log_derivatives=le.local_log_derivatives.astype(np.float32),
               shape=np.asarray(shape), bond_dim=D, chi=chi, model=np.asarray(model))
    if name == "tfim4x4_D2_chi4":
        # exact full-sum energy of the 4x4 TFIM state (all 2^16 configurations, no truncation)
        states = exact.all_configs(16)
        psi = exact.brute_amplitudes(T32, states, shape)
        hpsi = exact.apply_local_hamiltonian(psi, H.terms, shape, 2)
        out["exact_energy"] = float(np.dot(psi, hpsi) / np.dot(psi, psi))
    np.savez_compressed(Path(__file__).parent / f"{name}.npz", **out)


if __name__ == "__main__":
    for name, kw in CASES.items():
        make(name, **kw)
        print("wrote", name)
