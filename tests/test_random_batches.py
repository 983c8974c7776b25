"""Randomised uneven batches in the host emulation: 1-8 jobs of random kinds (init-cache, sweep, amp + O_k,
local energy) on random plans (lattices, bond dimensions, strategies, chain counts including 0), one
precision tier per batch, every workspace layout: each job's outputs are the bits of its single call."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import hamiltonian, make_case
from tests.test_batch_emulation import _assert_same_bits
from vmc_gb300.engine import PEPSBatch, PEPSEngine
from vmc_gb300.lowering import pack_tensors


def _job(emu_lib, rng, seed, precision):
    shape = (int(rng.integers(2, 5)), int(rng.integers(2, 5)))
    D = int(rng.integers(2, 4))
    strategies = ["ZipUp", "NoTruncation", "DensityMatrix"] + ([] if precision == "mixed" else ["Variational"])
    strategy = str(rng.choice(strategies))
    chi = 64 if strategy == "NoTruncation" else int(rng.integers(2, 7))
    if strategy == "DensityMatrix":
        chi = min(chi, D)
    n = int(rng.integers(0, 5))
    kind = str(rng.choice(["sweep", "amp_grad", "energy", "init"]))
    full = bool(rng.random() < 0.3)
    H = hamiltonian(str(rng.choice(["heisenberg", "tfim"])), shape)
    T, cfg, u = make_case(shape, D, max(n, 1), seed=seed)
    eng = PEPSEngine(shape, D, chi, 2, strategy, operator=H, device="cpu", lib=emu_lib,
                     options={"precision": precision})
    tens = torch.from_numpy(pack_tensors(T))
    c, ut = torch.from_numpy(cfg[:n].copy()), torch.from_numpy(u[:n].copy())
    if kind == "sweep":
        cache = eng.init_cache(tens, c.clone())
        job = eng.sweep_job(tens, c.clone(), ut, cache.clone(), full_gradient=full)
        return job, ("sweep", eng.sweep(tens, c.clone(), ut, cache, full_gradient=full))
    if kind == "amp_grad":
        return eng.amp_grad_job(tens, c, full_gradient=full), ("amp", eng.amp_grad(tens, c, full_gradient=full))
    if kind == "energy":
        la, sg, _ = eng.amp_grad(tens, c, want_O=False)
        return eng.local_energy_job(tens, c, la, sg), ("energy", eng.local_energy(tens, c, la, sg))
    return eng.init_cache_job(tens, c.clone()), ("init", (eng, tens, c, ut, eng.init_cache(tens, c.clone())))


@pytest.mark.parametrize("seed", range(16))
def test_random_batch_matches_single_calls(emu_lib, seed):
    rng = np.random.default_rng(3000 + seed)
    precision = "mixed" if rng.random() < 0.3 else "fp32"
    layout = str(rng.choice(["auto", "plan", "slot"]))
    pairs = [_job(emu_lib, rng, 100 * seed + j, precision) for j in range(int(rng.integers(1, 9)))]
    batch = PEPSBatch()
    outs = batch.run([job for job, _ in pairs], layout=layout)
    assert batch.status() == 0
    for (job, (kind, ref)), out in zip(pairs, outs):
        if kind == "sweep":
            if ref.configs.shape[0]:
                _assert_same_bits(ref, out)
            else:
                assert out.configs.shape[0] == 0 and out.E.numel() == 0
        elif kind == "amp":
            la, sg, O = ref
            assert torch.equal(out.logamp, la) and torch.equal(out.sign, sg) and torch.equal(out.O, O)
        elif kind == "energy":
            assert torch.equal(out.E, ref)
        else:
            eng, tens, c, ut, cache = ref
            if c.shape[0]:
                # caches may differ in padding nothing reads: the next sweep from either gives the same bits
                _assert_same_bits(eng.sweep(tens, c.clone(), ut, cache.clone()),
                                  eng.sweep(tens, c.clone(), ut, job.cache.clone()))
