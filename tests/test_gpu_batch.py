"""Uneven batches on the GPU: the four lattices and bond dimensions of the uneven-batch workload
(6x6 D4 chi16, 8x8 D5 chi25, 12x12 D6 chi36, 16x16 D6 chi48) in ONE persistent launch give, chain for
chain, the bits of their single launches; and a batch captured in a CUDA graph replays to the bits of
the same batch run eagerly."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import hamiltonian
from vmc_gb300.engine import PEPSBatch, PEPSEngine
from vmc_gb300.lowering import pack_tensors
from vmc_gb300.synthetic import initial_configs, random_tensors

pytestmark = pytest.mark.gpu

# (shape, D, chi, chains): the uneven-batch workload's shapes, a few chains of the large ones
UNEVEN = [((6, 6), 4, 16, 96), ((8, 8), 5, 25, 24), ((12, 12), 6, 36, 3), ((16, 16), 6, 48, 2)]


def _case(dev, shape, D, chi, n, seed):
    eng = PEPSEngine(shape, D, chi, 2, "ZipUp", operator=hamiltonian("heisenberg", shape), device=dev)
    tens = torch.from_numpy(pack_tensors(random_tensors(shape, D, seed=seed))).to(dev)
    n_sites = shape[0] * shape[1]
    cfg = torch.from_numpy(initial_configs(n, n_sites, seed=seed)).to(dev)
    u = torch.from_numpy(np.random.default_rng(seed + 100).random((n, n_sites))).to(dev)
    return eng, tens, cfg, u


def _same_bits(a, b):
    for k in ("configs", "O", "p", "E", "logamp", "sign", "margin", "gap"):
        x, y = getattr(a, k), getattr(b, k)
        assert (x is None) == (y is None), k
        if x is not None:
            assert torch.equal(x.contiguous().view(torch.uint8), y.contiguous().view(torch.uint8)), k


def test_uneven_shapes_in_one_launch_match_single_launches(cuda_device):
    cases = [_case(cuda_device, *spec, seed=5 + i) for i, spec in enumerate(UNEVEN)]
    singles, jobs = [], []
    for eng, tens, cfg, u in cases:
        cache = eng.init_cache(tens, cfg.clone())
        cache_b = cache.clone()
        singles.append(eng.sweep(tens, cfg.clone(), u, cache))
        jobs.append(eng.sweep_job(tens, cfg.clone(), u, cache_b))
    batch = PEPSBatch()
    outs = batch.run(jobs)
    torch.cuda.synchronize()
    batch.raise_on_status()
    for eng, _, _, _ in cases:
        eng.raise_on_status()
    for ref, out in zip(singles, outs):
        assert torch.isfinite(out.E).all() and torch.isfinite(out.logamp).all()
        _same_bits(ref, out)


def test_batch_replays_from_a_cuda_graph(cuda_device):
    cases = [_case(cuda_device, *spec, seed=30 + i) for i, spec in enumerate(UNEVEN[:2])]
    (e1, t1, c1, u1), (e2, t2, c2, _) = cases
    cache1 = e1.init_cache(t1, c1.clone())
    la2, sg2, _ = e2.amp_grad(t2, c2, want_O=False)
    start_cfg, start_cache = c1.clone(), cache1.clone()
    jobs = [e1.sweep_job(t1, c1, u1, cache1), e2.amp_grad_job(t2, c2), e2.local_energy_job(t2, c2, la2, sg2)]
    batch = PEPSBatch()
    batch.run(jobs)  # sizes the workspace outside the capture
    torch.cuda.synchronize()
    eager = [x.clone() for x in (jobs[0].out.configs, jobs[0].out.O, jobs[0].out.E, jobs[0].out.logamp,
                                 jobs[1].out.O, jobs[1].out.logamp, jobs[2].out.E)]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        batch.run(jobs)
    # the sweep job updates its chains in place: restart them from the same state, then replay
    for out in (jobs[1].out.O, jobs[2].out.E):
        out.zero_()
    c1.copy_(start_cfg)
    cache1.copy_(start_cache)
    g.replay()
    torch.cuda.synchronize()
    batch.raise_on_status()
    replayed = [jobs[0].out.configs, jobs[0].out.O, jobs[0].out.E, jobs[0].out.logamp, jobs[1].out.O,
                jobs[1].out.logamp, jobs[2].out.E]
    for a, b in zip(eager, replayed):
        assert torch.equal(a.view(torch.uint8), b.contiguous().view(torch.uint8))


def test_recomputing_sweep_matches_cached_sweep(cuda_device):
    """12x12 D6 chi36: the sweep that recomputes the bottom environments in the launch (memory per
    resident CTA) gives the bits of init_cache + sweep (memory per chain)."""
    eng, tens, cfg, u = _case(cuda_device, (12, 12), 6, 36, 6, seed=41)
    ref = eng.sweep(tens, cfg.clone(), u, eng.init_cache(tens, cfg.clone()))
    out = eng.sweep(tens, cfg.clone(), u, None)
    torch.cuda.synchronize()
    eng.raise_on_status()
    _same_bits(ref, out)
    per_chain = eng.cache_bytes(4096)
    per_cta = int(eng.lib.vmc_sweep_recompute_workspace_size(eng._plan, 4096)) - \
        int(eng.lib.vmc_workspace_size(eng._plan, 4096))
    assert per_cta < per_chain / 4  # 608 resident CTAs instead of 4096 chains
