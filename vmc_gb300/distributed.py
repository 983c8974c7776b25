"""Chain sharding and SR reductions across ranks (one process per GPU).

Chains are independent (the reference vmaps them, src/vmc/core/sampling.py:38),
so each rank samples its own shard with no collective on the data path.  The
only exchange is in the SR solve.  ``TDVPDriver(process_group=...)`` gathers the
shards' sample histories along the chain axis (``gather_chain_axis``), so every
rank holds the single-process arrays in the single-process order and solves the
same FP64 system: one all-gather of N x P_sliced values per derivative call,
against P_full^2 for an all-reduce of S (at 8x8, D=4: 4096 x 10,816 FP32
against 21,632^2 FP64).  ``parameter_space_qgt`` (one all-reduce of
[sum O, O^H O]) and ``gather_jacobian`` remain for callers that hold only the
sliced Jacobian of their shard.
"""
from __future__ import annotations

import torch
import torch.distributed as dist

from .qgt import SlicedJacobian, iter_sliced_blocks

__all__ = ["shard_chains", "global_energy", "parameter_space_qgt", "gather_jacobian", "gather_chain_axis",
           "group_rank_size"]


def shard_chains(n_chains: int, world_size: int, rank: int):
    """Contiguous shard [start, start+count) of n_chains for this rank."""
    base, extra = divmod(int(n_chains), int(world_size))
    count = base + (1 if rank < extra else 0)
    start = rank * base + min(rank, extra)
    return start, count


def _ready(group):
    return dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1


def group_rank_size(group):
    """(rank, world size) of this process in `group` ((0, 1) without an initialised process group)."""
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def gather_chain_axis(x: torch.Tensor, n_chains: int, group=None) -> torch.Tensor:
    """All-gather of per-rank histories x (steps, count_r, ...) over contiguous chain shards
    (``shard_chains``) into (steps, n_chains, ...), chains in global order."""
    if not _ready(group):
        return x
    ws = dist.get_world_size(group)
    counts = [shard_chains(n_chains, ws, r)[1] for r in range(ws)]
    cplx = x.is_complex()
    xr = torch.view_as_real(x) if cplx else x
    m = max(counts)
    pad = xr.new_zeros((xr.shape[0], m) + tuple(xr.shape[2:]))
    pad[:, :xr.shape[1]] = xr
    bufs = [torch.empty_like(pad) for _ in range(ws)]
    dist.all_gather(bufs, pad, group=group)
    out = torch.cat([b[:, :c] for b, c in zip(bufs, counts)], dim=1)
    return torch.view_as_complex(out.contiguous()) if cplx else out


def global_energy(e_local: torch.Tensor, group=None):
    """(mean, variance, n) of the local energies over all ranks."""
    e = e_local.reshape(-1).to(torch.float64)
    buf = torch.stack([e.sum(), (e * e).sum(), torch.tensor(float(e.numel()), dtype=torch.float64,
                                                             device=e.device)])
    if _ready(group):
        dist.all_reduce(buf, group=group)
    n = buf[2]
    mean = buf[0] / n
    return mean, buf[1] / n - mean * mean, int(n.item())


def parameter_space_qgt(jac: SlicedJacobian, group=None):
    """Global S = O^H O / N - mean^H mean over every rank's samples (one all-reduce)."""
    blocks = torch.cat(list(iter_sliced_blocks(jac)), dim=1)
    n_local = torch.tensor([float(blocks.shape[0])], dtype=torch.float64, device=blocks.device)
    gram = blocks.conj().T @ blocks
    osum = blocks.sum(dim=0)
    if _ready(group):
        dist.all_reduce(gram, group=group)
        dist.all_reduce(osum, group=group)
        dist.all_reduce(n_local, group=group)
    n = n_local[0]
    mean = osum / n
    return gram / n - mean.conj()[:, None] * mean[None, :], mean, int(n.item())


def gather_jacobian(o: torch.Tensor, p: torch.Tensor, group=None):
    """All-gather of the sliced Jacobian rows (SampleSpace needs every sample's row)."""
    if not _ready(group):
        return o, p
    ws = dist.get_world_size(group)
    counts = torch.tensor([o.shape[0]], device=o.device)
    all_counts = [torch.zeros_like(counts) for _ in range(ws)]
    dist.all_gather(all_counts, counts, group=group)
    m = int(max(c.item() for c in all_counts))
    pad_o = torch.zeros((m, o.shape[1]), dtype=o.dtype, device=o.device)
    pad_p = torch.zeros((m, p.shape[1]), dtype=p.dtype, device=p.device)
    pad_o[: o.shape[0]] = o
    pad_p[: p.shape[0]] = p
    go = [torch.zeros_like(pad_o) for _ in range(ws)]
    gp = [torch.zeros_like(pad_p) for _ in range(ws)]
    dist.all_gather(go, pad_o, group=group)
    dist.all_gather(gp, pad_p, group=group)
    rows = [int(c.item()) for c in all_counts]
    return (torch.cat([g[:r] for g, r in zip(go, rows)]), torch.cat([g[:r] for g, r in zip(gp, rows)]))
