"""One init_cache and one sweep of the 8x8 Heisenberg D=4 chi=16 workload on cuda:0, for profiler captures.

    python -m vmc_gb300.profile_sweep --precision mixed --chains 608
    python -m vmc_gb300.profile_sweep --precision fp32 --workload heis8x8_D5_chi25 --chains 304 \
        --threads 256 --tile-policy 4

The fused kernel launches twice (init_cache, then the sweep); an ncu capture of the sweep alone skips
the first: ``-k regex:peps_kernel -s 1 -c 1``.  608 chains are one wave on a GB300 (152 SMs x 4 CTAs).
"""
from __future__ import annotations

import argparse


def main(argv=None) -> None:
    import torch

    from .engine import PEPSEngine
    from .lowering import pack_tensors
    from .synthetic import WORKLOADS, initial_configs, uniform_stream

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--precision", choices=["fp32", "mixed"], default="mixed")
    ap.add_argument("--chains", type=int, default=608)
    ap.add_argument("--workload", default="heis8x8_D4_chi16")
    ap.add_argument("--threads", type=int, default=0, help="CTA threads (0: the plan's default)")
    ap.add_argument("--tile-policy", type=int, default=None, help="GEMM tile policy (0-4)")
    args = ap.parse_args(argv)
    w = WORKLOADS[args.workload]
    n, n_sites = args.chains, w.shape[0] * w.shape[1]
    dev = torch.device("cuda:0")
    options = None
    if args.threads or args.tile_policy is not None:
        options = {"threads": args.threads, "smem_kb": -1, "tile_policy": args.tile_policy or 0}
    eng = PEPSEngine(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, operator=w.operator(), device=dev,
                     dtype=w.dtype, precision=args.precision, options=options)
    tens = torch.from_numpy(pack_tensors(w.tensors(seed=0))).to(dev)
    cfg = torch.from_numpy(initial_configs(n, n_sites, w.phys_dim, seed=0)).to(dev)
    u = torch.from_numpy(next(uniform_stream(n, n_sites, seed=0))).to(dev)
    cache = eng.init_cache(tens, cfg)
    res = eng.sweep(tens, cfg, u, cache)
    torch.cuda.synchronize()
    eng.raise_on_status()
    print(f"{args.precision} {n} chains, options {eng.options}: mean E_loc {float(res.E.mean()):.6f}")


if __name__ == "__main__":
    main()
