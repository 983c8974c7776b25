"""Times the SampleSpace Gram of a sliced Jacobian on cuda:0: the engine's ``vmc_sliced_gram`` kernel
against the expanded-block build with cuBLAS FP64 GEMMs (``qgt.iter_sliced_blocks``, 16 column blocks
per slice), on synthetic FP32 log-derivatives with the 8x8 Heisenberg D=4 sliced layout by default.

    python -m vmc_gb300.profile_gram --n 4096 --ncols 10816 --reps 5
    python -m vmc_gb300.profile_gram --space parameter --reps 3

SampleSpace: the kernel computes n(n+1)/2 x ncols masked products (the lower triangle); the expanded
build computes n^2 x ncols x d multiply-adds, half of them on zeros.  ParameterSpace (d = 2): the kernel
computes about n x ncols^2 / 2 products into the (d ncols)^2 matrix; the expanded build computes
n x (d ncols)^2 multiply-adds.
"""
from __future__ import annotations

import argparse
import json


def main(argv=None) -> None:
    import torch

    from . import qgt as gq
    from .linalg import sliced_gram

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--ncols", type=int, default=10816)
    ap.add_argument("--d", type=int, default=2)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--kernel-only", action="store_true", help="skip the cuBLAS build (for profiler captures)")
    ap.add_argument("--space", choices=["sample", "parameter"], default="sample")
    args = ap.parse_args(argv)
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    o = torch.randn((args.n, args.ncols), generator=g, device=dev, dtype=torch.float32)
    p = torch.randint(0, args.d, (args.n, args.ncols), generator=g, device=dev, dtype=torch.int8)
    jac = gq.SlicedJacobian(o, p, (args.d,) * args.ncols)

    def timed(fn):
        out = fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1) / args.reps

    if args.space == "parameter":
        from .linalg import sliced_gram_params

        S, ms_k = timed(lambda: sliced_gram_params(o, p, args.d))
        res = {"space": "parameter", "n": args.n, "ncols": args.ncols, "d": args.d, "kernel_ms": round(ms_k, 3),
               "kernel_products_per_s": args.n * args.ncols * (args.ncols + 32) / 2 / (ms_k * 1e-3)}
        if not args.kernel_only:
            del S

            def expanded():
                E = torch.cat(list(gq.iter_sliced_blocks(jac)), dim=1)
                return E.T @ E

            G, ms_b = timed(expanded)
            S = sliced_gram_params(o, p, args.d)
            res.update({"cublas_expanded_ms": round(ms_b, 3),
                        "cublas_fp64_tflops": 2.0 * args.n * (args.d * args.ncols) ** 2 / (ms_b * 1e-3) / 1e12,
                        "speedup": ms_b / ms_k,
                        "rel_frobenius_diff": float(torch.linalg.norm(S - G) / torch.linalg.norm(G))})
        print(json.dumps(res))
        return
    T, ms_k = timed(lambda: sliced_gram(o, p))
    res = {"n": args.n, "ncols": args.ncols, "d": args.d, "kernel_ms": round(ms_k, 3),
           "kernel_products_per_s": args.n * (args.n + 1) / 2 * args.ncols / (ms_k * 1e-3)}
    if not args.kernel_only:
        def blocked():
            G = torch.zeros((args.n, args.n), dtype=torch.float64, device=dev)
            for ob in gq.iter_sliced_blocks(jac, 16):
                G += ob @ ob.T
            return G

        G, ms_b = timed(blocked)
        res.update({"cublas_blocked_ms": round(ms_b, 3),
                    "cublas_fp64_tflops": 2.0 * args.n * args.n * args.ncols * args.d / (ms_b * 1e-3) / 1e12,
                    "speedup": ms_b / ms_k,
                    "rel_frobenius_diff": float(torch.linalg.norm(T - G) / torch.linalg.norm(G))})
    print(json.dumps(res))


if __name__ == "__main__":
    main()
