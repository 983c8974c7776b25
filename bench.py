"""Throughput benchmark: PEPS samples/s for amplitude + O_k + E_loc.

A "step" is one Monte-Carlo sweep of every chain -- the reference's
transition (all sites Metropolis with environment reuse) followed by
estimate (O_k, E_loc, next bottom cache), kernels.py:131-245 -- i.e. one row
of LocalEstimates per chain.  Default workload: 8x8 open-boundary Heisenberg,
D=4, chi=16, ZipUp(16), 4096 chains, seeded synthetic tensors
N(0,1)/sqrt(2 D^4).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU (torchrun): every rank runs its own 4096 chains (replicas; the
chains are independent), value = all ranks' samples / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

def metric_name(w) -> str:
    return f"PEPS samples/s (amp+grad log psi+E_loc), D={w.bond_dim} chi={w.chi}"
UNIT = "samples/s"


def _worker_init():
    # one BLAS thread per worker process: the pool already uses every core
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"


def _oracle_chunk(args):
    """Time the FP64 NumPy restatement on one chunk of chains (runs in a worker process).  With keep > 0
    it also returns the first `keep` chains' sampled configurations, log|psi|, sign, E_loc and O_k: the
    FP64 reference of the bench line's accuracy report."""
    import numpy as np

    from oracle import peps as oracle
    from vmc_gb300.synthetic import WORKLOADS, initial_configs, random_tensors, uniform_stream

    wname, n, seed, keep = (tuple(args) + (0,))[:4]
    w = WORKLOADS[wname]
    # the engine's inputs: the seeded tensors rounded to its FP32 (complex64) elements
    rdt = np.complex64 if w.dtype == "complex64" else np.float32
    T = [[np.asarray(t).astype(rdt).astype(np.complex128 if w.dtype == "complex64" else np.float64) for t in row]
         for row in w.tensors(seed=0)]
    n_sites = w.shape[0] * w.shape[1]
    cfg = initial_configs(n, n_sites, w.phys_dim, seed=seed).astype(np.int64)
    u = next(uniform_stream(n, n_sites, seed=seed))
    strat = {"ZipUp": lambda: oracle.ZipUp(w.chi), "Variational": lambda: oracle.Variational(w.chi, 2)}.get(
        w.strategy, oracle.NoTruncation)()
    model = oracle.PEPS(T, w.shape, w.bond_dim, w.phys_dim, strategy=strat)
    init, trans, est = oracle.build_mc_kernels(model, w.operator())
    cache = init(T, cfg)
    t0 = time.perf_counter()
    c2, ctx = trans(T, cfg, u, cache)
    _, le = est(T, c2, ctx)
    dt = time.perf_counter() - t0
    ref = None
    if keep:
        k = min(keep, n)
        ref = {"configs": c2[:k], "logabs": np.log(np.abs(ctx.amp[:k])), "sign": np.sign(ctx.amp[:k]),
               "E": le.local_estimate[:k], "O": le.local_log_derivatives[:k]}
    return n, dt, ref


GI_SHAPE, GI_DMAX, GI_CHI, GI_G = (9, 9), 2, 32, 0.8
GI_METRIC = "GI-PEPS samples/s (plaquette sweep + grad log psi + E_loc), pure Z2 gauge 9x9, D=2/sector, chi=32"


def _gi_oracle_chunk(args):
    """Time the FP64 GI oracle (oracle/gi.py) on one chunk of chains of the pure-Z2 9x9 workload: bottom
    environments, one plaquette sweep and the estimate (runs in a worker process)."""
    import numpy as np

    from oracle import gi
    from oracle import peps as oracle

    n, seed = args
    cfg = gi.GIConfig(GI_SHAPE, 2, GI_DMAX)
    T = gi.init_tensors(cfg, seed=0)
    H = gi.z2_pure_gauge_hamiltonian(GI_SHAPE, h=1.0 / (2.0 * GI_G), g=GI_G / 2.0, N=2)
    strat = oracle.ZipUp(GI_CHI)
    R, C = GI_SHAPE
    samples = gi.random_physical_configuration(cfg, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    u = rng.random((n, R - 1, C - 1))
    deltas = np.ones((n, R - 1, C - 1), dtype=np.int64)
    t0 = time.perf_counter()
    cache = gi.init_cache(T, cfg, samples, strat)
    samples, amp, top, _ = gi.transition(T, cfg, samples, deltas, u, cache, strat)
    gi.estimate(T, cfg, samples, amp, H, strat, top)
    return n, time.perf_counter() - t0


def gi_oracle_rate(n_per_worker, workers, pool):
    """Samples/s of the GI oracle over `workers` processes (each one sweep of its chunk)."""
    t0 = time.perf_counter()
    res = pool.map(_gi_oracle_chunk, [(n_per_worker, 200 + i) for i in range(workers)])
    wall = time.perf_counter() - t0
    return sum(r[0] for r in res) / wall, sum(r[0] for r in res), wall


def cpu_oracle_rate(wname, n_per_worker, workers, pool, keep=0):
    """Samples/s of the oracle over `workers` processes (each one sweep of its chunk); with keep > 0 also
    the FP64 outputs of the first `keep` chains of chunk 0 (seed 100)."""
    t0 = time.perf_counter()
    res = pool.map(_oracle_chunk, [(wname, n_per_worker, 100 + i, keep if i == 0 else 0) for i in range(workers)])
    wall = time.perf_counter() - t0
    n = sum(r[0] for r in res)
    return n / wall, n, wall, res[0][2]


def accuracy_vs_oracle(eng, w, ref, dev):
    """Errors of one engine sweep on the oracle chunk's first chains (seed-100 configurations and
    uniforms, the same FP32 tensors) against the oracle's FP64 results: log psi (max abs), per-sample
    E_loc (median / max of |dE| / max(1, |E|)), the batch-mean E relative to the energy scale mean|E_loc|
    and relative to |mean E|, O_k (Frobenius over the batch), over the chains whose sampled
    configurations agree (a differing chain had an accept decision within float rounding of its
    threshold), the fraction of chains with an accept decision within 1e-4 of its threshold, and the
    fraction with a near-degenerate cut (relative eigen-gap below 1e-3)."""
    import numpy as np
    import torch

    from vmc_gb300.lowering import pack_tensors
    from vmc_gb300.synthetic import initial_configs, uniform_stream

    k = len(ref["E"])
    n_sites = w.shape[0] * w.shape[1]
    tens = torch.from_numpy(pack_tensors(w.tensors(seed=0))).to(dev)
    cfg = torch.from_numpy(initial_configs(k, n_sites, w.phys_dim, seed=100)).to(dev)
    u = torch.from_numpy(next(uniform_stream(k, n_sites, seed=100))).to(dev)
    cache = eng.init_cache(tens, cfg)
    res = eng.sweep(tens, cfg, u, cache)
    torch.cuda.synchronize()
    same = np.all(res.configs.cpu().numpy() == ref["configs"], axis=1)
    la, sg = res.logamp.cpu().numpy()[same], res.sign.cpu().numpy()[same]
    e, e_ref = res.E.cpu().numpy()[same], ref["E"][same]
    o, o_ref = res.O.cpu().numpy()[same], ref["O"][same]
    de = np.abs(e - e_ref)
    return {"chains": int(k), "same_configs": float(same.mean()),
            "logpsi_abs_max": float(np.max(np.abs(la - ref["logabs"][same]))),
            "sign_agree": bool(np.all(sg == ref["sign"][same])),
            "eloc_rel_median": float(np.median(de / np.maximum(1.0, np.abs(e_ref)))),
            "eloc_rel_max": float(np.max(de / np.maximum(1.0, np.abs(e_ref)))),
            "e_mean_vs_scale": float(abs(e.mean() - e_ref.mean()) / np.abs(e_ref).mean()),
            "e_mean_rel": float(abs(e.mean() - e_ref.mean()) / abs(e_ref.mean())),
            "o_frob_rel": float(np.linalg.norm(o - o_ref) / np.linalg.norm(o_ref)),
            "min_gap": float(res.gap.min().item()),
            # chains with a near-degenerate cut (relative eigen-gap below 1e-3 at some truncation)
            "near_degenerate": float((res.gap.cpu().numpy() < 1e-3).mean()),
            # chains with an accept decision within 1e-4 of its threshold (|min(1, ratio) - u|)
            "near_threshold": float((res.margin.cpu().numpy() < 1e-4).mean()) if res.margin is not None else None}


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, max clock, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def run_reference(args, rank, world):
    """--impl reference: the oracle restatement (the reference is JAX, absent on the box) on host cores."""
    import multiprocessing as mp

    from vmc_gb300.synthetic import WORKLOADS

    if rank != 0:
        return
    if args.workload == "uneven":
        print(json.dumps({"impl": "reference", "unavailable": "the uneven batch has no single reference "
                          "workload: it reports each lattice's own rate in per_shape"}), flush=True)
        return
    cores = len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    if args.workload == "gi9x9":
        # one chain per core and step: ~36 s of FP64 NumPy per chain on one core
        per = max(1, args.gi_ref_chains_per_core)
        with ctx.Pool(cores, initializer=_worker_init) as pool:
            for _ in range(args.warmup):
                gi_oracle_rate(per, cores, pool)
            t0 = time.perf_counter()
            n_total = 0
            for _ in range(args.steps):
                n_total += gi_oracle_rate(per, cores, pool)[1]
            wall = time.perf_counter() - t0
        value = n_total / wall
        print(json.dumps({
            "impl": "reference", "metric": GI_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "gi9x9", "vertices": list(GI_SHAPE), "degeneracy_per_charge": [GI_DMAX, GI_DMAX],
                       "chi": GI_CHI, "N": 2, "g": GI_G, "chains_per_step": per * cores,
                       "parallelism": "host processes"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per * cores} chains x 1 plaquette sweep + estimate per step, FP64 NumPy "
                                       "GI oracle restatement (the reference's JAX CPU path cannot be installed)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    w = WORKLOADS[args.workload]
    per = max(1, args.ref_chains_per_core)
    with ctx.Pool(cores, initializer=_worker_init) as pool:
        for _ in range(args.warmup):
            cpu_oracle_rate(args.workload, per, cores, pool)
        t0 = time.perf_counter()
        n_total = 0
        for _ in range(args.steps):
            _, n, _, _ = cpu_oracle_rate(args.workload, per, cores, pool)
            n_total += n
        wall = time.perf_counter() - t0
    value = n_total / wall
    line = {
        "impl": "reference", "metric": metric_name(w), "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128" if w.dtype == "complex64" else "f64", "data": "synthetic",
        "config": {"workload": w.name, "shape": list(w.shape), "bond_dim": w.bond_dim, "chi": w.chi,
                   "strategy": f"{w.strategy}({w.chi})", "model": w.model,
                   "chains_per_step": per * cores, "parallelism": "host processes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{per * cores} chains x 1 sweep per step, FP64 NumPy oracle restatement "
                                   "(the reference's JAX CPU path cannot be installed: no jax/flax wheels)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def e2e_public_api(w, n, rank, dev, ustream, args, barrier, options=None):
    """Same sweep through the user-facing API (PEPS + build_mc_kernels + make_mc_sampler),
    with every step's uniforms copied from pinned host memory and E_loc, log|psi| and
    sign read back to the host inside the timed region."""
    import torch

    from vmc_gb300.kernels import build_mc_kernels
    from vmc_gb300.peps import PEPS, NoTruncation, Variational, ZipUp
    from vmc_gb300.sampling import make_mc_sampler
    from vmc_gb300.synthetic import initial_configs, random_tensors

    n_sites = w.shape[0] * w.shape[1]
    strategy = {"ZipUp": ZipUp, "Variational": Variational}.get(w.strategy, lambda _: NoTruncation())(w.chi)
    model = PEPS(shape=w.shape, bond_dim=w.bond_dim, phys_dim=w.phys_dim, contraction_strategy=strategy,
                 device=dev, tensors=w.tensors(seed=0),
                 dtype=torch.complex64 if w.dtype == "complex64" else torch.float32, engine_options=options)
    init_cache, transition, estimate = build_mc_kernels(model, w.operator())
    sampler = make_mc_sampler(transition, estimate)
    cfg = torch.from_numpy(initial_configs(n, n_sites, w.phys_dim, seed=rank)).to(dev)
    cache = init_cache(model.tensors, cfg)
    host_u = [torch.from_numpy(next(ustream)).pin_memory() for _ in range(args.warmup + args.steps)]
    e_host = torch.empty(n, dtype=torch.float64).pin_memory()
    la_host = torch.empty(n, dtype=torch.float64).pin_memory()
    sg_host = torch.empty(n, dtype=torch.float64).pin_memory()

    def step(i, cfg, cache):
        u = host_u[i].to(dev, non_blocking=True)
        (cfg, _, cache), (_, est) = sampler(model.tensors, cfg, u[None], cache, n_steps=1)
        e_host.copy_(est.local_estimate[0], non_blocking=True)
        la_host.copy_(est.log_amp[0], non_blocking=True)
        sg_host.copy_(est.sign[0], non_blocking=True)
        return cfg, cache

    for i in range(args.warmup):
        cfg, cache = step(i, cfg, cache)
    barrier()
    stream = torch.cuda.current_stream(dev)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(args.steps):
        cfg, cache = step(args.warmup + i, cfg, cache)
    t1.record(stream)
    barrier()
    elapsed = t0.elapsed_time(t1) / 1e3
    h2d = n * n_sites * 8
    d2h = 3 * n * 8
    return n * args.steps / elapsed, h2d, d2h


def shipped_options(w, precision="fp32"):
    """The launch configuration the shipped GB300 autotune table holds for this workload and precision,
    or None (the engine's default) when the table has no entry for it."""
    from vmc_gb300 import autotune

    return autotune.shipped_options(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, 2, w.dtype,
                                    operator=w.operator(), precision=precision)


def unfused_rate(eng, tens, cfg, args, barrier):
    """The same evaluation split the way the reference's driver splits it: amplitude + O_k in one
    launch (vmc_peps_amp_grad) and E_loc in another (vmc_peps_local_energy), each contracting the
    lattice from scratch, on configurations already sampled.  It does no sampling, so it does less
    work than the fused sweep it is compared with.  Returns samples/s over --steps evaluations."""
    import torch

    n = cfg.shape[0]
    for _ in range(max(1, args.warmup)):
        la, sg, _ = eng.amp_grad(tens, cfg)
        eng.local_energy(tens, cfg, la, sg)
    barrier()
    stream = torch.cuda.current_stream(eng.device)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        la, sg, _ = eng.amp_grad(tens, cfg)
        eng.local_energy(tens, cfg, la, sg)
    t1.record(stream)
    barrier()
    eng.raise_on_status()
    return n * args.steps / (t0.elapsed_time(t1) / 1e3)


def time_sweeps(eng, tens, cfg0, uni, args, barrier, clock_index):
    """Device-resident sweeps: W untimed, then K timed between barriers with CUDA events on the launch
    stream (one pair per launch), nvidia-smi sampling clocks meanwhile.  Returns (elapsed s, per-launch
    ms, clock summary)."""
    import torch

    cfg = cfg0.clone()
    cache = eng.init_cache(tens, cfg)
    out = None
    for i in range(args.warmup):
        out = eng.sweep(tens, cfg, uni[i], cache, out=out)
    barrier()
    eng.raise_on_status()
    stream = torch.cuda.current_stream(eng.device)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    with ClockSampler(clock_index) as clocks:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            out = eng.sweep(tens, cfg, uni[args.warmup + i], cache, out=out)
            ev[i][1].record(stream)
        t_end.record(stream)
        barrier()
    eng.raise_on_status()
    return t_start.elapsed_time(t_end) / 1e3, [x.elapsed_time(y) for x, y in ev], clocks.summary()


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per sample of the fused kernel, from one ncu
# capture of one sweep launch of 608 chains (one wave) of the 8x8 D4 chi16 workload per precision; every
# chain reuses its CTA's slot, so a launch's traffic scales with its chains.  The captured launches come
# from `python -m vmc_gb300.profile_sweep --precision {fp32,mixed} --chains 608`.
NCU_DRAM_BYTES_PER_SAMPLE = {("heis8x8_D4_chi16", "fp32"): (3.451871e9 + 7.283181e9) / 608,
                             ("heis8x8_D4_chi16", "mixed"): (3.722690e9 + 8.795817e9) / 608}


def precision_of(args, w):
    """The headline tier: the mixed-precision engine (boundary-MPS chain in double-float) where it exists -- real
    ZipUp / NoTruncation workloads -- since only it meets the accuracy bars; FP32 elsewhere."""
    if args.precision != "auto":
        return args.precision
    return "mixed" if (w.dtype == "float32" and w.strategy in ("ZipUp", "NoTruncation")) else "fp32"


def run_ours(args, rank, world, local_rank):
    import multiprocessing as mp

    import numpy as np

    # the CPU baseline pool must exist before CUDA is initialised
    pool = None
    cores = len(os.sched_getaffinity(0))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pool = mp.get_context("spawn").Pool(cores, initializer=_worker_init)

    import torch
    import torch.distributed as dist

    from vmc_gb300.engine import PEPSEngine
    from vmc_gb300.lowering import pack_tensors
    from vmc_gb300.synthetic import WORKLOADS, initial_configs, uniform_stream

    w = WORKLOADS[args.workload]
    n = args.chains or w.n_chains
    dev = torch.device(f"cuda:{local_rank}")
    torch.cuda.set_device(dev)
    n_sites = w.shape[0] * w.shape[1]
    prec = precision_of(args, w)
    # the shipped launch table holds each tier's own choice (the engine's defaults where it has none)
    fp32_options = shipped_options(w)
    options = fp32_options if prec == "fp32" else dict(shipped_options(w, "mixed") or {}, precision="mixed")
    eng = PEPSEngine(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, operator=w.operator(), device=dev,
                     dtype=w.dtype, options=options)
    tens = torch.from_numpy(pack_tensors(w.tensors(seed=0))).to(dev)
    cfg0 = torch.from_numpy(initial_configs(n, n_sites, w.phys_dim, seed=rank)).to(dev)
    ustream = uniform_stream(n, n_sites, seed=1000 * rank)
    total = args.warmup + args.steps
    uni = torch.from_numpy(np.stack([next(ustream) for _ in range(total)])).to(dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---------------- device-resident throughput (value) ----------------
    elapsed, launch_ms, clk = time_sweeps(eng, tens, cfg0, uni, args, barrier, local_rank)
    elapsed = max_over_ranks(elapsed)
    value = world * n * args.steps / elapsed

    # ---------------- the plain FP32 engine on the same chains (the metric's denominator) ----------------
    plain, eng32 = None, None
    if prec == "mixed" and not args.no_plain:
        eng32 = PEPSEngine(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, operator=w.operator(), device=dev,
                           dtype=w.dtype, options=fp32_options)
        el32, ms32, clk32 = time_sweeps(eng32, tens, cfg0, uni, args, barrier, local_rank)
        el32 = max_over_ranks(el32)
        plain = {"value": world * n * args.steps / el32, "unit": UNIT, "precision": "fp32",
                 "kernel_ms_per_launch": statistics.mean(ms32), "clocks": clk32,
                 "launch_options": fp32_options or "engine default"}

    # ---------------- the unfused split (amp+O_k launch, then E_loc launch) ----------------
    unfused = unfused_rate(eng, tens, cfg0.clone(), args, barrier) if not args.no_unfused else None

    # ---------------- end-to-end through the public API, host buffers ----------------
    e2e_value, h2d, d2h = e2e_public_api(w, n, rank, dev, ustream, args, barrier, options)
    if world > 1:
        e2e_value = world * n * args.steps / max_over_ranks(n * args.steps / e2e_value)

    if rank != 0:
        return
    peaks, peak_kind = _peaks()
    flops = w.flops_per_sample()
    mean_launch_s = statistics.mean(launch_ms) / 1e3
    achieved = n * flops / mean_launch_s / 1e12 if flops else None
    peak = peaks.get("bf16_tflops")
    traffic = NCU_DRAM_BYTES_PER_SAMPLE.get((w.name, prec))
    kernel = "vmc::rm::peps_kernel" if prec == "mixed" else "vmc::rk::peps_kernel"
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved and peak else None,
                "traffic": traffic * n if traffic else None, "traffic_unit": "bytes per launch",
                "peak_kind": f"{peak_kind} bf16 burst (cuBLAS)", "kernel": kernel,
                "flop_per_sample": flops, "units_per_launch": n}
    cpu, accuracy = None, None
    if pool is not None:
        per = max(1, args.cpu_chains_per_core)
        keep = min(args.accuracy_chains, per)
        rate, ns, wall, ref = cpu_oracle_rate(w.name, per, cores, pool, keep=keep)
        pool.close()
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{ns} chains x 1 sweep ({wall:.1f} s), FP64 NumPy oracle restatement over {cores} "
                         "processes"}
        if ref is not None and w.dtype == "float32":
            accuracy = {"reference": f"FP64 oracle, the first {keep} chains of its sample (same FP32 tensors, "
                                     "configurations and uniforms), one sweep",
                        prec: accuracy_vs_oracle(eng, w, ref, dev)}
            if eng32 is not None:
                accuracy["fp32"] = accuracy_vs_oracle(eng32, w, ref, dev)
            accuracy["bars"] = {"e_mean_vs_scale": 1e-5, "o_frob_rel": 1e-4}
    # the kernel runs on the CUDA cores (the mixed tier's eigenvalues also on the FP64 units): the fraction of
    # the nominal FP32 FMA peak, at the SM clock sampled during the run (SMs x 128 lanes x 2 x clock)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    fp32_peak = n_sm * 128 * 2 * mhz * 1e6 / 1e12 if mhz else None
    roofline_fp32 = {"achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if achieved and fp32_peak else None,
                     "peak_kind": f"nominal FP32 FMA: {n_sm} SMs x 128 lanes x 2 x {mhz} MHz"}
    line = {
        "metric": metric_name(w), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64" if w.dtype == "complex64" else "f32",
        "data": "synthetic",
        "config": {"workload": w.name, "shape": list(w.shape), "bond_dim": w.bond_dim, "chi": w.chi,
                   "phys_dim": w.phys_dim, "strategy": f"{w.strategy}({w.chi})", "model": w.model,
                   "chains_per_gpu": n, "global_chains": n * world, "parallelism": f"replicas x{world}",
                   "precision": prec + (" (boundary-MPS chain in double-float with FP64 eigenvalues, FP32 elsewhere)" if prec == "mixed" else ""),
                   "launch_options": options or "engine default",
                   "l2": "inputs larger than L2 (bottom-env cache "
                         f"{eng.cache_bytes(n) / 1e9:.2f} GB read+written per step)"},
        "roofline": roofline,
        "roofline_fp32": roofline_fp32,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
        "kernel_ms_per_launch": statistics.mean(launch_ms),
    }
    if plain is not None:
        plain["mixed_over_plain"] = value / plain["value"]
        line["plain_fp32"] = plain
    if accuracy is not None:
        line["accuracy"] = accuracy
    if unfused is not None:
        line["unfused"] = {"value": unfused, "unit": UNIT, "launches_per_step": 2, "precision": prec,
                           "what": "amp+O_k launch then E_loc launch on sampled configurations (no "
                                   "sampling), device-resident; the fused sweep also samples",
                           "fused_over_unfused": value / unfused}
    print(json.dumps(line), flush=True)


UNEVEN = ["heis6x6_D4_chi16", "heis8x8_D5_chi25", "heis12x12_D6_chi36", "heis16x16_D6_chi48"]


def run_uneven(args, rank, world, local_rank):
    """--workload uneven: the four Heisenberg lattices of the uneven batch (6x6 D4 chi16, 8x8 D5 chi25,
    12x12 D6 chi36, 16x16 D6 chi48; --chains each, default 4096) in ONE persistent launch
    (vmc_peps_batch) captured in a CUDA graph.  value: samples/s of graph replays, inputs on the device;
    e2e: the eager PEPSBatch.run with host uniforms in and E/log|psi|/sign out; per_shape: every
    lattice launched alone (samples/s, algorithmic TFLOP/s and its roofline fraction)."""
    import torch

    from vmc_gb300.engine import PEPSBatch, PEPSEngine
    from vmc_gb300.lowering import pack_tensors
    from vmc_gb300.synthetic import WORKLOADS, initial_configs

    n = args.chains or 4096
    dev = torch.device(f"cuda:{local_rank}")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    total = args.warmup + args.steps
    gen = torch.Generator(device=dev).manual_seed(1000 * rank + 7)
    peaks, peak_kind = _peaks()
    peak = peaks.get("bf16_tflops")
    from vmc_gb300.autotune import tuned_options

    # launch configuration per lattice: the autotuned one (alone); the batch runs every plan with
    # one CTA size, so it takes the options of the lattice with the most work per chain
    tuned = {name: tuned_options(WORKLOADS[name].shape, WORKLOADS[name].bond_dim, WORKLOADS[name].chi,
                                 WORKLOADS[name].phys_dim, WORKLOADS[name].strategy, 2, WORKLOADS[name].dtype,
                                 operator=WORKLOADS[name].operator(), device=dev) for name in UNEVEN}
    dominant = max(UNEVEN, key=lambda name: WORKLOADS[name].flops_per_sample())
    batch_options = tuned[dominant]
    cases = []
    for name in UNEVEN:
        w = WORKLOADS[name]
        n_sites = w.shape[0] * w.shape[1]
        eng = PEPSEngine(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, operator=w.operator(), device=dev,
                         options=tuned[name])
        tens = torch.from_numpy(pack_tensors(w.tensors(seed=0))).to(dev)
        cfg0 = torch.from_numpy(initial_configs(n, n_sites, w.phys_dim, seed=rank)).to(dev)
        uni = torch.rand((total, n, n_sites), generator=gen, dtype=torch.float64, device=dev)
        cases.append((w, eng, tens, cfg0, uni))

    def timed(step_fn):
        for i in range(args.warmup):
            step_fn(i)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for i in range(args.steps):
            step_fn(args.warmup + i)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / args.steps

    # ---------------- every lattice alone ----------------
    per_shape, t_alone = [], 0.0
    for w, eng, tens, cfg0, uni in cases:
        cfg = cfg0.clone()
        cache = eng.init_cache(tens, cfg)
        box = {"out": None}

        def one(i, eng=eng, tens=tens, cfg=cfg, uni=uni, cache=cache, box=box):
            box["out"] = eng.sweep(tens, cfg, uni[i], cache, out=box["out"])

        t = timed(one)
        eng.raise_on_status()
        t_alone += t
        flops = w.flops_per_sample()
        tf = n * flops / t / 1e12
        per_shape.append({"workload": w.name, "options": tuned[w.name], "shape": list(w.shape),
                          "bond_dim": w.bond_dim, "chi": w.chi,
                          "chains": n, "samples_per_s": n / t, "ms_per_launch": 1e3 * t,
                          "tflops_algorithmic": tf, "roofline_frac": tf / peak if peak else None})
        del cache

    # ---------------- one launch over all four, captured in a CUDA graph ----------------
    jobs, ubuf = [], []
    for i, (w, eng, tens, cfg0, uni) in enumerate(cases):
        eng = PEPSEngine(w.shape, w.bond_dim, w.chi, w.phys_dim, w.strategy, operator=w.operator(), device=dev,
                         options=batch_options)
        cases[i] = (w, eng, tens, cfg0, uni)
        cfg = cfg0.clone()
        cache = eng.init_cache(tens, cfg)
        u = uni[0].clone()
        ubuf.append(u)
        jobs.append(eng.sweep_job(tens, cfg, u, cache))
    batch = PEPSBatch(dev)
    batch.run(jobs)
    torch.cuda.synchronize()
    batch.raise_on_status()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        batch.run(jobs)

    def replay(i):
        for u, (_, _, _, _, uni) in zip(ubuf, cases):
            u.copy_(uni[i], non_blocking=True)
        graph.replay()

    with ClockSampler(local_rank) as clocks:
        t_graph = timed(replay)
    batch.raise_on_status()

    # ---------------- end to end: eager batch, host uniforms in, results out ----------------
    host_u = [[uni[i].cpu().pin_memory() for i in range(total)] for (_, _, _, _, uni) in cases]
    host_out = [[torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(3)] for _ in cases]

    def e2e_step(i):
        for k, u in enumerate(ubuf):
            u.copy_(host_u[k][i], non_blocking=True)
        outs = batch.run(jobs)
        for k, o in enumerate(outs):
            for h, src in zip(host_out[k], (o.E, o.logamp, o.sign)):
                h.copy_(src, non_blocking=True)

    t_e2e = timed(e2e_step)
    batch.raise_on_status()
    h2d = sum(n * w.shape[0] * w.shape[1] * 8 for (w, _, _, _, _) in cases)
    d2h = len(cases) * 3 * n * 8
    samples = len(cases) * n
    flops = sum(n * w.flops_per_sample() for (w, _, _, _, _) in cases)
    achieved = flops / t_graph / 1e12
    clk = clocks.summary()
    line = {
        "metric": "PEPS samples/s (amp+grad log psi+E_loc), uneven batch in one launch: "
                  "6x6 D4 chi16 + 8x8 D5 chi25 + 12x12 D6 chi36 + 16x16 D6 chi48",
        "value": samples / t_graph, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_graph, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "uneven", "shapes": UNEVEN, "chains_per_shape": n, "model": "heisenberg",
                   "strategy": "ZipUp(chi)", "launch": "one persistent launch (vmc_peps_batch) in a CUDA graph",
                   "options_alone": tuned, "options_batch": batch_options,
                   "parallelism": "replicas x1",
                   "l2": "inputs larger than L2 (bottom-env caches of all four lattices)"},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "peak_kind": f"{peak_kind} bf16 burst (cuBLAS)", "kernel": "vmc::peps_kernel (batch)"},
        "per_shape": per_shape,
        "sequential_launches_ms": 1e3 * t_alone,
        "batch_vs_sequential": t_alone / t_graph,
        "cpu_baseline": None,
        "e2e": {"value": samples / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": (len(cases) + 1) * args.steps,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gi(args, rank, world, local_rank):
    """--workload gi9x9: the gauge-invariant PEPS of pure Z2 lattice gauge theory on 9x9 vertices
    (8x8 plaquettes), 2 states per charge sector, chi=32, --chains chains (default 4096).  H of the
    lattice-gauge workload, -g sum sigma^x - (1/g) sum prod sigma^z with g = 0.8, written in the
    electric basis the GI model samples: g/2 (2 - 2 (-1)^E) per link (the same up to a constant) and
    -1/(2g) (P + P^dag) per plaquette.  value: plaquette sweep + O_k + E_loc samples/s, inputs on the
    device; e2e: the public kernels (build_mc_kernels) with host uniforms in and E/log|psi|/sign out."""
    import multiprocessing as mp

    # the CPU baseline pool must exist before CUDA is initialised
    pool = None
    cores = len(os.sched_getaffinity(0))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pool = mp.get_context("spawn").Pool(cores, initializer=_worker_init)

    import torch

    from vmc_gb300 import ZipUp
    from vmc_gb300.gi import GIPEPS, GIPEPSConfig, build_gi_mc_kernels, z2_pure_gauge_hamiltonian

    n = args.chains or 4096
    g = GI_G
    shape, dmax, chi = GI_SHAPE, GI_DMAX, GI_CHI
    dev = torch.device(f"cuda:{local_rank}")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    cfg = GIPEPSConfig(shape=shape, N=2, phys_dim=1, Qx=0, degeneracy_per_charge=(dmax, dmax))
    model = GIPEPS(rngs=0, config=cfg, contraction_strategy=ZipUp(chi), device=dev)
    H = z2_pure_gauge_hamiltonian(shape, h=1.0 / (2.0 * g), g=g / 2.0)
    eng = model.engine(H)
    tens = model.packed()
    n_plaq = (shape[0] - 1) * (shape[1] - 1)
    total = args.warmup + args.steps
    gen = torch.Generator(device=dev).manual_seed(1000 * rank + 11)
    uni = torch.rand((total, n, n_plaq), generator=gen, dtype=torch.float64, device=dev)
    cfg0 = model.random_physical_configuration(rank, n)
    c = cfg0.clone()
    cache = eng.init_cache(tens, c)
    out = None
    for i in range(args.warmup):
        out = eng.sweep(tens, c, uni[i], cache, out=out)
    torch.cuda.synchronize()
    eng.raise_on_status()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        a.record(stream)
        for i in range(args.steps):
            out = eng.sweep(tens, c, uni[args.warmup + i], cache, out=out)
        b.record(stream)
        torch.cuda.synchronize()
    eng.raise_on_status()
    t = a.elapsed_time(b) / 1e3 / args.steps
    # end to end through the public kernels, host buffers
    init, trans, est = build_gi_mc_kernels(model, H)
    c = cfg0.clone()
    kcache = init(model.tensors, c)
    host_u = [uni[i].cpu().pin_memory() for i in range(total)]
    host = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(3)]

    def step(i, c, kcache):
        u = host_u[i].to(dev, non_blocking=True)
        c, _, ctx = trans(model.tensors, c, u, kcache)
        kcache, le = est(model.tensors, c, ctx)
        for h_, src in zip(host, (le.local_estimate, le.log_amp, le.sign)):
            h_.copy_(src, non_blocking=True)
        return c, kcache

    for i in range(args.warmup):
        c, kcache = step(i, c, kcache)
    torch.cuda.synchronize()
    a.record(stream)
    for i in range(args.steps):
        c, kcache = step(args.warmup + i, c, kcache)
    b.record(stream)
    torch.cuda.synchronize()
    t_e2e = a.elapsed_time(b) / 1e3 / args.steps
    cpu = None
    if pool is not None:
        rate, ns, wall = gi_oracle_rate(max(1, args.gi_ref_chains_per_core), cores, pool)
        pool.close()
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{ns} chains x 1 sweep ({wall:.1f} s), FP64 NumPy GI oracle over {cores} processes"}
    line = {
        "metric": GI_METRIC,
        "value": n / t, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "gi9x9", "vertices": list(shape), "degeneracy_per_charge": [dmax, dmax], "chi": chi,
                   "N": 2, "g": g, "model": "pure Z2 lattice gauge theory", "chains_per_gpu": n,
                   "parallelism": "replicas x1",
                   "l2": f"inputs larger than L2 (bottom-env cache {eng.cache_bytes(n) / 1e9:.2f} GB)"},
        "roofline": {"bound": "tensor", "achieved": None, "peak": None, "unit": "TFLOP/s", "frac": None,
                     "traffic": None, "note": "no algorithmic FLOP count exists for the GI path"},
        "cpu_baseline": cpu,
        "e2e": {"value": n / t_e2e, "unit": UNIT, "h2d_bytes_per_step": n * n_plaq * 8, "d2h_bytes_per_step": 3 * n * 8},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="heis8x8_D4_chi16")
    ap.add_argument("--chains", type=int, default=0)
    ap.add_argument("--cpu-chains-per-core", type=int, default=128)
    ap.add_argument("--ref-chains-per-core", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-unfused", action="store_true", help="skip the unfused amp+O_k / E_loc comparison leg")
    ap.add_argument("--gi-ref-chains-per-core", type=int, default=1,
                    help="GI workload: oracle chains per host core per step (reference arm and cpu_baseline)")
    ap.add_argument("--precision", choices=["auto", "mixed", "fp32"], default="auto",
                    help="engine tier of the headline: auto = mixed (double-float boundary-MPS chain) where it exists")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 leg beside a mixed headline")
    ap.add_argument("--accuracy-chains", type=int, default=64,
                    help="chains of the CPU-baseline sample whose FP64 results check both tiers")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        if args.workload == "uneven":
            run_uneven(args, rank, world, local_rank)
        elif args.workload == "gi9x9":
            run_gi(args, rank, world, local_rank)
        else:
            run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
