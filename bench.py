#!/usr/bin/env python
"""Benchmark of the FMM GEMM path on GB300.

Workload (one step): C := C + A*B, m = n = k = 16384, column-major FP64
operands uniform in [-1, 1) (seeded), computed by the split-precision FMM:
Strassen <2,2,2> at two recursion levels (49 products of 4096^3) with the FP64
operand sums split into 6 BF16 digit slices (21 slice pairs per product) on
the tcgen05 tensor cores. Operands are 2 GiB each, far larger than L2, so no
flush is needed between steps.

Metric: effective TFLOP/s = 2mnk / t (whole job over all ranks). Reported
beside it, once per run and outside the timed loop: the plain FP64 FMM and
the classical FP64 GEMM of this library at the same shape (time and max-norm
error against the classical result), the split form's error, the dominant
kernel's roofline, the end-to-end number through host buffers, and the
reference algorithm on the host cores (the oracle's C restatement, a bounded
sample of products).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs an independent replica of the workload (the
path needs no exchange); rank 0 prints one JSON line.
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

import numpy as np

ROOT = Path(__file__).resolve().parent
COEFFS = ROOT / "fmm_blis_gb300" / "coeffs"     # the algorithms shipped with the package
sys.path.insert(0, str(ROOT))
# many differently sized request buffers (served workload): grow segments
# instead of fragmenting fixed ones
os.environ.setdefault("PYTORCH_ALLOC_CONF", "expandable_segments:True")

METRIC = "eff. TFLOP/s (2mnk/t): split-BF16 FMM vs FP64 FMM at stated err; p99 latency"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--alg", default="222")
    p.add_argument("--levels", type=int, default=2)
    p.add_argument("--slices", type=int, default=6)
    p.add_argument("--fmt", choices=["bf16", "fp8"], default="bf16",
                   help="slice format of the split form: BF16 (base-256 digits) or FP8-E4M3 (base-32 digits)")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison runs")
    p.add_argument("--no-cpu", action="store_true", help="skip the host-core baseline")
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--f64-engine", choices=["dfma", "mma"], default=None,
                   help="micro-kernel of the plain FP64 form (default: the library's)")
    p.add_argument("--serve-seconds", type=float, default=10.0,
                   help="default workload: seconds of the bounded served stream (Poisson 200/s); 0 skips it")
    p.add_argument("--form", choices=["split", "fp64"], default="split",
                   help="split: split-BF16 FMM (the headline); fp64: the plain FP64 FMM drop-in")
    p.add_argument("--workload", choices=["fmm", "batch", "serve", "sweep", "accuracy"], default="fmm",
                   help="fmm: one square FMM GEMM per step (the headline); batch: 512 uneven GEMMs per step; "
                        "serve: Poisson request stream; sweep: plain FP64 FMM over algorithms, levels and "
                        "sizes; accuracy: split error per slice count")
    p.add_argument("--count", type=int, default=512, help="batch: GEMMs per step")
    p.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    p.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    p.add_argument("--split-fraction", type=float, default=0.9, help="serve: share of split-tagged requests")
    p.add_argument("--target", type=float, default=1e-10, help="split requests: target relative error")
    return p.parse_args()


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("bf16_tflops_sustained", 1737.1), d.get("bf16_tflops", 1926.8), d.get("hbm_gbs"), "measured"
    return 1700.0, 1900.0, 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_barrier(world: int) -> None:
    """All ranks meet (replicas: no data-path collective, only timing)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def rank_max(x: float, world: int, device) -> float:
    """The largest of the ranks' values (the slowest replica's time): one
    all-reduce of a float64 on `device` (cuda under NCCL, cpu under gloo)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def host_operands(n, seed=7):
    """Column-major float64 host operands (torch's CPU generator, seeded)."""
    import torch
    g = torch.Generator().manual_seed(seed)
    return [np.asfortranarray((torch.rand((n, n), generator=g, dtype=torch.float64) * 2 - 1).numpy().T)
            for _ in range(3)]


def cpu_reference_plan(alg, levels, n, target_s, arrays):
    """How many products of the flattened algorithm make a host-core sample of
    about target_s seconds at the full shape (one product timed first)."""
    import oracle
    from oracle import coeffs as oc

    flat = oc.power(oc.read(COEFFS / f"{alg}.txt"), levels)
    R = flat[3]
    oracle.set_threads(os.cpu_count() or 1)
    A, B, C = arrays
    t0 = time.perf_counter()
    oracle.fmm_dgemm(flat, A, B, C, r_begin=0, r_end=1)
    t1 = time.perf_counter() - t0
    return flat, max(1, min(R, int(target_s / max(t1, 1e-3)))), R


def cpu_reference_sample(flat, P, arrays):
    """Seconds for products 0..P-1 of the reference FMM algorithm (oracle,
    FP64) on the host cores at the full shape."""
    import oracle

    A, B, C = arrays
    t0 = time.perf_counter()
    oracle.fmm_dgemm(flat, A, B, C, r_begin=0, r_end=P)
    return time.perf_counter() - t0


def cpu_reference(alg, levels, n, target_s, arrays=None):
    """The reference FMM algorithm (oracle, FP64) on the host cores: a bounded
    sample of the products of the flattened algorithm at the full shape.
    Returns (eff TFLOP/s of the sample: its share P/R of 2n^3 over its time,
    dict)."""
    import oracle

    arrays = arrays if arrays is not None else host_operands(n)
    flat, P, R = cpu_reference_plan(alg, levels, n, target_s, arrays)
    tp = cpu_reference_sample(flat, P, arrays)
    eff = 2.0 * n ** 3 * (P / R) / tp / 1e12
    info = {"cores": oracle.num_threads(), "products": P, "of": R, "seconds": tp}
    return eff, info


def run_reference(args):
    """The reference arm: each step is a bounded sample of the workload on the
    host cores (products 0..P-1 of the R products of the FMM step at the full
    shape, P sized to a few seconds), timed; value = the sample's effective
    flops (its share P/R of 2mnk) over its time, ms_per_step = that time."""
    import oracle

    world, rank, _ = dist_setup()
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    per_step = max(2.0, 60.0 / max(steps + warm, 1))
    arrays = host_operands(args.n)
    flat, P, R = cpu_reference_plan(args.alg, args.levels, args.n, per_step, arrays)
    secs = []
    for i in range(warm + steps):
        t = cpu_reference_sample(flat, P, arrays)
        if i >= warm:
            secs.append(t)
    t_step = statistics.median(secs)
    sample_flops = 2.0 * args.n ** 3 * P / R
    value = sample_flops / t_step / 1e12
    cores = oracle.num_threads()
    sample = (f"FP64 FMM {args.alg} x{args.levels} levels at m=n=k={args.n}: products 0..{P - 1} of {R} per step "
              f"({t_step:.2f} s; {P}/{R} of the step's 2mnk)")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"FMM {args.alg} x{args.levels} levels, m=n=k={args.n} (reference algorithm, FP64, host "
                               f"cores), a sample of {P} of its {R} products per step",
                   "m": args.n, "n": args.n, "k": args.n, "alg": args.alg, "levels": args.levels,
                   "sample_products": P, "products": R},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


L2_BYTES = 129 * 2 ** 20


def l2_flush_buffer(torch, dev, operand_bytes):
    """A buffer to overwrite between timed steps when the operands would stay
    resident in L2 (less than twice its size); None otherwise."""
    if operand_bytes >= 2 * L2_BYTES:
        return None
    return torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)


def timed_steps(torch, stream, steps, fn, flush):
    """Total device milliseconds of `steps` calls of fn on `stream`: one event
    pair around the loop, or, with a flush buffer, one pair per step with the
    buffer overwritten (outside the events) between steps."""
    if flush is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)
    pairs = []
    for _ in range(steps):
        flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        pairs.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in pairs)


def batch_shapes(count, seed, lo=256, hi=8192):
    """count (m, n, k) triples, each dimension log-uniform in [lo, hi], seeded"""
    rng = np.random.default_rng(seed)
    return [tuple(int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi)))))) for _ in range(3))
            for _ in range(count)]


def _dev_operand(torch, rows, cols, seed, dev, phi=None):
    """column-major operand on the device: uniform [-1, 1) or, with phi, the
    wide-range case (u - 0.5) * exp(phi * g), u ~ U[0, 1), g ~ N(0, 1)"""
    g = torch.Generator(device=dev).manual_seed(seed)
    u = torch.rand((cols, rows), generator=g, device=dev, dtype=torch.float64)
    if phi is None:
        return u.mul_(2).sub_(1).t()
    z = torch.randn((cols, rows), generator=g, device=dev, dtype=torch.float64)
    return u.sub_(0.5).mul_(z.mul_(phi).exp_()).t()


def _time_once(torch, fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_sweep(args, fmm, dev, rank):
    """Plain FP64 FMM sweep: 232, 322, 333, 444 at one and two levels, square
    m = n = k in {4096, 8192, 12288, 16384} and (m, k, n) = (16384, 4096, 16384),
    (8192, 16384, 8192); each beside the classical FP64 GEMM of this library
    (time, and the max-norm difference against it in units of
    eps64 * k * max|A| * max|B|). One warm call, one timed call per case."""
    import torch

    shapes = [(n, n, n) for n in (4096, 8192, 12288, 16384)] + [(16384, 16384, 4096), (8192, 8192, 16384)]
    rows = []
    algs = {a: fmm.new_fmm(COEFFS / f"{a}.txt") for a in ("232", "322", "333", "444")}
    for (m, n, k) in shapes:
        A = _dev_operand(torch, m, k, 11, dev)
        B = _dev_operand(torch, k, n, 12, dev)
        C0 = _dev_operand(torch, m, n, 13, dev)
        Cc = C0.clone()
        fmm.dgemm(A, B, Cc.clone(), None, 0)
        ms_c = _time_once(torch, lambda: fmm.dgemm(A, B, Cc, None, 0))
        unit = 2.0 ** -52 * k * float(A.abs().max()) * float(B.abs().max())
        flops = 2.0 * m * n * k
        for name, f in algs.items():
            for L in (1, 2):
                Cf = C0.clone()
                fmm.dgemm(A, B, Cf.clone(), f, L)
                ms = _time_once(torch, lambda: fmm.dgemm(A, B, Cf, f, L))
                rows.append({"alg": name, "levels": L, "m": m, "n": n, "k": k, "ms": ms,
                             "tflops": flops / ms / 1e9, "vs_classical": ms_c / ms,
                             "err_units": float((Cf - Cc).abs().max()) / unit})
                del Cf
        rows.append({"alg": "classical", "levels": 0, "m": m, "n": n, "k": k, "ms": ms_c,
                     "tflops": flops / ms_c / 1e9, "vs_classical": 1.0, "err_units": 0.0})
        del A, B, C0, Cc
        torch.cuda.empty_cache()
    for f in algs.values():
        fmm.free_fmm(f)
    assert fmm.take_device_error() == 0
    if rank == 0:
        best = max((r for r in rows if r["m"] == r["n"] == r["k"] == 16384 and r["levels"] > 0),
                   key=lambda r: r["tflops"])
        print(json.dumps({"metric": METRIC, "value": best["tflops"], "unit": "TFLOP/s", "n_gpus": 1, "steps": 1,
                          "warmup": 1, "ms_per_step": best["ms"], "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": "plain FP64 FMM sweep (232, 322, 333, 444 x levels 1, 2; "
                                                 "square 4096..16384 and two rectangular shapes)"},
                          "rows": rows}))


def run_accuracy(args, fmm, dev, rank):
    """Split-form accuracy per slice count: 222 two levels and 333 one level
    at m = n = k in {8192, 16384}, inputs uniform [-1, 1) and the wide-range
    case with phi = 1 and 4; 3..7 BF16 slices and 7..12 FP8-E4M3 slices. Errors against the classical
    FP64 GEMM of this library: max-norm, max-norm relative to max|C|,
    relative Frobenius; the plain FP64 FMM's error beside them."""
    import torch

    from fmm_blis_gb300 import tune

    algs = {"222": (fmm.new_fmm(COEFFS / "222.txt"), 2),
            "333": (fmm.new_fmm(COEFFS / "333.txt"), 1)}
    tuner = tune.Tuner()
    rows = []
    for n in (8192, 16384):
        for dist, phi in (("uniform", None), ("hard_phi1", 1.0), ("hard_phi4", 4.0)):
            A = _dev_operand(torch, n, n, 21, dev, phi)
            B = _dev_operand(torch, n, n, 22, dev, phi)
            ref = torch.zeros((n, n), dtype=torch.float64, device=dev).t()
            fmm.dgemm(A, B, ref, None, 0)
            torch.cuda.synchronize()
            rmax, rfro = float(ref.abs().max()), float(torch.linalg.norm(ref))
            # the tuner's input-aware plan for a 1e-10 target, and what it gives
            p = tuner.plan_for(fmm, A, B, 1e-10)
            fp = None if p.alg == "classical" else fmm.new_fmm(COEFFS / f"{p.alg}.txt")
            Ct = torch.zeros_like(ref)
            fmm.split_dgemm(A, B, Ct, fp, p.levels, p.slices, fmt=p.fmt)
            torch.cuda.synchronize()
            tuned = {"plan": {"alg": p.alg, "levels": p.levels, "slices": p.slices, "fmt": p.fmt},
                     "shape_plan_slices": tuner.plan(n, n, n, "split", 1e-10).slices,
                     "max_rel": float((Ct - ref).abs().max()) / rmax}
            del Ct
            if fp is not None:
                fmm.free_fmm(fp)
            for name, (f, L) in algs.items():
                Cf = torch.zeros_like(ref)
                fmm.dgemm(A, B, Cf, f, L)
                torch.cuda.synchronize()
                e64 = float((Cf - ref).abs().max())
                del Cf
                errs = {}
                for fmt, slices in (("bf16", range(3, 8)), ("fp8", range(7, 13))):
                    for s in slices:
                        Cs = torch.zeros_like(ref)
                        fmm.split_dgemm(A, B, Cs, f, L, s, fmt=fmt)
                        torch.cuda.synchronize()
                        d = Cs - ref
                        errs[f"{fmt}/{s}"] = {"max": float(d.abs().max()), "max_rel": float(d.abs().max()) / rmax,
                                              "fro_rel": float(torch.linalg.norm(d)) / rfro,
                                              "ratio_to_fp64_fmm": float(d.abs().max()) / e64 if e64 > 0 else None}
                        del Cs, d
                rows.append({"n": n, "inputs": dist, "alg": name, "levels": L, "fp64_fmm_max_err": e64,
                             "fp64_fmm_max_rel": e64 / rmax, "split": errs, "tuner_1e-10": tuned})
            del A, B, ref
            torch.cuda.empty_cache()
    for f, _ in algs.values():
        fmm.free_fmm(f)
    assert fmm.take_device_error() == 0
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": None, "unit": "TFLOP/s", "n_gpus": 1, "steps": 1,
                          "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
                          "config": {"workload": "split accuracy per slice count, BF16 and FP8-E4M3 slices "
                                                 "(222 x2, 333 x1; n = 8192, 16384; uniform and wide-range inputs)"},
                          "rows": rows}))


def run_batch(args, fmm, dev, world, rank, barrier, max_over_ranks):
    """Batched uneven FMM: `count` independent GEMMs (m, n, k log-uniform in
    [256, 8192], entries uniform [-1, 1), seeded) per step, each with the
    plan the Tuner picks for it; one fmm_gpu_batch_dgemm call per step (one
    persistent launch for FP64 problems, persistent waves of up to 80 split
    problems, bounded by the workspace). The split-BF16 run at the target
    error is the line's value; the all-FP64 run is reported beside it."""
    import torch

    from fmm_blis_gb300 import serve, tune

    tuner = tune.Tuner()
    shapes = batch_shapes(args.count, 2024 + rank)
    algs = {}

    def alg(name):
        if name == "classical":
            return None
        if name not in algs:
            algs[name] = fmm.new_fmm(COEFFS / f"{name}.txt")
        return algs[name]

    g = torch.Generator(device=dev).manual_seed(77 + rank)
    ops = [(serve._colmajor_rand(torch, m, k, g, dev), serve._colmajor_rand(torch, k, n, g, dev),
            serve._colmajor_rand(torch, m, n, g, dev)) for m, n, k in shapes]
    flops = sum(2.0 * m * n * k for m, n, k in shapes)
    stream = torch.cuda.current_stream()
    results = {}
    for form in ("split",) if args.no_fp64 else ("split", "fp64"):
        plans = [tuner.plan(m, n, k, form, args.target) for m, n, k in shapes]
        probs = [{"A": A, "B": B, "C": C, "fmm": alg(p.alg), "levels": p.levels, "slices": p.slices, "fmt": p.fmt}
                 for (A, B, C), p in zip(ops, plans)]
        arr = fmm.make_batch(probs)
        need = fmm.batch_workspace_size(arr)
        free = torch.cuda.mem_get_info(dev)[0]
        ws_bytes = int(min(need, max(free - (8 << 30), 1 << 30)))
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        steps, warm = (args.steps, args.warmup) if form == "split" else (1, 1)
        for _ in range(warm):
            fmm.batch_dgemm(arr, workspace=ws, stream=stream)
        torch.cuda.synchronize()
        barrier()
        n0 = fmm.launch_count()
        fmm.read_kernel_timing()
        fmm.set_kernel_timing(form == "split")
        with Clocks(torch.cuda.current_device()) as clk:
            total = timed_steps(torch, stream, steps, lambda: fmm.batch_dgemm(arr, workspace=ws, stream=stream),
                                None)
            barrier()
        fmm.set_kernel_timing(False)
        ms = max_over_ranks(total / steps)
        gemm_ms, gemm_n, _ = fmm.read_kernel_timing()
        hist = {}
        for p in plans:
            key = f"{p.alg}x{p.levels}" + (f"/{p.fmt}{p.slices}" if p.slices else "")
            hist[key] = hist.get(key, 0) + 1
        results[form] = {"ms": ms, "tflops": world * flops / (ms / 1e3) / 1e12, "steps": steps,
                         "launches_per_step": (fmm.launch_count() - n0) / steps, "plans": hist,
                         "workspace_gib": ws_bytes / 2**30, "workspace_needed_gib": need / 2**30,
                         "gemm_kernel_ms_per_step": gemm_ms / steps if gemm_n else None,
                         "clocks": clk.summary()}
        del ws
        # accuracy of the split run against the FP64 classical result, on a sample
    errs = []
    for i in range(0, len(shapes), max(len(shapes) // 16, 1)):
        m, n, k = shapes[i]
        A, B, _ = ops[i]
        p = tuner.plan(m, n, k, "split", args.target)
        C1 = torch.zeros((n, m), dtype=torch.float64, device=dev).t()
        C2 = torch.zeros((n, m), dtype=torch.float64, device=dev).t()
        fmm.split_dgemm(A, B, C1, alg(p.alg), p.levels, p.slices, fmt=p.fmt)
        fmm.dgemm(A, B, C2, None, 0)
        torch.cuda.synchronize()
        errs.append(float((C1 - C2).abs().max() / C2.abs().max()))
    for f in algs.values():
        fmm.free_fmm(f)
    assert fmm.take_device_error() == 0
    if rank == 0:
        sp = results["split"]
        print(json.dumps({
            "metric": METRIC, "value": sp["tflops"], "unit": "TFLOP/s", "n_gpus": world, "steps": sp["steps"],
            "warmup": args.warmup, "ms_per_step": sp["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"batched uneven FMM: {args.count} GEMMs, m,n,k log-uniform [256, 8192], "
                                   f"split-BF16 at target relative error {args.target:g}, tuner plans",
                       "count": args.count, "total_gflop": flops / 1e9,
                       "l2": "operands of 512 problems (tens of GB) larger than L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "split_batch": sp, "fp64_batch": results.get("fp64"),
            "split_max_rel_err_sample": max(errs), "gpu_launches": sp["launches_per_step"] * sp["steps"],
            "clocks": sp["clocks"]}))


def host_operand(torch, fmm, n):
    """An n x n column-major float64 CPU tensor in the library's pinned host
    memory on huge pages (fmm.host_empty), as a caller of the host-buffer
    entry points would allocate its operands."""
    return torch.from_numpy(fmm.host_empty(n, n))


def huge_page_share(arrays):
    """Share of the arrays' bytes that the kernel backs with transparent huge
    pages (AnonHugePages of the overlapping /proc/self/smaps regions); None
    where smaps is unreadable."""
    spans = [(a.data_ptr(), a.data_ptr() + a.numel() * a.element_size()) for a in arrays]
    total = sum(hi - lo for lo, hi in spans)
    huge, cur = 0, False
    try:
        with open("/proc/self/smaps") as f:
            for line in f:
                head = line.split(None, 1)[0]
                if "-" in head and ":" not in head:
                    lo, hi = (int(x, 16) for x in head.split("-"))
                    cur = any(lo < b and hi > a for a, b in spans)
                elif cur and head == "AnonHugePages:":
                    huge += int(line.split()[1]) * 1024
    except OSError:
        return None
    return min(1.0, huge / total) if total else None


def copy_rates(torch, h_src, d_dst, h_dst, d_src, reps=3):
    """Host-link throughput with the caller's pinned buffers: best of `reps`
    host-to-device copies of h_src into d_dst and device-to-host copies of
    d_src into h_dst, timed with CUDA events on a side stream (GB/s)."""
    st = torch.cuda.Stream()
    nbytes = h_src.numel() * h_src.element_size()
    best = {"h2d": float("inf"), "d2h": float("inf")}
    for _ in range(reps):
        for kind, dst, src in (("h2d", d_dst, h_src), ("d2h", h_dst, d_src)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(st):
                e0.record()
                dst.copy_(src, non_blocking=True)
                e1.record()
            e1.synchronize()
            best[kind] = min(best[kind], e0.elapsed_time(e1))
    return {"h2d_gbs": nbytes / best["h2d"] / 1e6, "d2h_gbs": nbytes / best["d2h"] / 1e6}


def serve_window(torch, dev, rate, duration, split_fraction, target, seed, clocks=True):
    """Poisson arrivals at `rate` per second for `duration` seconds, m, n, k
    log-uniform in [128, 16384] (scaled down to fit HBM), each tagged
    split-BF16 at `target` (share split_fraction) or FP64 drop-in, served by
    the continuous-batching Server (per-form queues, HBM admission).
    Latency = completion - arrival; throughput = 2mnk of the requests that
    completed inside the window, over the window. Requests still unfinished
    at the end of the drain (2 x duration) count with their elapsed time."""
    from fmm_blis_gb300 import serve

    free, total = torch.cuda.mem_get_info(dev)
    srv = serve.Server(hbm_budget=int(free * 0.75), streams=4, max_batch=64, keep_results=False)
    reqs = serve.poisson_arrivals(rate, duration, seed=seed, split_fraction=split_fraction,
                                  target_rel_err=target, cap_bytes=int(free * 0.1))
    # warm-up: one request of each form and a small graph bucket
    srv.run([serve.Request(1024, 1024, 1024, "split", target, 1, 0.0),
             serve.Request(256, 256, 256, "split", target, 2, 0.0),
             serve.Request(1024, 1024, 1024, "fp64", target, 3, 0.0)])
    srv.completed.clear()
    clk = Clocks(torch.cuda.current_device()) if clocks else None
    if clk:
        clk.__enter__()
    t0 = time.perf_counter()
    srv.run(reqs, until_idle=True, max_s=duration * 2)
    t_end = time.perf_counter()
    if clk:
        clk.__exit__(None, None, None)
    done = [r for r in reqs if r.done is not None]
    lat = sorted(r.latency * 1e3 for r in done)
    open_lat = sorted((t_end - r.arrival) * 1e3 for r in reqs if r.done is None and r.rid >= 0)
    lat_all = sorted(lat + open_lat)
    flops_done = sum(r.flops for r in done if r.done <= t0 + duration)

    def pct(xs, q):
        return xs[min(len(xs) - 1, int(q * len(xs)))] if xs else None

    by_form = {}
    for form in ("split", "fp64"):
        ls = sorted(r.latency * 1e3 for r in done if r.form == form)
        lo = sorted((t_end - r.arrival) * 1e3 for r in reqs if r.form == form and r.done is None and r.rid >= 0)
        by_form[form] = {"arrivals": sum(1 for r in reqs if r.form == form), "completed": len(ls),
                         "p50_ms": pct(sorted(ls + lo), 0.50), "p99_ms": pct(sorted(ls + lo), 0.99)}
    out = {"rate_per_s": rate, "duration_s": duration, "split_fraction": split_fraction, "target_rel_err": target,
           "arrivals": len(reqs), "submitted": sum(1 for r in reqs if r.rid >= 0), "completed": len(done),
           "unfinished": len(open_lat), "p50_ms": pct(lat_all, 0.50), "p99_ms": pct(lat_all, 0.99),
           "p50_ms_completed": pct(lat, 0.50), "p99_ms_completed": pct(lat, 0.99),
           "sustained_tflops": flops_done / duration / 1e12, "by_form": by_form,
           "graph_path_requests": sum(1 for r in done if r.path == "graph"), "batches": srv.launched_batches,
           "peak_hbm_gib": srv.peak_used / 2**30, "hbm_budget_gib": srv.budget / 2**30,
           "placement_retries": srv.alloc_failures,
           "fp64_ctas": srv.fp64_ctas, "wall_s": t_end - t0}
    if clk:
        out["clocks"] = clk.summary()
    srv.close()
    return out


def run_serve(args, fmm, dev, world, rank, barrier, max_over_ranks):
    """Served GEMM stream (config 5): serve_window at --rate for --duration,
    --split-fraction split-tagged at --target, the rest FP64 drop-in."""
    import torch

    barrier()
    w = serve_window(torch, dev, args.rate, args.duration, args.split_fraction, args.target, seed=31 + rank)
    value = world * w["sustained_tflops"]
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": 1, "warmup": 1,
            "ms_per_step": w["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16+f64", "data": "synthetic",
            "config": {"workload": f"served GEMM stream: Poisson {args.rate:g}/s for {args.duration:g} s, "
                                   f"m,n,k log-uniform [128, 16384], {args.split_fraction:.0%} split-BF16 at "
                                   f"{args.target:g}, the rest FP64 drop-in",
                       "rate_per_s": args.rate, "duration_s": args.duration, "hbm_budget_gib": w["hbm_budget_gib"],
                       "l2": "operands resident per request; no flush", "parallelism": f"replicas x{world}"},
            **{k: v for k, v in w.items() if k not in ("rate_per_s", "duration_s", "hbm_budget_gib")}}))


def run_fp64(args, fmm, f, dev, world, rank, barrier, max_over_ranks):
    """The plain FP64 FMM as the timed step (one kernel launch per step,
    C := C + A*B, device operands), `e2e` through the host-buffer drop-in
    fmm_gpu_strassen_ab_ex; the classical FP64 GEMM of this library at the
    same shape is timed once beside it. The FP64 FMA pipe bounds this form:
    the roofline peak is the DFMA rate measured by fmm_gpu_fp64_pipe_rates."""
    import torch

    n, levels = args.n, args.levels
    flops = 2.0 * n ** 3
    g = torch.Generator(device=dev).manual_seed(1234 + rank)
    A = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    C0 = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    C = C0.clone()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        fmm.dgemm(A, B, C, f, levels, stream=stream)
    torch.cuda.synchronize()
    barrier()
    # operands smaller than twice L2: per-step events with an L2 flush between
    flush = l2_flush_buffer(torch, dev, 3 * n * n * 8)
    n_launch0 = fmm.launch_count()
    with Clocks(torch.cuda.current_device()) as clk:
        total = timed_steps(torch, stream, args.steps, lambda: fmm.dgemm(A, B, C, f, levels, stream=stream), flush)
        barrier()
    launches = fmm.launch_count() - n_launch0
    ms = max_over_ranks(total / args.steps)
    value = world * flops / (ms / 1e3) / 1e12
    # end to end through the host-buffer drop-in (fmm_gpu_strassen_ab_ex, bli_strassen_ab_ex's replacement) with
    # pinned host operands (fmm_gpu_host_alloc): every call uploads A, B and C and reads C back
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        hA, hB, hC = (host_operand(torch, fmm, n) for _ in range(3))
        hA.copy_(A)
        hB.copy_(B)
        hC.copy_(C0)
        fl = f if levels == 1 else fmm.kron(f, f)
        L = fmm.lib()

        def host_step():
            st = L.fmm_gpu_strassen_ab_ex(1.0, hA.data_ptr(), n, hB.data_ptr(), n, 1.0, hC.data_ptr(), n, n, n, n, fl)
            assert st == 0, st

        host_step()   # sizes the call's device buffers
        with Clocks(torch.cuda.current_device()) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                host_step()
            ms_e2e = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
        fmm.release_host_buffers()
        link = copy_rates(torch, hA, A, hC, C)
        op = n * n * 8
        e2e = {"value": flops / ms_e2e / 1e9, "unit": "TFLOP/s", "h2d_bytes_per_step": 3 * op,
               "d2h_bytes_per_step": op, "ms_per_step": ms_e2e,
               "call": "fmm_gpu_strassen_ab_ex (host buffers; device buffers kept between calls)",
               "host_buffers": "fmm_gpu_host_alloc (pinned, huge pages)",
               "link": {**link, "serial_copies_ms": 3 * op / link["h2d_gbs"] / 1e6 + op / link["d2h_gbs"] / 1e6},
               "clocks": clk_e2e.summary()}
        if levels != 1:
            fmm.free_fmm(fl)
    mt, kt, nt, R = f.m_tilde ** levels, f.k_tilde ** levels, f.n_tilde ** levels, f.R ** levels
    executed = 2.0 * (-(-n // mt)) * (-(-n // nt)) * (-(-n // kt)) * R
    clk_sum = clk.summary()
    # peak: the FP64 pipe's nominal rate, 2 FMA/clock/SM, with this GPU's SM count and its maximum SM clock (the
    # classical FP64 GEMM of this library reaches 99.5% of it at 16384^3); the compute-only probes of the DFMA and
    # FP64 MMA paths are reported beside it (they compare the two paths and stay below the pipe's rate)
    dfma_probe, dmma_probe, mixed_probe = fmm.fp64_pipe_rates()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_max = clk_sum.get("sm_max_mhz") or 2070.0
    peak = 2.0 * 2.0 * sms * sm_max * 1e6 / 1e12
    achieved = executed / (ms / 1e3) / 1e12
    extra = {}
    if rank == 0 and not args.no_fp64:
        Cc = C0.clone()
        Cf = C0.clone()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        fmm.dgemm(A, B, Cc, None, 0, stream=stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms_cls = t0.elapsed_time(t1)
        fmm.dgemm(A, B, Cf, f, levels, stream=stream)
        torch.cuda.synchronize()
        amax, bmax = float(A.abs().max()), float(B.abs().max())
        err = float((Cf - Cc).abs().max())
        extra = {"fp64_classical": {"tflops": flops / ms_cls / 1e9, "ms": ms_cls},
                 "fp64_fmm_vs_classical": ms_cls / ms,
                 "max_err_vs_classical": err,
                 "err_over_eps_k_amax_bmax": err / (2.0 ** -52 * n * amax * bmax)}
    assert fmm.take_device_error() == 0
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plain FP64 FMM {args.alg} x{levels} levels, m=n=k={n}", "m": n, "n": n, "k": n,
                       "alg": args.alg, "levels": levels,
                       "l2": ("L2 flushed between steps (per-step events)" if flush is not None
                              else "inputs larger than L2; no flush"),
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "fp64_pipe", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "fmm_f64_kernel",
                         "peak_kind": "nominal DFMA rate: 2 FMA/clock/SM x SMs (queried) x max SM clock (nvidia-smi)",
                         "executed_flops_per_step": executed},
            "fp64_pipes": {"dfma_probe_tflops": dfma_probe, "dmma_probe_tflops": dmma_probe,
                           "dfma_and_dmma_probe_tflops": mixed_probe, "sms": sms},
            "cpu_baseline": None, "e2e": e2e, "gpu_launches": launches, "clocks": clk_sum, **extra}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "serve":
        # a served mix keeps many streams busy (the server's, the library's side-work pool, graph slots): give
        # them their own hardware queues, so work behind a long FP64 batch on a shared queue does not wait for it
        # (read when the CUDA context is created, so before the first CUDA call)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch

    import fmm_blis_gb300 as fmm
    from fmm_blis_gb300 import build as fbuild

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    fbuild.build()
    if args.f64_engine:
        fmm.set_f64_engine(args.f64_engine)
    dev = torch.device("cuda", torch.cuda.current_device())
    n, levels, s = args.n, args.levels, args.slices
    f = fmm.new_fmm(COEFFS / f"{args.alg}.txt")
    flops = 2.0 * n ** 3

    def barrier():
        rank_barrier(world)

    def max_over_ranks(x: float) -> float:
        return rank_max(x, world, dev)

    if args.workload == "batch":
        run_batch(args, fmm, dev, world, rank, barrier, max_over_ranks)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload in ("sweep", "accuracy"):
        (run_sweep if args.workload == "sweep" else run_accuracy)(args, fmm, dev, rank)
        return
    if args.workload == "serve":
        run_serve(args, fmm, dev, world, rank, barrier, max_over_ranks)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.form == "fp64":
        run_fp64(args, fmm, f, dev, world, rank, barrier, max_over_ranks)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    g = torch.Generator(device=dev).manual_seed(1234 + rank)
    A = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    C0 = (torch.rand((n, n), generator=g, device=dev, dtype=torch.float64) * 2 - 1).t()
    C = C0.clone()
    fmt = args.fmt
    ws = torch.empty(fmm.split_workspace_size(n, n, n, f, levels, s, fmt), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def step(Cx):
        fmm.split_dgemm(A, B, Cx, f, levels, s, workspace=ws, stream=stream, fmt=fmt)

    for _ in range(args.warmup):
        step(C)
    torch.cuda.synchronize()
    barrier()
    n_launch0 = fmm.launch_count()
    fmm.read_kernel_timing()
    fmm.set_kernel_timing(True)
    flush = l2_flush_buffer(torch, dev, 3 * n * n * 8)
    with Clocks(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        barrier()
        total = timed_steps(torch, stream, args.steps, lambda: step(C), flush)
        barrier()
    fmm.set_kernel_timing(False)
    launches = fmm.launch_count() - n_launch0
    ms = max_over_ranks(total / args.steps)
    gemm_ms, gemm_n, gemm_products = fmm.read_kernel_timing()
    value = world * flops / (ms / 1e3) / 1e12

    # dominant kernel roofline: executed MMA flops per GEMM launch (a launch
    # covers a group of products, each pairs * 2 * me^3); FP8 against twice
    # the measured BF16 peak (the nominal FP8:BF16 rate ratio)
    mt = f.m_tilde ** levels
    me = -(-n // mt)
    pairs = s * (s + 1) // 2
    kernel_flops = pairs * 2.0 * me * me * me * gemm_products / max(gemm_n, 1)
    avg_launch_s = (gemm_ms / max(gemm_n, 1)) / 1e3
    peak_sus, peak_burst, hbm, peak_kind = peaks()
    peak_kind = f"{peak_kind} bf16 sustained"
    if fmt == "fp8":
        peak_sus, peak_kind = 2 * peak_sus, f"2x {peak_kind} (FP8 nominal ratio)"
    achieved = kernel_flops / avg_launch_s / 1e12
    # DRAM traffic per GEMM launch: the small-case capture (m=n=k=4096, ncu, one launch) per work item, times the
    # items of this workload's launches. At 16384 the concurrent tiles' slice panels exceed L2 by more, so this
    # scaled figure is a lower bound there.
    traffic, traffic_src = None, None
    tf = ROOT / "profiles" / "split_gemm_pair_kernel_traffic_222x2_4096.json"
    if tf.exists() and fmt == "bf16" and me >= 1024:
        cap = json.loads(tf.read_text())
        items_per_launch = (gemm_products / max(gemm_n, 1)) * (-(-me // 256)) ** 2
        traffic = (cap["dram_read"] + cap["dram_write"]) / cap["items"] * items_per_launch
        traffic_src = (f"ncu capture at m=n=k=4096 ({cap['items']} items), scaled by work items to "
                       f"{items_per_launch:.0f} items per launch; a lower bound at larger sizes")
    # single calls take 256 x 256 CTA-pair tiles once m_e >= 1024
    kernel = "split_gemm_pair_kernel" if me >= 1024 else "split_gemm_kernel"
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak_sus, "unit": "TFLOP/s",
                "frac": achieved / peak_sus, "traffic": traffic, "traffic_source": traffic_src,
                "kernel": kernel, "peak_kind": peak_kind,
                "flops_per_launch": kernel_flops, "avg_launch_ms": avg_launch_s * 1e3, "launches_timed": gemm_n,
                "products_per_launch": gemm_products / max(gemm_n, 1)}

    # end to end through the host-buffer C-ABI call (fmm_gpu_split_strassen_ab_ex)
    # with pinned host operands (fmm_gpu_host_alloc): every step uploads A, B and C and reads C back
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        hA, hB, hC = (host_operand(torch, fmm, n) for _ in range(3))
        hA.copy_(A)
        hB.copy_(B)
        hC.copy_(C0)
        torch.cuda.synchronize()

        def host_step():
            fmm.split_strassen_ab_ex(1.0, hA, hB, 1.0, hC, f, levels, s, fmt)

        host_step()   # sizes the call's device buffers
        with Clocks(torch.cuda.current_device()) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                host_step()
            ms_e2e = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
        # one more call with its timeline recorded (CUDA events inside the call), outside the timed steps
        fmm.set_host_timeline(True)
        host_step()
        fmm.set_host_timeline(False)
        timeline = fmm.read_host_timeline()
        fmm.release_host_buffers()
        # the host link on this machine, with the same pinned buffers: one operand up, C down (CUDA events)
        link = copy_rates(torch, hA, A, hC, C)
        op_bytes = n * n * 8
        up_ab = 2 * op_bytes / link["h2d_gbs"] / 1e6
        e2e = {"value": flops / ms_e2e / 1e9, "unit": "TFLOP/s", "h2d_bytes_per_step": 3 * n * n * 8,
               "d2h_bytes_per_step": n * n * 8, "ms_per_step": ms_e2e,
               "call": "fmm_gpu_split_strassen_ab_ex (host buffers, copies overlapped with the device work)",
               "host_buffers": "fmm_gpu_host_alloc (pinned, huge pages)",
               "link": {**link,
                        "serial_copies_ms": 3 * op_bytes / link["h2d_gbs"] / 1e6 + op_bytes / link["d2h_gbs"] / 1e6,
                        "upload_A_B_ms": up_ab,
                        # the call's GEMM starts once A and the first half of B's columns are up, and the call
                        # ends once C's last column chunk (1/8 of C) is down after the GEMM
                        "before_gemm_ms": 1.5 * op_bytes / link["h2d_gbs"] / 1e6,
                        "after_gemm_ms": op_bytes / 8 / link["d2h_gbs"] / 1e6},
               "host_huge_page_share": huge_page_share([hA, hB, hC]),
               "timeline_ms": timeline,
               "clocks": clk_e2e.summary()}

    extra = {}
    if rank == 0 and not args.no_fp64:
        # classical FP64 reference result and the plain FP64 FMM, once
        Cc = C0.clone()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        fmm.dgemm(A, B, Cc, None, 0, stream=stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms_cls = t0.elapsed_time(t1)
        Cf = C0.clone()
        t0.record(stream)
        fmm.dgemm(A, B, Cf, f, levels, stream=stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms_fmm = t0.elapsed_time(t1)
        Cs = C0.clone()
        step(Cs)
        torch.cuda.synchronize()
        err_fmm = float((Cf - Cc).abs().max())
        err_split = float((Cs - Cc).abs().max())
        del Cf, Cs, Cc
        extra = {
            "fp64_fmm": {"tflops": flops / ms_fmm / 1e9, "ms": ms_fmm, "max_err_vs_classical": err_fmm},
            "fp64_classical": {"tflops": flops / ms_cls / 1e9, "ms": ms_cls},
            "split": {"slices": s, "max_err_vs_classical": err_split,
                      "err_ratio_to_fp64_fmm": err_split / err_fmm if err_fmm > 0 else None},
            "speedup_split_vs_fp64_fmm": (flops / ms / 1e9) / (flops / ms_fmm / 1e9),
            "fp64_fmm_vs_classical": ms_cls / ms_fmm,
        }

    cpu = None
    if rank == 0 and not args.no_cpu:
        eff, info = cpu_reference(args.alg, levels, n, 15.0,
                                  [np.asfortranarray(X.cpu().numpy()) for X in (A, B, C0)])
        cpu = {"value": eff, "unit": "TFLOP/s", "cores": info["cores"], "kind": "port",
               "sample": (f"oracle FP64 FMM {args.alg} x{levels} at m=n=k={n}: products 0..{info['products'] - 1} "
                          f"of {info['of']} ({info['seconds']:.1f} s; value = their share of 2mnk over that time)")}

    served = None
    if rank == 0 and args.serve_seconds > 0:
        # config 5's served stream, bounded: Poisson 200/s for serve_seconds, split-tagged at 1e-10
        served = serve_window(torch, dev, 200.0, args.serve_seconds, 1.0, 1e-10, seed=31)

    assert fmm.take_device_error() == 0
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp8_e4m3" if fmt == "fp8" else "bf16", "data": "synthetic",
            "config": {"workload": f"split-{fmt.upper()} FMM {args.alg} x{levels} levels, m=n=k={n}, {s} slices",
                       "m": n, "n": n, "k": n, "alg": args.alg, "levels": levels, "slices": s, "fmt": fmt,
                       "l2": ("L2 flushed between steps (per-step events)" if flush is not None
                              else f"inputs (3 x {n * n * 8 / 2**30:.2f} GiB) larger than L2; no flush"),
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(), **extra,
        }
        if served is not None:
            out["served"] = served
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
