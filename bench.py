"""Benchmark of the exhaustive k-NN path on GB300.

Workload (one step): allknn self-join with NormCosine over n = 1,000,000
Float32 vectors of d = 96 drawn from a 1,000-cluster Gaussian mixture
(centres N(0,1), per-cluster sigma U[0.1, 0.5]) and L2-normalised; k = 32
neighbours excluding the object itself.  Inputs are seeded synthetic data.

Arms:
  default            the GPU engine (libssgpu.so) -- prints one JSON line
  --impl reference   the reference algorithm on the host cores: the oracle's
                     restatement of ExhaustiveSearch + allknn (the Julia
                     reference cannot run on this machine), timed on a bounded
                     sample of the same workload

The timed device region has the database resident in HBM (384 MB, larger than
the 129 MB L2, so no flush is needed between steps).  ``e2e`` repeats the step
through the public C ABI from pinned host memory: upload the database, run
allknn, read the (k, n) ids and distances back.
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DB = 1_000_000
DIM = 96
K = 32
N_CENTRES = 1000


def load_package():
    name = "similaritysearch_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "similaritysearch.jl_gb300")
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def make_mixture(n: int = N_DB, d: int = DIM, centres: int = N_CENTRES) -> np.ndarray:
    """Seeded Gaussian mixture, L2-normalised rows (n, d) Float32."""
    C_ = np.random.default_rng(3).standard_normal((centres, d), dtype=np.float32)
    sig = np.random.default_rng(4).uniform(0.1, 0.5, size=centres).astype(np.float32)
    g = np.random.default_rng(5)
    lab = g.integers(0, centres, size=n)
    X = g.standard_normal((n, d), dtype=np.float32)
    X *= sig[lab, None]
    X += C_[lab]
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    return X


class ClockSampler:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(X: np.ndarray, budget_s: float = 12.0, rows=None):
    """Times the oracle's allknn restatement (ExhaustiveSearch semantics,
    @simd-style 16-lane sums, all host threads) on a sample of query rows."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(21)
    probe = rng.choice(X.shape[0], size=32, replace=False)
    t0 = time.perf_counter()
    O.allknn_rows("normcosine", X, K + 1, probe, lanes=16, nthreads=threads)
    dt = time.perf_counter() - t0
    per_row = dt / probe.size
    nrows = int(max(64, min(20000, budget_s / max(per_row, 1e-6))))
    if rows is None:
        rows = rng.choice(X.shape[0], size=nrows, replace=False)
    t0 = time.perf_counter()
    ids, dists = O.allknn_rows("normcosine", X, K + 1, rows, lanes=16, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": rows.size / dt, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{rows.size} query rows of the allknn workload against all {X.shape[0]} objects "
                      f"(k+1={K + 1}), oracle C restatement, 16-lane sums, {threads} OpenMP threads",
            "seconds": dt}, rows, ids, dists


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    X = make_mixture(N_DB)
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(22)
    # size each step so the whole run stays within a few minutes
    probe = rng.choice(X.shape[0], size=32, replace=False)
    t0 = time.perf_counter()
    O.allknn_rows("normcosine", X, K + 1, probe, lanes=16, nthreads=threads)
    per_row = (time.perf_counter() - t0) / probe.size
    total_budget = 120.0
    rows_per_step = int(max(32, min(20000, total_budget / max(1, args.steps + args.warmup) / max(per_row, 1e-6))))
    times = []
    for s in range(args.warmup + args.steps):
        rows = rng.choice(X.shape[0], size=rows_per_step, replace=False)
        t0 = time.perf_counter()
        O.allknn_rows("normcosine", X, K + 1, rows, lanes=16, nthreads=threads)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    tmean = sum(times) / len(times)
    qps = rows_per_step / tmean
    sample = (f"{rows_per_step} query rows per step of the allknn workload (n={N_DB}, d={DIM}, "
              f"k={K} excluding self) against all objects, oracle C restatement of ExhaustiveSearch/allknn "
              f"(reference is Julia, absent), 16-lane sums, {threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": config_dict("fp32"),
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


METRIC = "queries/s @ recall@10>=0.99 (allknn NormCosine n=1e6 d=96 k=32 excl. self)"
DATA = ("synthetic: seeded 1000-cluster Gaussian mixture (centres N(0,1), sigma U[0.1,0.5]), "
        "L2-normalised, n=1,000,000, d=96")


def config_dict(mode):
    return {"workload": "allknn self-join NormCosine, n=1,000,000, d=96, k=32 excluding self",
            "n": N_DB, "d": DIM, "k": K, "exclude_self": True, "mode": mode,
            "l2_policy": "inputs larger than L2 (384 MB database > 129 MB L2); no flush",
            "parallelism": "replicas only (one independent index per GPU)"}


def gpu_arm(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    ss = load_package()
    ss.build()
    N = ss._native
    L = N.lib()

    X = make_mixture(N_DB)
    n, d = X.shape
    mode = args.mode

    # --- device-resident timing -------------------------------------------------
    stream = torch.cuda.current_stream()
    h = C.c_void_p()
    N.check(L.ssg_create(N.METRIC_NORMCOSINE, N.ELEM_F32, d, n, X.ctypes.data_as(C.c_void_p), d,
                         {"fp32": N.PREC_FP32, "bf16": N.PREC_BF16, "fp8": N.PREC_FP8}[mode], C.byref(h)))
    N.check(L.ssg_set_stream(h, C.c_void_p(stream.cuda_stream)), h)
    if args.overfetch is not None:
        N.check(L.ssg_set_param(h, b"overfetch", float(args.overfetch)), h)
    ids_d = torch.empty((n, K), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((n, K), dtype=torch.float32, device="cuda")

    def step():
        N.check(L.ssg_allknn_device(h, K, 1, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dists_d.data_ptr())), h)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    N.check(L.ssg_set_param(h, b"profile", 1.0), h)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
            v = C.c_double()
            L.ssg_get_param(h, b"kernel_launches", C.byref(v))
            launches += int(v.value)
        e1.record(stream)
        torch.cuda.synchronize()
    t_ms = e0.elapsed_time(e1)
    if world > 1:
        dist.barrier()
    v = C.c_double()
    L.ssg_get_param(h, b"main_kernel_ms", C.byref(v))
    main_ms = v.value
    L.ssg_get_param(h, b"main_kernel_launches", C.byref(v))
    main_launches = int(v.value)
    N.check(L.ssg_set_param(h, b"profile", 0.0), h)

    t_max = t_ms
    if world > 1:
        tt = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    ms_per_step = t_max / args.steps
    qps = world * n * args.steps / (t_max / 1e3)

    ids_host = ids_d.cpu().numpy().view(np.uint32)
    dists_host = dists_d.cpu().numpy()
    L.ssg_destroy(h)

    # --- end to end through the C ABI from pinned host memory -------------------
    Xp = torch.from_numpy(X).pin_memory()
    oi = torch.empty((n, K), dtype=torch.int32).pin_memory()
    od = torch.empty((n, K), dtype=torch.float32).pin_memory()
    prec = {"fp32": N.PREC_FP32, "bf16": N.PREC_BF16, "fp8": N.PREC_FP8}[mode]

    def e2e_step():
        hh = C.c_void_p()
        N.check(L.ssg_create(N.METRIC_NORMCOSINE, N.ELEM_F32, d, n, C.c_void_p(Xp.data_ptr()), d, prec,
                             C.byref(hh)))
        try:
            if args.overfetch is not None:
                N.check(L.ssg_set_param(hh, b"overfetch", float(args.overfetch)), hh)
            N.check(L.ssg_allknn(hh, K, 1, C.c_void_p(oi.data_ptr()), C.c_void_p(od.data_ptr())), hh)
        finally:
            L.ssg_destroy(hh)

    e2e_steps = max(1, min(args.steps, 3))
    e2e_step()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        tt = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e_qps = world * n * e2e_steps / e2e_s

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # --- roofline of the dominant (scan) kernel ---------------------------------
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    avg_launch_ms = main_ms / max(1, main_launches)
    queries_per_launch = n * args.steps / max(1, main_launches)
    flops_per_launch = 2.0 * queries_per_launch * n * d
    achieved = flops_per_launch / (avg_launch_ms / 1e3) / 1e12
    if mode == "fp32":
        # FP32 SIMT peak: 152 SMs x 128 lanes x 2 flop x max SM clock (no measured FP32 peak exists)
        peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
        peak_note = "FP32 SIMT nominal at measured max SM clock (152x128x2xclk); not a measured copy/GEMM peak"
    else:
        peak = peaks.get("bf16_tflops", 1900.0)
        peak_note = "bf16_tflops of measured" if "bf16_tflops" in peaks else "bf16 fallback 1.9 PF"
    roof = {"bound": "tensor" if mode != "fp32" else "fp32", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None, "kernel": "scan",
            "per_launch_ms": avg_launch_ms, "flops_per_launch": flops_per_launch, "peak_note": peak_note}

    # --- CPU baseline + recall on the sampled rows --------------------------------
    if args.skip_cpu:
        print(json.dumps({"metric": METRIC, "value": qps, "unit": "queries/s", "n": n,
                          "ms_per_step": ms_per_step, "roofline": roof, "gpu_launches": launches}), flush=True)
        return
    cpu, rows, cids, cdists = cpu_baseline(X, budget_s=args.cpu_budget)
    # exclude self from the oracle rows like the GPU did
    gold = np.zeros((rows.size, K), dtype=np.uint32)
    for r, j in enumerate(rows):
        keep = [t for t in range(K + 1) if cids[r, t] != j + 1][:K]
        gold[r] = cids[r, keep]
    got = ids_host[rows]
    rec10 = float(np.mean([len(set(gold[r, :10]) & set(got[r, :10])) / 10 for r in range(rows.size)]))
    rec32 = float(np.mean([len(set(gold[r]) & set(got[r])) / K for r in range(rows.size)]))
    line = {
        "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if mode == "fp32" else mode, "data": DATA,
        "config": config_dict(mode),
        "recall": {"recall@10": rec10, "recall@32": rec32, "sample_rows": int(rows.size),
                   "gold": "oracle ExhaustiveSearch restatement (FP32, 16-lane sums)"},
        "roofline": roof,
        "cpu_baseline": {k: v for k, v in cpu.items() if k != "seconds"},
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": int(X.nbytes),
                "d2h_bytes_per_step": int(n * K * 8), "steps": e2e_steps},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    global N_DB
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--mode", default="fp32", choices=["fp32", "bf16", "fp8"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--n", type=int, default=N_DB,
                    help="database size (profiling captures use a smaller case of the same workload)")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline (profiling runs)")
    ap.add_argument("--overfetch", type=float, default=None,
                    help="candidates per neighbour kept by the reduced-precision scan")
    args = ap.parse_args()
    N_DB = args.n
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
