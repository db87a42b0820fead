"""Benchmark of the exhaustive k-NN path on GB300.

Headline workload (one step): allknn self-join with NormCosine over
n = 1,000,000 Float32 vectors of d = 96 drawn from a 1,000-cluster Gaussian
mixture (centres N(0,1), per-cluster sigma U[0.1, 0.5]) and L2-normalised;
k = 32 neighbours excluding the object itself.  Inputs are seeded synthetic
data of the shapes the benchmark names (no dataset is involved).

The metric is queries/s at recall@10 >= 0.99: the headline `value` is the
reduced-precision method (BF16 tensor-core distances over-fetching
1.25 x (k+1) candidates, re-ranked in exact FP32), whose recall against the
oracle is measured on a sample of rows in the same run; `modes.fp32` is the
plain FP32 method on the same data (same results as ExhaustiveSearch).

Arms:
  default            the GPU engine (libssgpu.so) -- prints one JSON line
  --impl reference   the reference algorithm on the host cores: the oracle's
                     restatement of ExhaustiveSearch + allknn (the Julia
                     reference cannot run on this machine), timed on a bounded
                     sample of the same workload

Other workloads of the benchmark suite (`--workload c1|c3|c4|c5`) print a
line of the same shape: C1 searchbatch SqL2 (d=128, n=100,000, m=1,000,
k=10); C3 Hamming (2,000,000 sketches of 1,024 bits, 10,000 queries at 10 %
bit flips, k=100); C4 a request stream of 200 uneven batches (1-4096
queries, k in {1, 10, 100}) over 2,000,000 vectors of d=768 in FP8 with the
exact rerank, per call and coalesced; C5 the learned shortlist on the C4
database.

The timed device region has the database resident in HBM (the C2 database is
384 MB FP32, larger than the 129 MB L2, so no flush is needed between steps).
``e2e`` repeats the step through the public C ABI from pinned host memory:
upload the database, run the search, read the (k, n) ids and distances back.
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
HEADLINE_MODE = "bf16"
HEADLINE_OVERFETCH = 1.25
HEADLINE_SCAN_TRAFFIC = 630.12e9 + 0.684e9

METRIC = "queries/s @ recall@10>=0.99 (allknn NormCosine n=1e6 d=96 k=32 excl. self)"
DATA = ("synthetic: seeded 1000-cluster Gaussian mixture (centres N(0,1), sigma U[0.1,0.5]), "
        "L2-normalised, n=1,000,000, d=96")


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


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def roofline_flops(mode, flops_per_launch, avg_launch_ms):
    """Roofline of a contraction kernel from its algorithmic flops per launch."""
    pk = peaks()
    achieved = flops_per_launch / (avg_launch_ms / 1e3) / 1e12
    if mode == "fp32":
        sm_max = pk.get("sm_max_mhz", 2070.0)
        # FP32 SIMT peak: 152 SMs x 128 lanes x 2 flop x the measured max SM clock
        peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
        note = "FP32 SIMT nominal at the measured max SM clock (152x128x2xclk): no measured FP32 peak exists"
        bound = "fp32"
    else:
        peak = pk.get("bf16_tflops", 1900.0)
        note = "bf16_tflops of measured" if "bf16_tflops" in pk else "bf16 fallback 1.9 PF"
        bound = "tensor"
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": None, "kernel": "scan", "per_launch_ms": avg_launch_ms,
            "flops_per_launch": flops_per_launch, "peak_note": note}


def roofline_bytes(bytes_per_launch, avg_launch_ms):
    pk = peaks()
    achieved = bytes_per_launch / (avg_launch_ms / 1e3) / 1e9
    peak = pk.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "scan", "per_launch_ms": avg_launch_ms, "bytes_per_launch": bytes_per_launch,
            "peak_note": "hbm_gbs of measured" if "hbm_gbs" in pk else "hbm fallback 6.8 TB/s"}


# ---------------------------------------------------------------------------
# CPU side: the oracle restatement (baseline and reference arm)
# ---------------------------------------------------------------------------

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
        "config": config_dict(HEADLINE_MODE, HEADLINE_OVERFETCH),
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict(mode, overfetch):
    return {"workload": "allknn self-join NormCosine, n=1,000,000, d=96, k=32 excluding self",
            "n": N_DB, "d": DIM, "k": K, "exclude_self": True, "mode": mode,
            "overfetch": overfetch if mode != "fp32" else None,
            "l2_policy": "inputs larger than L2 (384 MB database > 129 MB L2); no flush",
            "parallelism": "replicas only (one independent index per GPU)"}


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

class Ctx:
    def __init__(self):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(self.local)
        if self.world > 1:
            dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
        ss = load_package()
        ss.build()
        self.ss = ss
        self.N = ss._native
        self.L = self.N.lib()

    def max_over_ranks(self, v):
        return self.ss.shard.max_over_ranks(v, device="cuda")

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()


PREC = {"fp32": 0, "bf16": 1, "fp8": 2}


def timed_device_steps(cx, h, step, steps, warmup):
    """W untimed + K timed steps on the library's stream (torch's current
    stream); returns (ms per step max over ranks, launches, scan ms, scan launches, clocks)."""
    torch, N, L = cx.torch, cx.N, cx.L
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    N.check(L.ssg_set_param(h, b"profile", 1.0), h)
    cx.barrier()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(cx.local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
            v = C.c_double()
            L.ssg_get_param(h, b"kernel_launches", C.byref(v))
            launches += int(v.value)
        e1.record(stream)
        torch.cuda.synchronize()
    t_ms = cx.max_over_ranks(e0.elapsed_time(e1))
    cx.barrier()
    v = C.c_double()
    L.ssg_get_param(h, b"main_kernel_ms", C.byref(v))
    main_ms = v.value
    L.ssg_get_param(h, b"main_kernel_launches", C.byref(v))
    main_launches = int(v.value)
    N.check(L.ssg_set_param(h, b"profile", 0.0), h)
    return t_ms / steps, launches, main_ms, main_launches, clk.summary()


def allknn_mode(cx, X, mode, overfetch, steps, warmup):
    torch, N, L = cx.torch, cx.N, cx.L
    n, d = X.shape
    h = C.c_void_p()
    N.check(L.ssg_create(N.METRIC_NORMCOSINE, N.ELEM_F32, d, n, X.ctypes.data_as(C.c_void_p), d, PREC[mode],
                         C.byref(h)))
    N.check(L.ssg_set_stream(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)), h)
    if mode != "fp32" and overfetch is not None:
        N.check(L.ssg_set_param(h, b"overfetch", float(overfetch)), h)
    ids_d = torch.empty((n, K), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((n, K), dtype=torch.float32, device="cuda")

    def step():
        N.check(L.ssg_allknn_device(h, K, 1, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dists_d.data_ptr())), h)

    ms, launches, main_ms, main_launches, clocks = timed_device_steps(cx, h, step, steps, warmup)
    ids_host = ids_d.cpu().numpy().view(np.uint32)
    dists_host = dists_d.cpu().numpy()
    L.ssg_destroy(h)
    avg = main_ms / max(1, main_launches)
    q_per_launch = n * steps / max(1, main_launches)
    roof = roofline_flops(mode, 2.0 * q_per_launch * n * d, avg)
    if mode == "bf16" and n == 1_000_000 and d == 96 and main_launches == steps:
        # DRAM bytes (read + write) of one headline scan launch, from one ncu
        # capture of it (1-pass dram__bytes_read/write.sum metrics)
        roof["traffic"] = HEADLINE_SCAN_TRAFFIC
        roof["traffic_note"] = "dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture of this launch"
    return {"ms_per_step": ms, "qps": cx.world * n / (ms / 1e3), "launches": launches, "roofline": roof,
            "clocks": clocks, "ids": ids_host, "dists": dists_host}


def allknn_e2e(cx, X, mode, overfetch, steps):
    torch, N, L = cx.torch, cx.N, cx.L
    n, d = X.shape
    Xp = torch.from_numpy(X).pin_memory()
    oi = torch.empty((n, K), dtype=torch.int32).pin_memory()
    od = torch.empty((n, K), dtype=torch.float32).pin_memory()

    def e2e_step():
        hh = C.c_void_p()
        N.check(L.ssg_create(N.METRIC_NORMCOSINE, N.ELEM_F32, d, n, C.c_void_p(Xp.data_ptr()), d, PREC[mode],
                             C.byref(hh)))
        try:
            if mode != "fp32" and overfetch is not None:
                N.check(L.ssg_set_param(hh, b"overfetch", float(overfetch)), hh)
            N.check(L.ssg_allknn(hh, K, 1, C.c_void_p(oi.data_ptr()), C.c_void_p(od.data_ptr())), hh)
        finally:
            L.ssg_destroy(hh)

    e2e_step()
    cx.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e_step()
    torch.cuda.synchronize()
    s = cx.max_over_ranks(time.perf_counter() - t0)
    return {"value": cx.world * n * steps / s, "unit": "queries/s", "h2d_bytes_per_step": int(X.nbytes),
            "d2h_bytes_per_step": int(n * K * 8), "steps": steps}


def recall_vs(gold_rows, cids, got):
    """recall@10 / recall@32 of GPU rows against oracle rows (self removed)."""
    gold = np.zeros((gold_rows.size, K), dtype=np.uint32)
    for r, j in enumerate(gold_rows):
        keep = [t for t in range(K + 1) if cids[r, t] != j + 1][:K]
        gold[r] = cids[r, keep]
    g = got[gold_rows]
    r10 = float(np.mean([len(set(gold[r, :10]) & set(g[r, :10])) / 10 for r in range(gold_rows.size)]))
    r32 = float(np.mean([len(set(gold[r]) & set(g[r])) / K for r in range(gold_rows.size)]))
    return r10, r32


def fp64_check(X, got_ids, got_d, rows):
    """recall@10 / recall@32 against the FP64 oracle (self excluded) and the
    largest |reported distance - FP64 distance of the same id| on `rows`."""
    from oracle import oracle as O
    fi, _ = O.searchbatch_f64("normcosine", X, X[rows], K + 1, nthreads=os.cpu_count() or 1)
    gold = np.array([[i for i in fi[r] if i != j + 1][:K] for r, j in enumerate(rows)], dtype=np.uint32)
    g = got_ids[rows]
    r10 = float(np.mean([len(set(gold[r, :10]) & set(g[r, :10])) / 10 for r in range(rows.size)]))
    r32 = float(np.mean([len(set(gold[r]) & set(g[r])) / K for r in range(rows.size)]))
    dmax = 0.0
    for r, j in enumerate(rows):
        for t in range(K):
            i = int(g[r, t])
            if i:
                dmax = max(dmax, abs(float(got_d[j, t]) - O.evaluate_f64("normcosine", X[i - 1], X[j])))
    return {"recall@10": r10, "recall@32": r32, "max_abs_ddist": dmax, "sample_rows": int(rows.size)}


def gpu_arm(args):
    cx = Ctx()
    X = make_mixture(N_DB)
    n = X.shape[0]
    mode = args.mode
    of = args.overfetch if args.overfetch is not None else HEADLINE_OVERFETCH
    head = allknn_mode(cx, X, mode, of, args.steps, args.warmup)
    if args.skip_cpu:
        if cx.rank == 0:
            print(json.dumps({"metric": METRIC, "value": head["qps"], "unit": "queries/s", "n": n, "mode": mode,
                              "ms_per_step": head["ms_per_step"], "roofline": head["roofline"],
                              "gpu_launches": head["launches"]}), flush=True)
        return
    e2e = allknn_e2e(cx, X, mode, of, max(1, min(args.steps, 3)))
    modes = {mode: {"value": head["qps"], "ms_per_step": head["ms_per_step"], "roofline_frac":
                    head["roofline"]["frac"]}}
    plain = None
    if mode != "fp32" and not args.no_plain:
        plain = allknn_mode(cx, X, "fp32", None, 1, 1)
        modes["fp32"] = {"value": plain["qps"], "ms_per_step": plain["ms_per_step"],
                         "roofline": plain["roofline"], "note": "plain FP32 method, 1 warm-up + 1 timed step"}
    if cx.rank != 0:
        return
    cpu, rows, cids, _ = cpu_baseline(X, budget_s=args.cpu_budget)
    r10, r32 = recall_vs(rows, cids, head["ids"])
    f64 = fp64_check(X, head["ids"], head["dists"], rows[:256])
    modes[mode]["recall@10"], modes[mode]["recall@32"] = r10, r32
    if plain is not None:
        p10, p32 = recall_vs(rows, cids, plain["ids"])
        modes["fp32"]["recall@10"], modes["fp32"]["recall@32"] = p10, p32
        modes["speedup_vs_fp32"] = head["qps"] / plain["qps"]
    line = {
        "metric": METRIC, "value": head["qps"], "unit": "queries/s", "n_gpus": cx.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if mode == "fp32" else mode, "data": DATA,
        "config": config_dict(mode, of),
        "recall": {"recall@10": r10, "recall@32": r32, "sample_rows": int(rows.size),
                   "gold": "oracle ExhaustiveSearch restatement (FP32, 16-lane sums)", "vs_fp64": f64},
        "roofline": head["roofline"],
        "cpu_baseline": {k: v for k, v in cpu.items() if k != "seconds"},
        "e2e": e2e,
        "clocks": head["clocks"],
        "gpu_launches": head["launches"],
        "modes": modes,
    }
    print(json.dumps(line), flush=True)
    if cx.world > 1:
        cx.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Other workloads of the suite: C1 (SqL2 searchbatch) and C3 (Hamming)
# ---------------------------------------------------------------------------

def make_c1():
    X = np.random.default_rng(1).standard_normal((100_000, 128), dtype=np.float32)
    Q = np.random.default_rng(2).standard_normal((1_000, 128), dtype=np.float32)
    return X, Q, 10


def make_c3(n=2_000_000, m=10_000):
    W = 16
    X = np.random.default_rng(6).integers(0, 2**64 - 1, size=(n, W), dtype=np.uint64, endpoint=True)
    src = np.random.default_rng(7).integers(0, n, size=m)
    flips = np.random.default_rng(8).random((m, W * 64)) < 0.1
    mask = np.ascontiguousarray(np.packbits(flips, axis=1)).view(np.uint64)
    return X, X[src] ^ mask, 100


def workload_arm(args):
    cx = Ctx()
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    if args.workload == "c1":
        X, Q, k = make_c1()
        metric, elem, mname = N.METRIC_SQL2, N.ELEM_F32, "sql2"
        desc = "searchbatch SqL2, n=100,000, d=128, m=1,000, k=10 (N(0,1) data)"
    else:
        X, Q, k = make_c3(args.n if args.n is not None else 2_000_000)
        metric, elem, mname = N.METRIC_HAMMING, N.ELEM_U64, "hamming"
        desc = f"searchbatch Bits.Hamming, n={X.shape[0]:,} sketches x 1024 bits, m=10,000 (10% flips), k=100"
    mode = args.mode if args.workload == "c1" else "fp32"
    n, d = X.shape
    m = Q.shape[0]
    h = C.c_void_p()
    N.check(L.ssg_create(metric, elem, d, n, X.ctypes.data_as(C.c_void_p), d, PREC[mode], C.byref(h)))
    N.check(L.ssg_set_stream(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)), h)
    if mode != "fp32" and args.overfetch is not None:
        N.check(L.ssg_set_param(h, b"overfetch", float(args.overfetch)), h)
    Qd = torch.from_numpy(Q.view(np.int64) if Q.dtype == np.uint64 else Q).cuda()
    ids_d = torch.empty((m, k), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((m, k), dtype=torch.float32, device="cuda")

    def step():
        N.check(L.ssg_search_device(h, C.c_void_p(Qd.data_ptr()), m, k, C.c_void_p(ids_d.data_ptr()),
                                    C.c_void_p(dists_d.data_ptr()), 0), h)

    ms, launches, main_ms, main_launches, clocks = timed_device_steps(cx, h, step, args.steps, args.warmup)
    gi = ids_d.cpu().numpy().view(np.uint32)
    gd = dists_d.cpu().numpy()
    L.ssg_destroy(h)
    avg = main_ms / max(1, main_launches)
    if args.workload == "c1":
        roof = roofline_flops(mode, 2.0 * m * n * d, avg)
    else:
        # one pass over the sketches + the queries + the results (bytes per call)
        roof = roofline_bytes(8.0 * d * n + 8.0 * d * m + 8.0 * k * m, avg)
        roof["popcount_words_per_s"] = n * m * d / (avg / 1e3)
        # the binding roof at m = 1e4: 64-bit XOR + POPC issue, 16 32-bit
        # POPC per clock per SM = 8 words per clock per SM (nominal, at the
        # measured maximum SM clock; no measured INT peak exists)
        words_peak = 152 * 8 * peaks().get("sm_max_mhz", 2070.0) * 1e6
        roof["popcount_peak_words_per_s"] = words_peak
        roof["popcount_frac"] = roof["popcount_words_per_s"] / words_peak
    # e2e: create from host + search from host + results to host
    Xp = torch.from_numpy(X.view(np.int64) if X.dtype == np.uint64 else X).pin_memory()
    Qp = torch.from_numpy(Q.view(np.int64) if Q.dtype == np.uint64 else Q).pin_memory()
    oi = torch.empty((m, k), dtype=torch.int32).pin_memory()
    od = torch.empty((m, k), dtype=torch.float32).pin_memory()

    def e2e_step():
        hh = C.c_void_p()
        N.check(L.ssg_create(metric, elem, d, n, C.c_void_p(Xp.data_ptr()), d, PREC[mode], C.byref(hh)))
        try:
            if mode != "fp32" and args.overfetch is not None:
                N.check(L.ssg_set_param(hh, b"overfetch", float(args.overfetch)), hh)
            N.check(L.ssg_search(hh, C.c_void_p(Qp.data_ptr()), d, m, k, C.c_void_p(oi.data_ptr()),
                                 C.c_void_p(od.data_ptr()), 0), hh)
        finally:
            L.ssg_destroy(hh)

    e2e_step()
    t0 = time.perf_counter()
    for _ in range(2):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / 2
    # CPU baseline + parity on a sample of queries (oracle restatement)
    threads = os.cpu_count() or 1
    sample = np.random.default_rng(23).choice(m, size=min(m, args.cpu_queries), replace=False)
    t0 = time.perf_counter()
    ri, rd = O.searchbatch(mname, X, Q[sample], k, lanes=16 if mname != "hamming" else 1, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    parity = {"sample_queries": int(sample.size),
              "ids_equal": bool(np.array_equal(gi[sample], ri)) if mname == "hamming" else None,
              "dists_equal": bool(np.array_equal(gd[sample], rd)) if mname == "hamming" else None,
              "recall@k": O.macrorecall(ri, gi[sample])}
    if mname != "hamming":
        parity["max_rel_ddist"] = float(np.max(np.abs(gd[sample] - rd) / np.maximum(np.abs(rd), 1.0)))
    line = {"metric": f"queries/s ({args.workload})", "value": m / (ms / 1e3), "unit": "queries/s",
            "n_gpus": cx.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64" if mname == "hamming" else ("f32" if mode == "fp32" else mode),
            "data": "synthetic, seeded", "config": {"workload": desc, "mode": mode},
            "roofline": roof, "parity": parity,
            "cpu_baseline": {"value": sample.size / cpu_s, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{sample.size} queries against all {n:,} objects, oracle C restatement"},
            "e2e": {"value": m / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(X.nbytes + Q.nbytes),
                    "d2h_bytes_per_step": int(m * k * 8)},
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line), flush=True)


def make_c4(n=2_000_000, d=768, batches=200):
    """C4: 4,096-cluster mixture (sigma U[0.05, 0.3]) with log-normal(0, 0.25)
    norms; batch sizes round(LogNormal(ln 64, 1)) clipped to [1, 4096]; k
    uniform over {1, 10, 100}; queries drawn from the same mixture."""
    centres = np.random.default_rng(9).standard_normal((4096, d), dtype=np.float32)
    sig = np.random.default_rng(10).uniform(0.05, 0.3, size=4096).astype(np.float32)

    def draw(count, seed_lab, seed_norm):
        g = np.random.default_rng(seed_lab)
        out = np.empty((count, d), dtype=np.float32)
        for s0 in range(0, count, 250_000):
            c = min(250_000, count - s0)
            lab = g.integers(0, 4096, size=c)
            blk = g.standard_normal((c, d), dtype=np.float32)
            blk *= sig[lab, None]
            blk += centres[lab]
            blk /= np.linalg.norm(blk, axis=1, keepdims=True)
            out[s0:s0 + c] = blk
        out *= np.random.default_rng(seed_norm).lognormal(0.0, 0.25, size=(count, 1)).astype(np.float32)
        return out

    X = draw(n, 11, 12)
    sizes = np.clip(np.round(np.random.default_rng(13).lognormal(np.log(64), 1.0, size=batches)), 1, 4096)
    sizes = sizes.astype(np.int64)
    ks = np.random.default_rng(14).choice([1, 10, 100], size=batches)
    Q = draw(int(sizes.sum()), 15, 16)
    return X, Q, sizes, ks


def c4_arm(args):
    cx = Ctx()
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    X, Q, sizes, ks = make_c4(args.n if args.n is not None else 2_000_000, batches=args.batches)
    n, d = X.shape
    mode = args.mode if args.mode != "bf16" else "fp8"
    mname = args.metric
    metric = {"ip": N.METRIC_IP, "sql2": N.METRIC_SQL2}[mname]
    h = C.c_void_p()
    N.check(L.ssg_create(metric, N.ELEM_F32, d, n, X.ctypes.data_as(C.c_void_p), d, PREC[mode], C.byref(h)))
    N.check(L.ssg_set_stream(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)), h)
    Qd = torch.from_numpy(Q).cuda()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    kmax = int(ks.max())
    ids_d = torch.empty((int(sizes.max()), kmax), dtype=torch.int32, device="cuda")
    dd_d = torch.empty((int(sizes.max()), kmax), dtype=torch.float32, device="cuda")

    def run_stream(plain):
        N.check(L.ssg_set_param(h, b"plain", 1.0 if plain else 0.0), h)
        lat, results = [], []
        for b in range(len(sizes)):
            m, k = int(sizes[b]), int(ks[b])
            q = C.c_void_p(Qd.data_ptr() + int(offs[b]) * d * 4)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            N.check(L.ssg_search_device(h, q, m, k, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dd_d.data_ptr()), 0), h)
            torch.cuda.synchronize()
            lat.append(time.perf_counter() - t0)
            # the call writes m rows of k contiguously
            results.append(ids_d.view(-1)[:m * k].view(m, k).cpu().numpy().view(np.uint32).copy())
        return np.array(lat), results

    # over-fetch picked by the autotuner: smallest with recall@10 >= 0.99 on a
    # calibration sample against the plain method on the same index
    nc = min(2048, Q.shape[0])
    calib = Qd[:nc].contiguous()
    ci = torch.empty((nc, 10), dtype=torch.int32, device="cuda")
    cd = torch.empty((nc, 10), dtype=torch.float32, device="cuda")
    N.check(L.ssg_set_param(h, b"plain", 1.0), h)
    N.check(L.ssg_search_device(h, C.c_void_p(calib.data_ptr()), nc, 10, C.c_void_p(ci.data_ptr()),
                                C.c_void_p(cd.data_ptr()), 0), h)
    gold_c = ci.cpu().numpy().view(np.uint32).copy()
    N.check(L.ssg_set_param(h, b"plain", 0.0), h)
    chosen = None
    for c in (1.0, 1.25, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0, 16.0):
        N.check(L.ssg_set_param(h, b"overfetch", c), h)
        N.check(L.ssg_search_device(h, C.c_void_p(calib.data_ptr()), nc, 10, C.c_void_p(ci.data_ptr()),
                                    C.c_void_p(cd.data_ptr()), 0), h)
        if O.macrorecall(gold_c, ci.cpu().numpy().view(np.uint32)) >= 0.997:
            chosen = c
            break
    chosen = chosen or 16.0
    N.check(L.ssg_set_param(h, b"overfetch", chosen), h)
    calls = [0]

    def run_windows(window):
        """The same stream, `window` consecutive batches per ssg_search_batches
        call (one scan per window, CUDA-graph replay of repeated shapes)."""
        N.check(L.ssg_set_param(h, b"plain", 0.0), h)
        lat, results = [], []
        calls[0] = 0
        out_i = torch.empty(int((sizes * ks).sum()), dtype=torch.int32, device="cuda")
        out_d = torch.empty(int((sizes * ks).sum()), dtype=torch.float32, device="cuda")
        ooff = np.concatenate([[0], np.cumsum(sizes * ks)])
        for w0 in range(0, len(sizes), window):
            win = range(w0, min(len(sizes), w0 + window))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            # one call per window: the library packs the window's batches of
            # each distinct k into one search (so a k = 100 batch does not make
            # every batch of its window keep 100 candidates)
            bs = list(win)
            nb = len(bs)
            if nb:
                P = C.c_void_p * nb
                qp = P(*[Qd.data_ptr() + int(offs[b]) * d * 4 for b in bs])
                mp = (C.c_int64 * nb)(*[int(sizes[b]) for b in bs])
                kp = (C.c_int32 * nb)(*[int(ks[b]) for b in bs])
                ip = P(*[out_i.data_ptr() + int(ooff[b]) * 4 for b in bs])
                dp = P(*[out_d.data_ptr() + int(ooff[b]) * 4 for b in bs])
                N.check(L.ssg_search_batches(h, nb, qp, mp, kp, ip, dp), h)
                calls[0] += 1
            torch.cuda.synchronize()
            lat.append(time.perf_counter() - t0)
        allids = out_i.cpu().numpy().view(np.uint32)
        for b in range(len(sizes)):
            results.append(allids[ooff[b]:ooff[b + 1]].reshape(int(sizes[b]), int(ks[b])).copy())
        return np.array(lat), results

    run_stream(False)  # warm-up pass
    with ClockSampler(cx.local) as clk:
        lat_r, res_r = run_stream(False)
    window = max(1, args.window)
    # warm-up: the first pass sizes the buffers, the second sees each shape
    # once more (eager), the third captures the graphs; the timed pass replays
    for _ in range(3):
        run_windows(window)
    r0 = 0.0
    v = C.c_double()
    N.check(L.ssg_get_param(h, b"graph_replays", C.byref(v)), h)
    r0 = v.value
    lat_w, res_w = run_windows(window)
    N.check(L.ssg_get_param(h, b"graph_replays", C.byref(v)), h)
    replays = int(v.value - r0)
    lat_p, res_p = run_stream(True)
    # recall@10 of the reduced method against the plain method (k >= 10 batches)
    rec, cnt = 0.0, 0
    for b in range(len(sizes)):
        if ks[b] >= 10:
            rec += O.macrorecall(res_p[b][:, :10], res_r[b][:, :10]) * sizes[b]
            cnt += sizes[b]
    rec = rec / max(1, cnt)
    rec_w, cnt_w = 0.0, 0
    for b in range(len(sizes)):
        if ks[b] >= 10:
            rec_w += O.macrorecall(res_p[b][:, :10], res_w[b][:, :10]) * sizes[b]
            cnt_w += sizes[b]
    rec_w = rec_w / max(1, cnt_w)
    # FP64 oracle on a few queries of the first k>=10 batch
    b0 = int(np.nonzero(ks >= 10)[0][0])
    bq = np.nonzero((ks >= 10) & (sizes >= 8))[0]
    b0 = int(bq[0]) if bq.size else b0
    qs = Q[offs[b0]:offs[b0] + min(8, sizes[b0])]
    fi, _ = O.searchbatch_f64(mname, X, qs, 10, nthreads=os.cpu_count() or 1)
    r64_red = O.macrorecall(fi, res_r[b0][:qs.shape[0], :10])
    r64_pl = O.macrorecall(fi, res_p[b0][:qs.shape[0], :10])
    L.ssg_destroy(h)
    tq = int(sizes.sum())
    line = {"metric": "queries/s (c4 batched stream)", "value": tq / lat_r.sum(), "unit": "queries/s",
            "n_gpus": cx.world, "batches": int(len(sizes)), "higher_is_better": True, "vs_baseline": None,
            "dtype": mode, "data": "synthetic, seeded 4096-cluster mixture, log-normal norms",
            "config": {"workload": f"{'IP' if mname == 'ip' else 'SqL2'} request stream, n={n:,}, d={d}, "
                                   f"{len(sizes)} batches "
                                   f"(sizes LogNormal(ln 64,1) in [1,4096], k in {{1,10,100}})",
                       "mode": mode, "overfetch_autotuned": chosen,
                       "batching": "value: one ssg_search_device call per batch; coalesced: each window of "
                                   "consecutive batches in one ssg_search_batches call (one packed search "
                                   "per distinct k)"},
            "latency_ms": {"p50": float(np.percentile(lat_r, 50) * 1e3), "p99": float(np.percentile(lat_r, 99) * 1e3)},
            "recall@10_vs_plain": rec, "recall@10_vs_fp64_sample": {"reduced": r64_red, "plain": r64_pl,
                                                                    "queries": int(qs.shape[0])},
            "plain_fp32": {"value": tq / lat_p.sum(),
                           "latency_ms": {"p50": float(np.percentile(lat_p, 50) * 1e3),
                                          "p99": float(np.percentile(lat_p, 99) * 1e3)}},
            "speedup_vs_plain": float(lat_p.sum() / lat_r.sum()),
            "coalesced": {"window_batches": window, "value": tq / lat_w.sum(), "unit": "queries/s",
                          "latency_ms_per_window": {"p50": float(np.percentile(lat_w, 50) * 1e3),
                                                    "p99": float(np.percentile(lat_w, 99) * 1e3)},
                          "graph_replays": replays, "calls": calls[0], "recall@10_vs_plain": rec_w,
                          "speedup_vs_plain": float(lat_p.sum() / lat_w.sum())},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def c5_arm(args):
    """C5: the learned shortlist on the C4 database under SqL2 (768 -> 256 ->
    64 network, 200k-object sample, 5M triplets, 20 epochs, shortlist 512,
    exact FP32 rerank to k = 10) beside the plain FP32 method and the same
    pipeline with a 64-d random projection instead of the trained network."""
    cx = Ctx()
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    X, Q, _, _ = make_c4(args.n if args.n is not None else 2_000_000, batches=200)
    n, d = X.shape
    m, k = min(10_000, Q.shape[0]), 10
    Q = np.ascontiguousarray(Q[:m])
    h = C.c_void_p()
    N.check(L.ssg_create(N.METRIC_SQL2, N.ELEM_F32, d, n, X.ctypes.data_as(C.c_void_p), d, PREC["fp32"],
                         C.byref(h)))
    N.check(L.ssg_set_stream(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)), h)
    Qd = torch.from_numpy(Q).cuda()
    ids_d = torch.empty((m, k), dtype=torch.int32, device="cuda")
    dd_d = torch.empty((m, k), dtype=torch.float32, device="cuda")

    def get(key):
        v = C.c_double()
        N.check(L.ssg_get_param(h, key.encode(), C.byref(v)), h)
        return v.value

    def timed(steps, warmup):
        for _ in range(warmup):
            N.check(L.ssg_search_device(h, C.c_void_p(Qd.data_ptr()), m, k, C.c_void_p(ids_d.data_ptr()),
                                        C.c_void_p(dd_d.data_ptr()), 0), h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            N.check(L.ssg_search_device(h, C.c_void_p(Qd.data_ptr()), m, k, C.c_void_p(ids_d.data_ptr()),
                                        C.c_void_p(dd_d.data_ptr()), 0), h)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        return m / dt, dt * 1e3, ids_d.cpu().numpy().view(np.uint32).copy(), int(get("learned_used"))

    steps, warmup = max(1, args.steps), max(1, args.warmup)
    qps_plain, ms_plain, gold, _ = timed(1, 1)
    # random projection: the pipeline without a trained network
    N.check(L.ssg_set_param(h, b"learned_target", 0.0), h)
    N.check(L.ssg_train_mlp(h, 200_000, 0, 0, 0, 64, 1024, 1e-3, 15), h)
    rp_est = get("learned_recall")
    qps_rp, ms_rp, got_rp, _ = timed(steps, warmup)
    # the trained network
    N.check(L.ssg_set_param(h, b"learned_target", 0.99), h)
    N.check(L.ssg_train_mlp(h, 200_000, args.triplets, args.epochs, 256, 64, 1024, 1e-3, 15), h)
    stats = {key: get(key) for key in ("learned_recall", "train_loss", "train_seconds", "train_steps")}
    with ClockSampler(cx.local) as clk:
        qps_l, ms_l, got_l, used = timed(steps, warmup)
    # FP64 oracle on a sample of the queries
    ns = 16
    fi, _ = O.searchbatch_f64("sql2", X, Q[:ns], k, nthreads=os.cpu_count() or 1)
    L.ssg_destroy(h)
    line = {"metric": "queries/s (c5 learned shortlist)", "value": qps_l, "unit": "queries/s",
            "n_gpus": cx.world, "steps": steps, "warmup": warmup, "ms_per_step": ms_l, "higher_is_better": True,
            "vs_baseline": None, "dtype": "fp32 rerank, bf16-operand network",
            "data": "synthetic, seeded 4096-cluster mixture, log-normal norms",
            "config": {"workload": f"SqL2 searchbatch m={m}, k={k}, n={n:,}, d={d}; MLP {d}->256->64, "
                                   f"200k sample, {args.triplets:,} triplets, {args.epochs} epochs, shortlist 512",
                       "learned_used": used},
            "recall@10_vs_plain": O.macrorecall(gold, got_l),
            "recall@10_vs_fp64_sample": {"learned": O.macrorecall(fi, got_l[:ns]),
                                         "plain": O.macrorecall(fi, gold[:ns]), "queries": ns},
            "estimated_recall": stats["learned_recall"], "training": stats,
            "random_projection": {"value": qps_rp, "recall@10_vs_plain": O.macrorecall(gold, got_rp),
                                  "estimated_recall": rp_est},
            "plain_fp32": {"value": qps_plain, "ms_per_step": ms_plain},
            "speedup_vs_plain": qps_l / qps_plain, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    global N_DB
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--mode", default=HEADLINE_MODE, choices=["fp32", "bf16", "fp8"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 = the headline allknn workload; c1 / c3 = the suite's other searchbatch workloads")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--cpu-queries", type=int, default=64, help="c1/c3: queries timed on the CPU")
    ap.add_argument("--batches", type=int, default=200, help="c4: batches in the request stream")
    ap.add_argument("--triplets", type=int, default=5_000_000, help="c5: training triplets")
    ap.add_argument("--metric", default="ip", choices=["ip", "sql2"], help="c4: metric of the request stream")
    ap.add_argument("--window", type=int, default=8, help="c4: batches coalesced per ssg_search_batches call")
    ap.add_argument("--epochs", type=int, default=20, help="c5: training epochs")
    ap.add_argument("--n", type=int, default=None,
                    help="database size (profiling captures use a smaller case of the same workload)")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="omit the plain FP32 comparison run")
    ap.add_argument("--overfetch", type=float, default=None,
                    help="candidates per neighbour kept by the reduced-precision scan")
    args = ap.parse_args()
    if args.n is not None and args.workload == "c2":
        N_DB = args.n
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "c4":
        c4_arm(args)
    elif args.workload == "c5":
        c5_arm(args)
    elif args.workload != "c2":
        workload_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
