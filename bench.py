"""Benchmark of the exhaustive k-NN path on GB300.

Headline workload (one step): allknn self-join with NormCosine over
n = 1,000,000 Float32 vectors of d = 96 drawn from a 1,000-cluster Gaussian
mixture (centres N(0,1), per-cluster sigma U[0.1, 0.5]) and L2-normalised;
k = 32 neighbours excluding the object itself (C2).  Inputs are seeded
synthetic data of the shapes the benchmark names (no dataset is involved;
similaritysearch.jl_gb300/workloads.py generates them).

The metric is queries/s at recall@10 >= 0.99.  The headline `value` is the
reduced-precision method: BF16 tensor-core distances keeping
overfetch x (k+1) candidates per object, re-ranked in exact FP32.  The
over-fetch is the smallest of a fixed ladder whose recall@32 against the
plain method reaches 0.99 on calibration rows; recall is then reported on
other rows against the oracle and the FP64 ranking.  `modes.fp32` is the
plain FP32 method (results identical to ExhaustiveSearch's) as the library
runs it by default, on the tensor cores in two-piece BF16 form with the
exact rerank and completeness check, timed with the same steps;
`modes.fp32_cuda_cores` is the same method on the CUDA cores (FP32 FMA
GEMM form, its roofline against the FP32 peak), timed with fewer steps.

`suite` carries the other configurations in the same run, each with its own
roofline, CPU baseline, end-to-end figure and clocks: C1 (searchbatch SqL2,
d=128, n=100,000, m=1,000, k=10), C3 (Hamming over 2,000,000 sketches of
1,024 bits, k=100, at m=10,000 and at m=64), C4 (a request stream of 200
uneven batches over 2,000,000 vectors of d=768 in FP8 with the exact rerank,
IP and SqL2, per call and coalesced) and C5 (the learned shortlist on the C4
database beside the plain method and a random projection).

Arms:
  default            the GPU engine (libssgpu.so): one JSON line
  --impl reference   the reference algorithm on the host cores: the oracle's
                     restatement of ExhaustiveSearch + allknn (the Julia
                     reference cannot run on this machine), timed on a bounded
                     sample of the headline workload
  --workload cN      one configuration of the suite alone (profiling runs)

The timed device region has the database resident in HBM (the C2 database is
384 MB FP32, larger than the 129 MB L2, so no flush is needed between steps).
``e2e`` repeats the step through the public C ABI from pinned host memory:
upload the database, run the search, read the ids and distances back.
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
OVERFETCH_LADDER = (1.25, 1.5, 1.75)
# DRAM bytes (read + write) of one headline scan launch at n = 1e6 and
# over-fetch 1.5, from the one-pass ncu capture summarised in
# profiles/tc_wide_bf16_allknn.md
HEADLINE_SCAN_TRAFFIC = 56.662e9 + 0.815e9
HEADLINE_TRAFFIC_OVERFETCH = 1.5

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


def workloads():
    load_package()
    from similaritysearch_gb300 import workloads as W
    return W


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


def fp32_simt_peak_tflops():
    # FP32 SIMT peak: 152 SMs x 128 lanes x 2 flop x the measured max SM clock
    return 152 * 128 * 2 * peaks().get("sm_max_mhz", 2070.0) * 1e6 / 1e12


def roofline_flops(mode, flops_per_launch, avg_launch_ms):
    """Roofline of a contraction kernel from its algorithmic flops per launch."""
    pk = peaks()
    achieved = flops_per_launch / (avg_launch_ms / 1e3) / 1e12
    if mode == "fp32":
        peak = fp32_simt_peak_tflops()
        note = "FP32 SIMT nominal at the measured max SM clock (152x128x2xclk): no measured FP32 peak exists"
        bound = "fp32"
    else:
        peak = pk.get("bf16_tflops", 1900.0)
        note = "bf16_tflops of measured" if "bf16_tflops" in pk else "bf16 fallback 1.9 PF"
        bound = "tensor"
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": None, "kernel": "scan", "per_launch_ms": avg_launch_ms,
            "flops_per_launch": flops_per_launch, "peak_note": note}


def plain_tc_roofline(pairs, d, avg_launch_ms):
    """Roofline of the plain method's scan on the tensor cores: the two-piece
    BF16 products run over K = 3 kp (kp = d padded to 32)."""
    k3 = 3 * ((d + 31) // 32 * 32)
    r = roofline_flops("bf16", 2.0 * pairs * k3, avg_launch_ms)
    r["flops_note"] = ("tensor-core work of the two-piece scan, 2 x pairs x 3 kp (lo.hi + hi.lo + hi.hi); "
                       "the FP32 problem itself is 2 x pairs x d = %.4g flop per launch" % (2.0 * pairs * d))
    return r


def roofline_bytes(bytes_per_launch, avg_launch_ms, kernel="scan"):
    pk = peaks()
    achieved = bytes_per_launch / (avg_launch_ms / 1e3) / 1e9
    peak = pk.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": kernel, "per_launch_ms": avg_launch_ms, "bytes_per_launch": bytes_per_launch,
            "peak_note": "hbm_gbs of measured" if "hbm_gbs" in pk else "hbm fallback 6.8 TB/s"}


def recall_rows(gold, got, k):
    return float(np.mean([len(set(g[:k].tolist()) & set(r[:k].tolist())) / k for g, r in zip(gold, got)]))


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


def cpu_searchbatch_baseline(name, X, Q, k, budget_s=8.0, lanes=16):
    """The oracle's searchbatch restatement on all host threads over a sample
    of the queries sized to ~budget_s seconds: (baseline dict, sample, ids, dists)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(23)
    probe = rng.choice(Q.shape[0], size=min(Q.shape[0], 8), replace=False)
    t0 = time.perf_counter()
    O.searchbatch(name, X, Q[probe], k, lanes=lanes, nthreads=threads)
    per_q = (time.perf_counter() - t0) / probe.size
    nq = int(max(8, min(Q.shape[0], budget_s / max(per_q, 1e-6))))
    sample = np.sort(rng.choice(Q.shape[0], size=nq, replace=False))
    t0 = time.perf_counter()
    ri, rd = O.searchbatch(name, X, Q[sample], k, lanes=lanes, nthreads=threads)
    dt = time.perf_counter() - t0
    return ({"value": sample.size / dt, "unit": "queries/s", "cores": threads, "kind": "port",
             "sample": f"{sample.size} queries against all {X.shape[0]:,} objects, oracle C restatement "
                       f"({'integer popcounts' if name == 'hamming' else f'{lanes}-lane sums'}), {threads} threads"},
            sample, ri, rd)


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    X = workloads().make_c2(N_DB)
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
        "config": config_dict("bf16", None),
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict(mode, overfetch, calib=None):
    d = {"workload": "allknn self-join NormCosine, n=1,000,000, d=96, k=32 excluding self",
         "n": N_DB, "d": DIM, "k": K, "exclude_self": True, "mode": mode,
         "overfetch": overfetch if mode != "fp32" else None,
         "l2_policy": "inputs larger than L2 (384 MB database > 129 MB L2); no flush",
         "parallelism": "replicas only (one independent index per GPU)"}
    if calib is not None:
        d["overfetch_rule"] = ("smallest of %s whose recall@32 against the plain FP32 method reaches 0.99 on "
                               "%d calibration rows (disjoint from the reported recall rows)"
                               % (list(OVERFETCH_LADDER), calib["rows"]))
        d["overfetch_calibration"] = calib["recall@32"]
    return d


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

    def create(self, metric, elem, X, prec, **params):
        h = C.c_void_p()
        n, d = X.shape
        self.N.check(self.L.ssg_create(metric, elem, d, n, X.ctypes.data_as(C.c_void_p), d, prec, C.byref(h)))
        self.N.check(self.L.ssg_set_stream(h, C.c_void_p(self.torch.cuda.current_stream().cuda_stream)), h)
        for k, v in params.items():
            self.set(h, k, v)
        return h

    def set(self, h, key, value):
        self.N.check(self.L.ssg_set_param(h, key.encode(), float(value)), h)

    def get(self, h, key):
        v = C.c_double()
        self.N.check(self.L.ssg_get_param(h, key.encode(), C.byref(v)), h)
        return v.value

    def dev(self, A):
        """A host array as a device tensor (UInt64 sketches travel as int64)."""
        return self.torch.from_numpy(A.view(np.int64) if A.dtype == np.uint64 else A).cuda()

    def pinned(self, A):
        return self.torch.from_numpy(A.view(np.int64) if A.dtype == np.uint64 else A).pin_memory()


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
            launches += int(cx.get(h, "kernel_launches"))
        e1.record(stream)
        torch.cuda.synchronize()
    t_ms = cx.max_over_ranks(e0.elapsed_time(e1))
    cx.barrier()
    main_ms = cx.get(h, "main_kernel_ms")
    main_launches = int(cx.get(h, "main_kernel_launches"))
    N.check(L.ssg_set_param(h, b"profile", 0.0), h)
    return t_ms / steps, launches, main_ms, main_launches, clk.summary()


def allknn_once(cx, h, n):
    torch = cx.torch
    ids_d = torch.empty((n, K), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((n, K), dtype=torch.float32, device="cuda")
    cx.N.check(cx.L.ssg_allknn_device(h, K, 1, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dists_d.data_ptr())), h)
    torch.cuda.synchronize()
    return ids_d.cpu().numpy().view(np.uint32), dists_d.cpu().numpy()


def allknn_mode(cx, X, mode, overfetch, steps, warmup, **params):
    torch = cx.torch
    n, d = X.shape
    h = cx.create(cx.N.METRIC_NORMCOSINE, cx.N.ELEM_F32, X, PREC[mode], **params)
    if mode != "fp32" and overfetch is not None:
        cx.set(h, "overfetch", overfetch)
    ids_d = torch.empty((n, K), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((n, K), dtype=torch.float32, device="cuda")

    def step():
        cx.N.check(cx.L.ssg_allknn_device(h, K, 1, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dists_d.data_ptr())), h)

    ms, launches, main_ms, main_launches, clocks = timed_device_steps(cx, h, step, steps, warmup)
    ids_host = ids_d.cpu().numpy().view(np.uint32)
    dists_host = dists_d.cpu().numpy()
    plain_tc = mode == "fp32" and cx.get(h, "last_plain_tc") == 1.0
    fallbacks = cx.get(h, "fallbacks")
    cx.L.ssg_destroy(h)
    avg = main_ms / max(1, main_launches)
    q_per_launch = n * steps / max(1, main_launches)
    roof = (plain_tc_roofline(q_per_launch * n, d, avg) if plain_tc
            else roofline_flops(mode, 2.0 * q_per_launch * n * d, avg))
    if mode == "bf16" and n == 1_000_000 and d == 96 and main_launches == steps and overfetch == HEADLINE_TRAFFIC_OVERFETCH:
        roof["traffic"] = HEADLINE_SCAN_TRAFFIC
        roof["traffic_note"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one launch at over-fetch %.2f, "
                                "one ncu capture (profiles/tc_wide_bf16_allknn.md)" % HEADLINE_TRAFFIC_OVERFETCH)
    return {"ms_per_step": ms, "qps": cx.world * n / (ms / 1e3), "launches": launches, "roofline": roof,
            "clocks": clocks, "ids": ids_host, "dists": dists_host, "fallbacks": fallbacks, "plain_tc": plain_tc}


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


def oracle_gold_rows(gold_rows, cids):
    """Oracle allknn rows of k+1 (self included) -> k, self removed."""
    gold = np.zeros((gold_rows.size, K), dtype=np.uint32)
    for r, j in enumerate(gold_rows):
        keep = [t for t in range(K + 1) if cids[r, t] != j + 1][:K]
        gold[r] = cids[r, keep]
    return gold


def fp64_check(X, got_ids, got_d, rows):
    """recall@10 / recall@32 against the FP64 oracle (self excluded) and the
    largest |reported distance - FP64 distance of the same id| on `rows`."""
    from oracle import oracle as O
    fi, _ = O.searchbatch_f64("normcosine", X, X[rows], K + 1, nthreads=os.cpu_count() or 1)
    gold = np.array([[i for i in fi[r] if i != j + 1][:K] for r, j in enumerate(rows)], dtype=np.uint32)
    g = got_ids[rows]
    dmax = 0.0
    for r, j in enumerate(rows):
        for t in range(K):
            i = int(g[r, t])
            if i:
                dmax = max(dmax, abs(float(got_d[j, t]) - O.evaluate_f64("normcosine", X[i - 1], X[j])))
    return {"recall@10": recall_rows(gold, g, 10), "recall@32": recall_rows(gold, g, K), "max_abs_ddist": dmax,
            "sample_rows": int(rows.size)}


def choose_overfetch(cx, X, plain_ids, calib_rows):
    """The smallest over-fetch of the ladder whose BF16 allknn reaches
    recall@32 >= 0.99 against the plain method on the calibration rows."""
    h = cx.create(cx.N.METRIC_NORMCOSINE, cx.N.ELEM_F32, X, PREC["bf16"])
    tried = {}
    chosen = OVERFETCH_LADDER[-1]
    try:
        for of in OVERFETCH_LADDER:
            cx.set(h, "overfetch", of)
            ids, _ = allknn_once(cx, h, X.shape[0])
            r = recall_rows(plain_ids[calib_rows], ids[calib_rows], K)
            tried[str(of)] = r
            if r >= 0.99:
                chosen = of
                break
    finally:
        cx.L.ssg_destroy(h)
    return chosen, {"rows": int(calib_rows.size), "recall@32": tried}


def gpu_arm(args):
    cx = Ctx()
    W = workloads()
    X = W.make_c2(N_DB)
    n = X.shape[0]
    mode = args.mode
    rng = np.random.default_rng(24)
    calib_rows = np.sort(rng.choice(n, size=min(n, 20000), replace=False))
    plain = None
    modes = {}
    if mode != "fp32" and not args.no_plain:
        if cx.world == 1:
            plain = allknn_mode(cx, X, "fp32", None, args.steps, args.warmup)
            modes["fp32"] = {"value": plain["qps"], "ms_per_step": plain["ms_per_step"],
                             "roofline": plain["roofline"], "steps": args.steps, "warmup": args.warmup,
                             "fallbacks": plain["fallbacks"], "plain_on_tensor_cores": plain["plain_tc"],
                             "note": "plain FP32 method: results identical to ExhaustiveSearch's (lanes=1 sums); "
                                     "two-piece BF16 tensor-core scan, exact FP32 rerank, certified complete"}
            cc_steps = max(1, min(args.steps, 2))
            cc = allknn_mode(cx, X, "fp32", None, cc_steps, 1, plain_tc=0)
            modes["fp32_cuda_cores"] = {
                "value": cc["qps"], "ms_per_step": cc["ms_per_step"], "roofline": cc["roofline"],
                "steps": cc_steps, "warmup": 1, "fallbacks": cc["fallbacks"],
                "ids_equal_to_fp32": bool(np.array_equal(cc["ids"], plain["ids"])),
                "dists_equal_to_fp32": bool(np.array_equal(cc["dists"], plain["dists"])),
                "note": "the plain method on the CUDA cores (FP32 FMA GEMM form + exact rerank)"}
            del cc
        else:
            # replicas: the plain method runs once, untimed, for the over-fetch calibration
            plain = allknn_mode(cx, X, "fp32", None, 1, 0)
    calib = None
    if args.overfetch is not None:
        of = args.overfetch
    elif plain is not None:
        of, calib = choose_overfetch(cx, X, plain["ids"], calib_rows)
    else:
        of = OVERFETCH_LADDER[0]
    head = allknn_mode(cx, X, mode, of, args.steps, args.warmup)
    if args.skip_cpu:
        if cx.rank == 0:
            print(json.dumps({"metric": METRIC, "value": head["qps"], "unit": "queries/s", "n": n, "mode": mode,
                              "overfetch": of, "ms_per_step": head["ms_per_step"], "roofline": head["roofline"],
                              "fallbacks": head["fallbacks"], "plain_on_tensor_cores": head["plain_tc"],
                              "gpu_launches": head["launches"]}), flush=True)
        return
    e2e = allknn_e2e(cx, X, mode, of, max(1, min(args.steps, 3)))
    modes[mode] = {"value": head["qps"], "ms_per_step": head["ms_per_step"],
                   "roofline_frac": head["roofline"]["frac"], "overfetch": of if mode != "fp32" else None}
    if mode == "fp32":
        modes[mode].update({"fallbacks": head["fallbacks"], "plain_on_tensor_cores": head["plain_tc"]})
    four_k = None
    if mode == "bf16" and cx.world == 1 and not args.no_plain:
        # the configuration as written: FP32 rerank of the top 4k candidates
        # (over-fetch 4 x (k+1) = 132 per object: beyond two heaps per object,
        # so CTA pairs keep one heap per object)
        four_k = allknn_mode(cx, X, "bf16", 4.0, 3, 1)
        modes["bf16_4k"] = {"value": four_k["qps"], "ms_per_step": four_k["ms_per_step"], "overfetch": 4.0,
                            "steps": 3, "warmup": 1, "roofline": four_k["roofline"],
                            "note": "rerank of the top 4k = 132 candidates per object; the scan keeps them in one heap per object on CTA pairs"}
    suite = None
    if cx.world == 1 and args.suite != "none":
        suite = run_suite(cx, args)
    if cx.rank != 0:
        return
    cpu, rows, cids, _ = cpu_baseline(X, budget_s=args.cpu_budget)
    gold = oracle_gold_rows(rows, cids)
    r10, r32 = recall_rows(gold, head["ids"][rows], 10), recall_rows(gold, head["ids"][rows], K)
    f64 = fp64_check(X, head["ids"], head["dists"], rows[:256])
    modes[mode]["recall@10"], modes[mode]["recall@32"] = r10, r32
    if four_k is not None:
        modes["bf16_4k"]["recall@10"] = recall_rows(gold, four_k["ids"][rows], 10)
        modes["bf16_4k"]["recall@32"] = recall_rows(gold, four_k["ids"][rows], K)
    if plain is not None and "fp32" in modes:
        modes["fp32"]["recall@10"] = recall_rows(gold, plain["ids"][rows], 10)
        modes["fp32"]["recall@32"] = recall_rows(gold, plain["ids"][rows], K)
        modes["speedup_vs_fp32"] = head["qps"] / plain["qps"]
        if "fp32_cuda_cores" in modes:
            modes["speedup_vs_fp32_cuda_cores"] = head["qps"] / modes["fp32_cuda_cores"]["value"]
            modes["fp32_tc_speedup_vs_cuda_cores"] = plain["qps"] / modes["fp32_cuda_cores"]["value"]
    line = {
        "metric": METRIC, "value": head["qps"], "unit": "queries/s", "n_gpus": cx.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if mode == "fp32" else mode, "data": DATA,
        "config": config_dict(mode, of, calib),
        "recall": {"recall@10": r10, "recall@32": r32, "sample_rows": int(rows.size),
                   "gold": "oracle ExhaustiveSearch restatement (FP32, 16-lane sums), self removed",
                   "vs_fp64": f64},
        "roofline": head["roofline"],
        "cpu_baseline": {k: v for k, v in cpu.items() if k != "seconds"},
        "e2e": e2e,
        "clocks": head["clocks"],
        "gpu_launches": head["launches"],
        "modes": modes,
    }
    if suite is not None:
        line["suite"] = suite
    elif cx.world > 1:
        line["suite"] = {"skipped": "replicas at N > 1 report the headline only; the suite runs at N = 1"}
    print(json.dumps(line), flush=True)
    if cx.world > 1:
        cx.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# The suite's other configurations
# ---------------------------------------------------------------------------

def search_entry(cx, name, X, Q, k, mode, steps, warmup, desc, roof_fn, parity_lanes=1, cpu_budget=8.0,
                 **params):
    """A searchbatch configuration: device-resident timing, the scan kernel's
    roofline, parity on the CPU baseline's sample, end-to-end through the C
    ABI, clocks."""
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    metric = {"sql2": N.METRIC_SQL2, "hamming": N.METRIC_HAMMING, "ip": N.METRIC_IP}[name]
    elem = N.ELEM_U64 if name == "hamming" else N.ELEM_F32
    n, d = X.shape
    m = Q.shape[0]
    h = cx.create(metric, elem, X, PREC[mode], **params)
    Qd = cx.dev(Q)
    ids_d = torch.empty((m, k), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((m, k), dtype=torch.float32, device="cuda")

    def step():
        N.check(L.ssg_search_device(h, C.c_void_p(Qd.data_ptr()), m, k, C.c_void_p(ids_d.data_ptr()),
                                    C.c_void_p(dists_d.data_ptr()), 0), h)

    ms, launches, main_ms, main_launches, clocks = timed_device_steps(cx, h, step, steps, warmup)
    gi = ids_d.cpu().numpy().view(np.uint32).copy()
    gd = dists_d.cpu().numpy().copy()
    fallbacks = cx.get(h, "fallbacks")
    plain_tc = mode == "fp32" and cx.get(h, "last_plain_tc") == 1.0
    L.ssg_destroy(h)
    del Qd, ids_d, dists_d
    avg = main_ms / max(1, main_launches)
    roof = plain_tc_roofline(m * n, d, avg) if plain_tc else roof_fn(avg)
    # end to end: create from pinned host memory + search from host + results to host
    Xp, Qp = cx.pinned(X), cx.pinned(Q)
    oi = torch.empty((m, k), dtype=torch.int32).pin_memory()
    od = torch.empty((m, k), dtype=torch.float32).pin_memory()

    def e2e_step():
        hh = C.c_void_p()
        N.check(L.ssg_create(metric, elem, d, n, C.c_void_p(Xp.data_ptr()), d, PREC[mode], C.byref(hh)))
        try:
            for key, v in params.items():
                N.check(L.ssg_set_param(hh, key.encode(), float(v)), hh)
            N.check(L.ssg_search(hh, C.c_void_p(Qp.data_ptr()), d, m, k, C.c_void_p(oi.data_ptr()),
                                 C.c_void_p(od.data_ptr()), 0), hh)
        finally:
            L.ssg_destroy(hh)

    e2e_step()
    t0 = time.perf_counter()
    for _ in range(3):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / 3
    del Xp, Qp
    cpu, sample, ri, rd = cpu_searchbatch_baseline(name, X, Q, k, budget_s=cpu_budget,
                                                   lanes=1 if name == "hamming" else 16)
    parity = {"sample_queries": int(sample.size), "gold": "oracle restatement, same queries"}
    if name == "hamming":
        parity["ids_equal"] = bool(np.array_equal(gi[sample], ri))
        parity["dists_equal"] = bool(np.array_equal(gd[sample], rd))
    if name != "hamming":
        si, sd = (ri, rd) if parity_lanes == 16 else O.searchbatch(name, X, Q[sample], k, lanes=1,
                                                                    nthreads=os.cpu_count() or 1)
        parity["ids_equal_lanes1"] = bool(np.array_equal(gi[sample], si))
        parity["dists_equal_lanes1"] = bool(np.array_equal(gd[sample], sd))
        parity["max_rel_ddist_vs_16lane"] = float(np.max(np.abs(gd[sample] - rd) / np.maximum(np.abs(rd), 1.0)))
    parity["recall@k"] = O.macrorecall(ri, gi[sample])
    return {"workload": desc, "metric": "queries/s", "value": m / (ms / 1e3), "unit": "queries/s",
            "ms_per_step": ms, "steps": steps, "warmup": warmup, "mode": mode,
            "dtype": "u64" if name == "hamming" else ("f32" if mode == "fp32" else mode),
            "roofline": roof, "parity": parity, "fallbacks": fallbacks, "plain_on_tensor_cores": plain_tc,
            "cpu_baseline": cpu,
            "e2e": {"value": m / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(X.nbytes + Q.nbytes),
                    "d2h_bytes_per_step": int(m * k * 8)},
            "clocks": clocks, "gpu_launches": launches,
            "l2_policy": "database larger than L2" if X.nbytes > 129e6 else
                         "database smaller than L2: steady-state L2-resident timing"}


def suite_c1(cx, args):
    W = workloads()
    X, Q, k = W.make_c1()
    m, (n, d) = Q.shape[0], X.shape
    desc = "searchbatch SqL2, n=100,000, d=128, m=1,000, k=10 (N(0,1) data)"
    e = search_entry(cx, "sql2", X, Q, k, "fp32", max(args.steps, 20), args.warmup, desc,
                     lambda ms: roofline_flops("fp32", 2.0 * m * n * d, ms))
    cc = search_entry(cx, "sql2", X, Q, k, "fp32", max(args.steps, 20), args.warmup, desc,
                      lambda ms: roofline_flops("fp32", 2.0 * m * n * d, ms), cpu_budget=1.0, plain_tc=0)
    bf = search_entry(cx, "sql2", X, Q, k, "bf16", max(args.steps, 20), args.warmup, desc,
                      lambda ms: roofline_flops("bf16", 2.0 * m * n * d, ms), cpu_budget=1.0, overfetch=2.0)
    e["modes"] = {"bf16": {"value": bf["value"], "ms_per_step": bf["ms_per_step"], "overfetch": 2.0,
                           "recall@k_vs_oracle": bf["parity"]["recall@k"], "roofline": bf["roofline"]},
                  "fp32_cuda_cores": {"value": cc["value"], "ms_per_step": cc["ms_per_step"],
                                      "roofline": cc["roofline"], "parity": cc["parity"], "e2e": cc["e2e"],
                                      "note": "the plain method on the CUDA cores (FP32 FMA GEMM form)"}}
    return e


def suite_c3(cx, args):
    W = workloads()
    X, Q, k = W.make_c3()
    n, words = X.shape
    out = {}
    for tag, m in (("m10000", Q.shape[0]), ("m64", 64)):
        Qm = np.ascontiguousarray(Q[:m])
        desc = f"searchbatch Bits.Hamming, n={n:,} sketches x 1024 bits, m={m:,} (10% flips), k=100"

        def roof(ms, m=m):
            # one pass over the sketches + the queries + the results (bytes per call)
            r = roofline_bytes(8.0 * words * n + 8.0 * words * m + 8.0 * k * m, ms)
            # the binding roof at these m: 64-bit XOR + POPC issue, 16 32-bit
            # POPC per clock per SM = 8 words per clock per SM (nominal, at
            # the measured maximum SM clock; no measured INT peak exists)
            words_peak = 152 * 8 * peaks().get("sm_max_mhz", 2070.0) * 1e6
            r["popcount_words_per_s"] = n * m * words / (ms / 1e3)
            r["popcount_peak_words_per_s"] = words_peak
            r["popcount_frac"] = r["popcount_words_per_s"] / words_peak
            return r

        out[tag] = search_entry(cx, "hamming", X, Qm, k, "fp32", max(args.steps, 10 if m > 64 else 50),
                                args.warmup, desc, roof, cpu_budget=6.0)
    out["note"] = ("the binding roof is the XOR + POPC issue rate down to m ~ 6 queries (16 m popcounts per "
                   "128-byte row against the HBM rate), so the HBM fraction stays small by construction at m = 64")
    return out


def c4_stream(cx, h, Qd, sizes, ks, offs, d, plain):
    """Each batch of the stream as one ssg_search_device call: per-call
    latencies (host clock around the call and its synchronisation) and the
    result rows."""
    torch, N, L = cx.torch, cx.N, cx.L
    kmax = int(ks.max())
    ids_d = torch.empty((int(sizes.max()), kmax), dtype=torch.int32, device="cuda")
    dd_d = torch.empty((int(sizes.max()), kmax), dtype=torch.float32, device="cuda")
    cx.set(h, "plain", 1.0 if plain else 0.0)
    lat, results = [], []
    for b in range(len(sizes)):
        m, k = int(sizes[b]), int(ks[b])
        q = C.c_void_p(Qd.data_ptr() + int(offs[b]) * d * 4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(L.ssg_search_device(h, q, m, k, C.c_void_p(ids_d.data_ptr()), C.c_void_p(dd_d.data_ptr()), 0), h)
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t0)
        results.append(ids_d.view(-1)[:m * k].view(m, k).cpu().numpy().view(np.uint32).copy())
    cx.set(h, "plain", 0.0)
    return np.array(lat), results


def c4_windows(cx, h, Qd, sizes, ks, offs, d, window):
    """The same stream, `window` consecutive batches per ssg_search_batches
    call (one packed search per distinct k, CUDA-graph replay of repeated
    shapes)."""
    torch, N, L = cx.torch, cx.N, cx.L
    lat = []
    out_i = torch.empty(int((sizes * ks).sum()), dtype=torch.int32, device="cuda")
    out_d = torch.empty(int((sizes * ks).sum()), dtype=torch.float32, device="cuda")
    ooff = np.concatenate([[0], np.cumsum(sizes * ks)])
    calls = 0
    for w0 in range(0, len(sizes), window):
        bs = list(range(w0, min(len(sizes), w0 + window)))
        nb = len(bs)
        P = C.c_void_p * nb
        qp = P(*[Qd.data_ptr() + int(offs[b]) * d * 4 for b in bs])
        mp = (C.c_int64 * nb)(*[int(sizes[b]) for b in bs])
        kp = (C.c_int32 * nb)(*[int(ks[b]) for b in bs])
        ip = P(*[out_i.data_ptr() + int(ooff[b]) * 4 for b in bs])
        dp = P(*[out_d.data_ptr() + int(ooff[b]) * 4 for b in bs])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(L.ssg_search_batches(h, nb, qp, mp, kp, ip, dp), h)
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t0)
        calls += 1
    allids = out_i.cpu().numpy().view(np.uint32)
    results = [allids[ooff[b]:ooff[b + 1]].reshape(int(sizes[b]), int(ks[b])).copy() for b in range(len(sizes))]
    return np.array(lat), results, calls


def suite_c4(cx, args, data):
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    X, Q, sizes, ks, H = data
    n, d = X.shape
    offs = np.concatenate([[0], np.cumsum(sizes)])
    tq = int(sizes.sum())
    out = {}
    for name in ("ip", "sql2"):
        metric = N.METRIC_IP if name == "ip" else N.METRIC_SQL2
        h = cx.create(metric, N.ELEM_F32, X, PREC["fp8"])
        Qd = torch.from_numpy(Q).cuda()
        # over-fetch: the autotuner's rule on 2,048 calibration queries of
        # their own seeds (neither the timed stream nor the held-out queries)
        # against the plain method; recall is then reported on the whole
        # stream and on the held-out queries
        Qc = torch.from_numpy(workloads().c4_calibration_queries(2048, d)).cuda()
        nc = Qc.shape[0]
        ci = torch.empty((nc, 10), dtype=torch.int32, device="cuda")
        cd = torch.empty((nc, 10), dtype=torch.float32, device="cuda")
        cx.set(h, "plain", 1.0)
        N.check(L.ssg_search_device(h, C.c_void_p(Qc.data_ptr()), nc, 10, C.c_void_p(ci.data_ptr()),
                                    C.c_void_p(cd.data_ptr()), 0), h)
        gold_c = ci.cpu().numpy().view(np.uint32).copy()
        cx.set(h, "plain", 0.0)
        chosen = 16.0
        for c in (1.0, 1.25, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0, 16.0):
            cx.set(h, "overfetch", c)
            N.check(L.ssg_search_device(h, C.c_void_p(Qc.data_ptr()), nc, 10, C.c_void_p(ci.data_ptr()),
                                        C.c_void_p(cd.data_ptr()), 0), h)
            if O.macrorecall(gold_c, ci.cpu().numpy().view(np.uint32)) >= 0.997:
                chosen = c
                break
        cx.set(h, "overfetch", chosen)
        c4_stream(cx, h, Qd, sizes, ks, offs, d, False)  # warm-up pass
        cx.set(h, "profile", 1.0)
        with ClockSampler(cx.local) as clk:
            lat_r, res_r = c4_stream(cx, h, Qd, sizes, ks, offs, d, False)
        scan_ms, scans = cx.get(h, "main_kernel_ms"), int(cx.get(h, "main_kernel_launches"))
        cx.set(h, "profile", 0.0)
        window = max(1, args.window)
        for _ in range(3):  # sizes the buffers, sees each shape, captures the graphs
            c4_windows(cx, h, Qd, sizes, ks, offs, d, window)
        r0 = cx.get(h, "graph_replays")
        lat_w, res_w, calls = c4_windows(cx, h, Qd, sizes, ks, offs, d, window)
        replays = int(cx.get(h, "graph_replays") - r0)
        lat_p, res_p = c4_stream(cx, h, Qd, sizes, ks, offs, d, True)
        # the same plain method on the CUDA cores (identical results)
        cx.set(h, "plain_tc", 0.0)
        lat_pc, res_pc = c4_stream(cx, h, Qd, sizes, ks, offs, d, True)
        cx.set(h, "plain_tc", 1.0)
        plain_same = all(np.array_equal(a, b) for a, b in zip(res_p, res_pc))
        big = [b for b in range(len(sizes)) if ks[b] >= 10]
        wts = sizes[big].astype(np.float64)
        rec = float(np.average([O.macrorecall(res_p[b][:, :10], res_r[b][:, :10]) for b in big], weights=wts))
        rec_w = float(np.average([O.macrorecall(res_p[b][:, :10], res_w[b][:, :10]) for b in big], weights=wts))
        # held-out queries (seeds the stream and the calibration never saw):
        # recall@10 against the FP64 ranking, reduced and plain
        Hd = torch.from_numpy(H).cuda()
        hi = torch.empty((H.shape[0], 10), dtype=torch.int32, device="cuda")
        hd = torch.empty((H.shape[0], 10), dtype=torch.float32, device="cuda")
        got = {}
        for plain in (0.0, 1.0):
            cx.set(h, "plain", plain)
            N.check(L.ssg_search_device(h, C.c_void_p(Hd.data_ptr()), H.shape[0], 10, C.c_void_p(hi.data_ptr()),
                                        C.c_void_p(hd.data_ptr()), 0), h)
            got[plain] = hi.cpu().numpy().view(np.uint32).copy()
        cx.set(h, "plain", 0.0)
        fi, _ = O.searchbatch_f64(name, X, H, 10, nthreads=os.cpu_count() or 1)
        # end to end: one request through ssg_search from host memory (queries
        # up, results down), per call, over the stream
        Qp = torch.from_numpy(Q).pin_memory()
        oi = torch.empty(int(sizes.max()) * int(ks.max()), dtype=torch.int32).pin_memory()
        od = torch.empty(int(sizes.max()) * int(ks.max()), dtype=torch.float32).pin_memory()
        t0 = time.perf_counter()
        for b in range(len(sizes)):
            N.check(L.ssg_search(h, C.c_void_p(Qp.data_ptr() + int(offs[b]) * d * 4), d, int(sizes[b]), int(ks[b]),
                                 C.c_void_p(oi.data_ptr()), C.c_void_p(od.data_ptr()), 0), h)
        e2e_s = time.perf_counter() - t0
        L.ssg_destroy(h)
        del Qd, Qc, Hd, ci, cd, hi, hd
        torch.cuda.empty_cache()
        cpu, _, _, _ = cpu_searchbatch_baseline(name, X, H, 10, budget_s=5.0)
        # HBM bytes one scan of the stream reads per batch (FP8 rows + the
        # two epilogue coefficients per row) plus its queries and results
        bytes_total = float(scans) * n * (d + 8) + tq * d * 4 + float((sizes * ks).sum()) * 8
        roof = roofline_bytes(bytes_total / max(1, scans), scan_ms / max(1, scans), kernel="tc_stream_kernel")
        roof["note"] = ("HBM bytes per scan launch (n x (d + 8) FP8 row bytes + queries + results), averaged over "
                        "the stream's launches; large batches are tensor-bound instead")
        out[name] = {
            "workload": f"{'IP' if name == 'ip' else 'SqL2'} request stream, n={n:,}, d={d}, {len(sizes)} batches "
                        f"(sizes LogNormal(ln 64,1) in [1,4096], k in {{1,10,100}}), FP8 e4m3 + exact FP32 rerank",
            "metric": "queries/s", "value": tq / lat_r.sum(), "unit": "queries/s", "dtype": "fp8",
            "overfetch_autotuned": chosen,
            "latency_ms": {"p50": float(np.percentile(lat_r, 50) * 1e3), "p99": float(np.percentile(lat_r, 99) * 1e3)},
            "recall@10_vs_plain_stream": rec,
            "recall@10_vs_fp64_heldout": {"reduced": O.macrorecall(fi, got[0.0]), "plain": O.macrorecall(fi, got[1.0]),
                                          "queries": int(H.shape[0])},
            "plain_fp32": {"value": tq / lat_p.sum(), "latency_ms": {"p50": float(np.percentile(lat_p, 50) * 1e3),
                                                                     "p99": float(np.percentile(lat_p, 99) * 1e3)}},
            "speedup_vs_plain": float(lat_p.sum() / lat_r.sum()),
            "plain_fp32_cuda_cores": {"value": tq / lat_pc.sum(),
                                      "latency_ms": {"p50": float(np.percentile(lat_pc, 50) * 1e3),
                                                     "p99": float(np.percentile(lat_pc, 99) * 1e3)},
                                      "ids_equal_to_plain_fp32": plain_same,
                                      "note": "plain_fp32 runs on the tensor cores (two-piece BF16, certified "
                                              "exact); this is the same method on the CUDA cores"},
            "speedup_vs_plain_cuda_cores": float(lat_pc.sum() / lat_r.sum()),
            "coalesced": {"window_batches": window, "value": tq / lat_w.sum(), "unit": "queries/s",
                          "latency_ms_per_window": {"p50": float(np.percentile(lat_w, 50) * 1e3),
                                                    "p99": float(np.percentile(lat_w, 99) * 1e3)},
                          "graph_replays": replays, "calls": calls, "recall@10_vs_plain_stream": rec_w,
                          "speedup_vs_plain": float(lat_p.sum() / lat_w.sum())},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": tq / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(Q.nbytes),
                    "d2h_bytes_per_step": int((sizes * ks).sum()) * 8,
                    "note": "one ssg_search per batch from host memory over the whole stream (step = stream)"},
            "clocks": clk.summary(),
        }
    return out


def suite_c5(cx, args, data):
    """The learned shortlist on the C4 database under SqL2 (768 -> 256 -> 64
    network, 200k-object sample, 5M triplets, 20 epochs, exact FP32 rerank to
    k = 10) beside the plain FP32 method and the same pipeline with a 64-d
    random projection: each at its smallest shortlist reaching recall@10 >=
    0.99 against the plain method on held-out queries."""
    torch, N, L = cx.torch, cx.N, cx.L
    from oracle import oracle as O
    X, Q, _, _, H = data
    n, d = X.shape
    m, k = min(10_000, Q.shape[0]), 10
    Qs = np.ascontiguousarray(Q[:m])
    h = cx.create(N.METRIC_SQL2, N.ELEM_F32, X, PREC["fp32"])
    Qd = torch.from_numpy(Qs).cuda()
    Hd = torch.from_numpy(H).cuda()
    ids_d = torch.empty((m, k), dtype=torch.int32, device="cuda")
    dd_d = torch.empty((m, k), dtype=torch.float32, device="cuda")

    def run(Qt, mq):
        N.check(L.ssg_search_device(h, C.c_void_p(Qt.data_ptr()), mq, k, C.c_void_p(ids_d.data_ptr()),
                                    C.c_void_p(dd_d.data_ptr()), 0), h)

    def timed(steps, warmup):
        for _ in range(warmup):
            run(Qd, m)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            run(Qd, m)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        return m / (ms / 1e3), ms, ids_d.cpu().numpy().view(np.uint32).copy()

    def heldout():
        run(Hd, H.shape[0])
        torch.cuda.synchronize()
        return ids_d[:H.shape[0]].cpu().numpy().view(np.uint32).copy()

    steps, warmup = max(3, args.steps // 2), max(3, args.warmup)
    qps_plain, ms_plain, gold = timed(steps, warmup)
    gold_h = heldout()
    # the same plain method on the CUDA cores (identical results)
    cx.set(h, "plain_tc", 0.0)
    qps_plain_cc, ms_plain_cc, gold_cc = timed(1, 1)
    cx.set(h, "plain_tc", 1.0)
    ladder = (512, 256, 128, 64, 32)

    def sweep(tag):
        """Smallest shortlist of the ladder whose recall@10 against the plain
        method on the held-out queries reaches 0.99 (learned path forced)."""
        cx.set(h, "learned_target", 0.0)
        rows, best = {}, None
        for S in ladder:
            cx.set(h, "shortlist", S)
            r = O.macrorecall(gold_h, heldout())
            rows[S] = r
            if r >= 0.99:
                best = S
            else:
                break
        return best, rows

    # random projection: the same pipeline without a trained network
    cx.set(h, "learned_target", 0.0)
    N.check(L.ssg_train_mlp(h, 200_000, 0, 0, 0, 64, 1024, 1e-3, 15), h)
    rp_best, rp_rows = sweep("random")
    cx.set(h, "shortlist", rp_best or ladder[0])
    qps_rp, ms_rp, got_rp = timed(steps, warmup)
    rp = {"value": qps_rp, "ms_per_step": ms_rp, "shortlist": rp_best or ladder[0],
          "recall@10_vs_plain": O.macrorecall(gold, got_rp), "heldout_recall_by_shortlist": rp_rows,
          "estimated_recall": cx.get(h, "learned_recall")}
    # the trained network
    N.check(L.ssg_train_mlp(h, 200_000, args.triplets, args.epochs, 256, 64, 1024, 1e-3, 15), h)
    stats = {key: cx.get(h, key) for key in ("learned_recall", "train_loss", "train_seconds", "train_steps")}
    tr_best, tr_rows = sweep("trained")
    S = tr_best or ladder[0]
    cx.set(h, "shortlist", S)
    cx.set(h, "learned_target", 0.99)
    est = cx.get(h, "learned_recall")
    with ClockSampler(cx.local) as clk:
        qps_l, ms_l, got_l = timed(steps, warmup)
    used = int(cx.get(h, "learned_used"))
    got_h = heldout()
    ns = 32
    fi, _ = O.searchbatch_f64("sql2", X, H[:ns], k, nthreads=os.cpu_count() or 1)
    cpu, _, _, _ = cpu_searchbatch_baseline("sql2", X, H, k, budget_s=5.0)
    # end to end: queries up from pinned host memory, results down, per step
    Qp = torch.from_numpy(Qs).pin_memory()
    oi = torch.empty((m, k), dtype=torch.int32).pin_memory()
    od = torch.empty((m, k), dtype=torch.float32).pin_memory()
    N.check(L.ssg_search(h, C.c_void_p(Qp.data_ptr()), d, m, k, C.c_void_p(oi.data_ptr()),
                         C.c_void_p(od.data_ptr()), 0), h)
    t0 = time.perf_counter()
    for _ in range(3):
        N.check(L.ssg_search(h, C.c_void_p(Qp.data_ptr()), d, m, k, C.c_void_p(oi.data_ptr()),
                             C.c_void_p(od.data_ptr()), 0), h)
    e2e_s = (time.perf_counter() - t0) / 3
    L.ssg_destroy(h)
    del Qd, Hd, ids_d, dd_d
    torch.cuda.empty_cache()
    # step bytes: the 64-d BF16 embeddings of the database, the shortlist's
    # rows gathered for the exact rerank, the queries
    step_bytes = float(n) * 64 * 2 + float(m) * S * d * 4 + float(m) * d * 4
    roof = roofline_bytes(step_bytes, ms_l, kernel="learned step (embed + 64-d scan + rerank)")
    return {"workload": f"SqL2 searchbatch m={m}, k={k}, n={n:,}, d={d}; MLP {d}->256->64, 200k sample, "
                        f"{args.triplets:,} triplets, {args.epochs} epochs",
            "metric": "queries/s", "value": qps_l, "unit": "queries/s", "ms_per_step": ms_l, "steps": steps,
            "warmup": warmup, "dtype": "bf16-operand network, fp32 rerank", "shortlist": S,
            "learned_used": used, "estimated_recall": est,
            "recall@10_vs_plain": O.macrorecall(gold, got_l),
            "recall@10_vs_plain_heldout": O.macrorecall(gold_h, got_h),
            "recall@10_vs_fp64_heldout": {"learned": O.macrorecall(fi, got_h[:ns]),
                                          "plain": O.macrorecall(fi, gold_h[:ns]), "queries": ns},
            "heldout_recall_by_shortlist": tr_rows, "training": stats, "random_projection": rp,
            "plain_fp32": {"value": qps_plain, "ms_per_step": ms_plain,
                           "note": "two-piece BF16 on the tensor cores, certified exact"},
            "plain_fp32_cuda_cores": {"value": qps_plain_cc, "ms_per_step": ms_plain_cc,
                                      "ids_equal_to_plain_fp32": bool(np.array_equal(gold, gold_cc))},
            "speedup_vs_plain_cuda_cores": qps_l / qps_plain_cc,
            "speedup_vs_plain": qps_l / qps_plain, "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": m / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(Qs.nbytes),
                    "d2h_bytes_per_step": int(m * k * 8)},
            "clocks": clk.summary()}


def run_suite(cx, args):
    wanted = {"c1", "c3", "c4", "c5"} if args.suite == "all" else set(args.suite.split(","))
    out = {}
    t_all = time.perf_counter()
    for name, fn in (("c1", suite_c1), ("c3", suite_c3)):
        if name in wanted:
            t0 = time.perf_counter()
            out[name] = fn(cx, args)
            out[name]["wall_s"] = time.perf_counter() - t0
    if wanted & {"c4", "c5"}:
        W = workloads()
        X, Q, sizes, ks = W.make_c4(batches=args.batches)
        data = (X, Q, sizes, ks, W.c4_heldout_queries(64))
        for name, fn in (("c4", suite_c4), ("c5", suite_c5)):
            if name in wanted:
                t0 = time.perf_counter()
                out[name] = fn(cx, args, data)
                out[name]["wall_s"] = time.perf_counter() - t0
    out["wall_s"] = time.perf_counter() - t_all
    return out


def workload_arm(args):
    """One configuration of the suite alone, printed as its own line."""
    cx = Ctx()
    if args.workload in ("c4", "c5"):
        W = workloads()
        X, Q, sizes, ks = W.make_c4(args.n if args.n is not None else 2_000_000, batches=args.batches)
        data = (X, Q, sizes, ks, W.c4_heldout_queries(64))
        res = suite_c4(cx, args, data) if args.workload == "c4" else suite_c5(cx, args, data)
    else:
        res = suite_c1(cx, args) if args.workload == "c1" else suite_c3(cx, args)
    print(json.dumps({"workload": args.workload, "n_gpus": cx.world, "result": res}), flush=True)


def main():
    global N_DB
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--mode", default="bf16", choices=["fp32", "bf16", "fp8"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 = the headline line (with the suite); c1/c3/c4/c5 = one configuration alone")
    ap.add_argument("--suite", default="all", help="suite entries with the headline: all, none, or e.g. c1,c3")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--batches", type=int, default=200, help="c4: batches in the request stream")
    ap.add_argument("--triplets", type=int, default=5_000_000, help="c5: training triplets")
    ap.add_argument("--window", type=int, default=8, help="c4: batches coalesced per ssg_search_batches call")
    ap.add_argument("--epochs", type=int, default=20, help="c5: training epochs")
    ap.add_argument("--n", type=int, default=None,
                    help="database size (profiling captures use a smaller case of the same workload)")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline and the suite (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="omit the plain FP32 comparison run")
    ap.add_argument("--overfetch", type=float, default=None,
                    help="candidates per neighbour kept by the reduced-precision scan (default: calibrated)")
    args = ap.parse_args()
    if args.n is not None and args.workload == "c2":
        N_DB = args.n
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload != "c2":
        workload_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
