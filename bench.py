#!/usr/bin/env python
"""Benchmark of the TBSLA SpMV hot path on GB300.

Workload (the large-SpMV configuration): square CSR matrix, n = 16,777,216
rows, row lengths Zipf(2) on [1, 4096] rescaled to mean 16 (~268M entries),
70% of the columns uniform over [0, n) and 30% within +-1024 of the diagonal,
values U[-1,1) stored in FP64 (--prec selects FP32 / BF16 storage), x U[0,1),
seed 1.  One step = one y = A x (tbsla::cpp::MatrixCSR::Ax).

Metric: SpMV HBM GB/s of algorithmic bytes per step
  B = nnz*(s_v + 4) + 4*(n+1) + 8*n (x, counted once) + 8*n (y)
divided by the step's device time (CUDA events on the launching stream, L2
flushed between steps).  `e2e` is the same metric through the C ABI's host
entry point tbsla_Ax with pinned host x / y: the host->device copy of x and
the device->host copy of y are inside the timed region.  The CPU baseline is
the reference's CSR Ax loop (the reference core compiled from its sources
where available, else the oracle's restatement of it) on all host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank runs an independent replica (the path has
no exchange step on one GPU); the value is the sum of bytes over the max time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SMS = 152  # GB300 streaming multiprocessors
METRIC = "SpMV HBM GB/s (% peak); CG time-to-1e-8 residual: learned vs Jacobi PCG, 1 GB300"
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "csr_spmv_powerlaw_n16M_fp64.md")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["spmv", "small", "formats", "pagerank", "cg", "learned"], default="spmv",
                   help="spmv: the large-SpMV headline; small: the 10^4-row matrix in every format and the "
                        "2000^2 DENSE GEMV; formats: every format at n = 2^22 rows and a 32768 x 16384 DENSE "
                        "GEMV; pagerank: the PageRank graph; cg: batched CG; "
                        "learned: learned-preconditioner PCG against Jacobi-PCG")
    p.add_argument("--train-systems", type=int, default=2000, help="learned: training systems (seeds 1000..)")
    p.add_argument("--epochs", type=int, default=1, help="learned: passes over the training systems")
    p.add_argument("--eval-systems", type=int, default=32, help="learned: held-out systems (seeds 9000..)")
    p.add_argument("--eval-n", type=int, default=128, help="learned: held-out grid size n (n^3 unknowns)")
    p.add_argument("--factor-prec", choices=["f32", "bf16"], default="bf16",
                   help="learned: storage precision of the factor L")
    p.add_argument("--n", type=int, default=None, help="rows (spmv: 2^24, pagerank and formats: 2^22)")
    p.add_argument("--formats", type=str, default="coo,scoo,csr,ell,dense,dense_f32,dense_bf16",
                   help="formats: which formats to run (dense_f32 / dense_bf16: DENSE with narrow values)")
    p.add_argument("--prec", choices=["f64", "f32", "bf16"], default="f64")
    p.add_argument("--tile", type=int, default=2048, help="row-block kernel: entries per block")
    p.add_argument("--algo", choices=["sell", "merge", "rowblock"], default="sell")
    p.add_argument("--sell", type=str, default="0,0,16384,0",
                   help="sliced-ELL kernel: short_thr,long_thr,sigma,col_block (thresholds 0: 128 for FP64 values "
                        "with several column blocks, else 64; col_block 0: 2^23 columns)")
    p.add_argument("--items", type=int, default=0,
                   help="merge: items per thread (0 = 8); sell: steps per lane in flight (0 = automatic)")
    p.add_argument("--no-forms", action="store_true", help="skip the FP32 / BF16 side measurements")
    p.add_argument("--no-learned", action="store_true",
                   help="spmv: skip the learned-vs-Jacobi and batched-CG measurements of the default run")
    p.add_argument("--autotune", action="store_true",
                   help="spmv: time the CSR kernel configurations on the matrix first and keep the fastest; "
                        "cg / pagerank: tune the batched forms' settings (cached in a JSON file, "
                        "TBSLA_TUNE_CACHE)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    a = p.parse_args()
    a.warmup = max(a.warmup, 3)
    if a.n is None:
        a.n = 1 << 22 if a.workload in ("pagerank", "formats") else 1 << 24
    return a


def algorithmic_bytes(n: int, nnz: int, s_v: int) -> int:
    return nnz * (s_v + 4) + 4 * (n + 1) + 8 * n + 8 * n


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """dram bytes per launch from the committed ncu summary, if present."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.startswith("dram_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip().split()[0]))
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        # nvidia-smi's start-up (NVML initialisation) slowed the host-driven
        # pageable copies that ran beside it: wait for its first sample (at
        # most 3 s) so that the timed region sees only its steady sampling
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 3.0:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def job_throughput(local_ms: float, local_bytes: int, ws: int, device: str = "cuda"):
    """Replicas: the job's time is the slowest rank's, its bytes the sum over
    ranks (every rank processes its own copy of the workload).  Returns
    (max time in ms, whole-job GB/s)."""
    total_ms = local_ms
    total_bytes = local_bytes
    if ws > 1:
        import torch
        import torch.distributed as td

        t = torch.tensor([local_ms], device=device, dtype=torch.float64)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        total_ms = float(t.item())
        b = torch.tensor([float(local_bytes)], device=device, dtype=torch.float64)
        td.all_reduce(b, op=td.ReduceOp.SUM)
        total_bytes = float(b.item())
    return total_ms, total_bytes / (total_ms * 1e-3) / 1e9


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_reference_time(arrays, x, n, nnz, seconds: float, reps_min: int = 2, reps_max: int = 50):
    """Times the reference's CSR Ax loop on all host cores: the reference core
    compiled from its own sources when it is available here, otherwise the
    oracle's restatement of that loop (same loop, same OpenMP schedule)."""
    import ctypes as C

    import numpy as np

    import oracle

    rp, ci, va = arrays["rowptr"], arrays["colidx"], arrays["values"]
    y = np.zeros(n)
    kind = "port"
    run = None
    R = oracle.ref() if os.path.exists(oracle._build.REF_SO) else None
    if R is not None:
        try:
            h = C.c_void_p(R.ref_new(2))
            meta = np.array([n, n, n, n, 0, 0, 0, 0, 1, 1, 0], np.int32)
            R.ref_adopt(h, C.c_void_p(meta.ctypes.data), C.c_long(nnz), C.c_void_p(va.ctypes.data),
                        C.c_void_p(rp.ctypes.data), C.c_void_p(ci.ctypes.data))
            kind = "reference"

            def run():
                R.ref_Ax(h, C.c_void_p(y.ctypes.data), C.c_void_p(x.ctypes.data), 0)
        except OSError:
            R = None
    if run is None:
        def run():
            oracle.csr_ax(rp, ci, va, x, y, threads=True)
    run()  # warm-up (first touch)
    times = []
    t_end = time.perf_counter() + seconds
    while (len(times) < reps_min or time.perf_counter() < t_end) and len(times) < reps_max:
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    return kind, times, y


def gather_ceiling(m, x, s, flush, ms_spmv: float, warmup: int) -> dict:
    """The x-gather part of the SpMV alone, as a measured ceiling for its
    access pattern: torch.index_select (a library gather kernel) over the
    matrix's own column indices, one column block of 2^23 columns at a time
    as the sliced-ELL launches walk them, L2 flushed before each block, CUDA
    events.  It moves an index (4 B) in and an entry (8 B) out per gather,
    where the SpMV streams a value and a column (12 B) per entry."""
    import numpy as np
    import torch

    a = m.arrays()
    rp, ci = a["rowptr"], a["colidx"]
    nnz = int(rp[-1])
    xt = torch.from_numpy(x).cuda()
    cb = 8388608
    blocks = []
    for lo in range(0, len(x), cb):
        c = ci[:nnz]
        sel = c[(c >= lo) & (c < lo + cb)]
        blocks.append(torch.from_numpy(np.ascontiguousarray(sel)).cuda())
    outs = [torch.empty(len(b), dtype=torch.float64, device="cuda") for b in blocks]
    torch.cuda.synchronize()
    times = []
    with torch.cuda.stream(s):
        for rep in range(warmup + 3):
            t = 0.0
            for b, o in zip(blocks, outs):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                torch.index_select(xt, 0, b, out=o)
                e1.record(s)
                s.synchronize()
                t += e0.elapsed_time(e1)
            if rep >= warmup:
                times.append(t)
    ms = statistics.median(times)
    del blocks, outs
    torch.cuda.empty_cache()
    return {"gathers": nnz, "ms": ms, "gathers_per_s": nnz / (ms * 1e-3),
            "spmv_gathers_per_s": nnz / (ms_spmv * 1e-3), "spmv_fraction_of_ceiling": ms / ms_spmv,
            "kernel": "torch.index_select over the column indices, per column block, L2 flushed"}


def run_ours(a):
    import ctypes as C

    import numpy as np
    import torch

    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    if ws > 1:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = a.n
    t0 = time.time()
    m = T.MatrixCSR()
    m.fill_powerlaw(n, 16.0, 2.0, 4096, 0.3, 1024, 1)
    nnz = m.get_nnz()
    t_gen = time.time() - t0
    m.set_tile(a.tile)
    m.set_algorithm({"sell": m.SELL, "merge": m.MERGE, "rowblock": m.ROWBLOCK}[a.algo], a.items)
    m.set_sell_params(*[int(t) for t in a.sell.split(",")])
    prec = {"f64": T.F64, "f32": T.F32, "bf16": T.BF16}[a.prec]
    s_v = {"f64": 8, "f32": 4, "bf16": 2}[a.prec]
    m.set_precision(prec)
    t0 = time.time()
    m.upload()
    t_up = time.time() - t0
    tuned = None
    if a.autotune:
        t0 = time.time()
        best, trials = m.autotune(reps=3)
        names = {m.SELL: "sell", m.MERGE: "merge", m.ROWBLOCK: "rowblock"}
        a.algo = names[best["algorithm"]]
        a.items, a.tile = best["items"], best["tile"]
        a.sell = f"{best['short_thr']},{best['long_thr']},{best['sigma']},{best['col_block']}"
        tuned = {"chosen": {k: v for k, v in best.items()}, "trials": len(trials),
                 "seconds": round(time.time() - t0, 2)}
    x = T.fill_uniform(n, 0.0, 1.0, 1)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    s = torch.cuda.Stream()
    B = algorithmic_bytes(n, nnz, s_v)

    def timed_steps(mat, k):
        evs = []
        with torch.cuda.stream(s):
            for _ in range(k):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                mat.Ax_device(yt, xt, stream=s)
                e1.record(s)
                evs.append((e0, e1))
        s.synchronize()
        return [e0.elapsed_time(e1) for e0, e1 in evs]

    timed_steps(m, a.warmup)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    clk.start()
    step_ms = timed_steps(m, a.steps)
    torch.cuda.synchronize()
    clocks = clk.stop()
    if ws > 1:
        torch.distributed.barrier()
    total_ms, value = job_throughput(sum(step_ms), B * a.steps, ws, "cuda")
    ms_step = total_ms / a.steps
    kernel_gbs = B / (statistics.mean(step_ms) * 1e-3) / 1e9
    launches = m.kernel_launches()  # of one SpMV on this device copy
    peak, peak_kind = peaks()

    # end to end through the C ABI's host entry point, pinned host buffers
    hx, hy = C.c_void_p(), C.c_void_p()
    T.check(T.lib.tbsla_host_alloc(C.byref(hx), n * 8))
    T.check(T.lib.tbsla_host_alloc(C.byref(hy), n * 8))
    xh = np.ctypeslib.as_array(C.cast(hx, C.POINTER(C.c_double)), shape=(n,))
    yh = np.ctypeslib.as_array(C.cast(hy, C.POINTER(C.c_double)), shape=(n,))
    xh[:] = x
    for _ in range(a.warmup):
        m.Ax(yh, xh)
    e2e = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        T.check(T.lib.tbsla_Ax(m._h, hy, hx, 0))
        e2e.append(time.perf_counter() - t0)
    e2e_val = B / statistics.mean(e2e) / 1e9
    y_dev = yt.cpu().numpy()
    assert np.array_equal(y_dev, yh), "device-pointer and host entry points disagree"

    extra = {"gflops": 2 * nnz / (ms_step * 1e-3) / 1e9, "gen_s": round(t_gen, 2), "upload_s": round(t_up, 2),
             "step_ms_min": min(step_ms), "step_ms_max": max(step_ms),
             "device_bytes": m.device_bytes()}
    if a.algo == "sell" and a.prec == "f64" and ws == 1:
        extra["gather_ceiling"] = gather_ceiling(m, x, s, flush, ms_step, a.warmup)
    if not a.no_forms and a.prec == "f64":
        for name, pv, sv in (("f32", T.F32, 4), ("bf16", T.BF16, 2)):
            m.set_precision(pv)
            m.upload()
            timed_steps(m, a.warmup)
            ms = statistics.mean(timed_steps(m, a.steps))
            extra[f"{name}_values"] = {"ms_per_step": ms,
                                       "GB/s": algorithmic_bytes(n, nnz, sv) / (ms * 1e-3) / 1e9,
                                       "frac_of_peak": algorithmic_bytes(n, nnz, sv) / (ms * 1e-3) / 1e9 / peak}
        m.set_precision(prec)

    if ws == 1 and not a.no_learned:
        # the metric's second half, in the same default run: learned-PCG
        # (network inference on the GPU + solve) against Jacobi-PCG on the
        # 32 held-out 128^3 diffusion systems, and the 64-system batched
        # Jacobi-PCG workload
        r = learned_vs_jacobi(a, T, local)
        extra["learned_vs_jacobi"] = {
            "ratio": r["ratio"], "target": 0.5, "ratio_refresh50": r["ratio_refresh50"], "timed": r["timed"],
            "learned_ms": r["solvers"]["learned_pcg"]["ms"], "factor_ms": r["solvers"]["learned_pcg"]["factor_ms"],
            "jacobi_ms": r["solvers"]["jacobi_pcg"]["ms"],
            "refresh": {"learned": r["solvers"]["learned_pcg"]["refresh"], "jacobi": r["solvers"]["jacobi_pcg"]["refresh"]},
            "sweep_ms": {k: {rf: round(v["ms"], 1) for rf, v in sw.items()} for k, sw in r["sweep"].items()},
            "iterations_mean": {"learned": r["solvers"]["learned_pcg"]["iterations_mean"],
                                "jacobi": r["solvers"]["jacobi_pcg"]["iterations_mean"]},
            "max_rel_residual_fp64": max(r["solvers"]["learned_pcg"]["max_rel_residual_fp64"],
                                         r["solvers"]["jacobi_pcg"]["max_rel_residual_fp64"]),
            "all_converged": r["solvers"]["learned_pcg"]["all_converged"] and r["solvers"]["jacobi_pcg"]["all_converged"],
            "fallbacks": r["solvers"]["learned_pcg"]["fallbacks"], "engine": r["engine"],
            "systems": r["systems"], "n": r["n"], "reps": r["reps"], "train": r["train"], "clocks": r["clocks"]}
        extra["batched_cg_jacobi"] = batched_cg_jacobi(T, reps=3)

    cpu = None
    if rank == 0 and ws == 1:
        arrays = m.arrays()
        kind, times, y_cpu = cpu_reference_time(arrays, x, n, nnz, a.cpu_seconds)
        import oracle

        scale = oracle.csr_absrow(arrays["rowptr"], arrays["colidx"], arrays["values"], x)
        if a.prec == "f64":
            extra["max_err_vs_cpu_normalized"] = oracle.rel_err_normalized(y_dev, y_cpu, scale)
        cpu = {"value": B / statistics.median(times) / 1e9, "unit": "GB/s", "cores": os.cpu_count(),
               "kind": kind,
               "sample": f"{len(times)} full Ax steps on the same matrix (median), OMP_NUM_THREADS="
                         f"{os.environ.get('OMP_NUM_THREADS', 'all')}"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "GB/s",
        "n_gpus": ws,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": a.prec,
        "data": "synthetic: seeded generator (power-law rows, seed 1), no dataset",
        "config": {"workload": f"csr_spmv_powerlaw_n{n}_mean16_zipf2_max4096_local30pct_{a.prec}",
                   "format": "CSR", "n": n, "nnz": nnz, "value_dtype": a.prec, "x_y_dtype": "f64",
                   "bytes_per_step": B, "csr_kernel": a.algo, "autotune": tuned,
                   "work_split": {"merge": f"{a.items} items/thread", "rowblock": f"{a.tile} nnz/block",
                                  "sell": f"one lane per row <= {a.sell.split(',')[0] if a.sell.split(',')[0] != '0' else 'auto (128 for FP64 with column blocks, else 64)'} sorted per "
                                          f"{a.sell.split(',')[2]}-row window, else 2..32 lanes per row, slices "
                                          f"<= {a.sell.split(',')[1] if a.sell.split(',')[1] != '0' else 'the same'} steps; "
                                          f"{a.items or 'automatic'} steps/lane in flight; "
                                          f"column blocks of {int(a.sell.split(',')[3]) or 8388608} columns"}[a.algo],
                   "l2": "flushed (256 MB write) between steps; inputs 3.2+ GB > L2",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": kernel_gbs, "peak": peak, "unit": "GB/s",
                     "frac": kernel_gbs / peak, "peak_source": peak_kind, "traffic": profile_traffic(),
                     "algorithmic_bytes": B},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "GB/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "ms_per_step": statistics.mean(e2e) * 1e3},
        "gpu_launches": a.steps * launches,
        "clocks": clocks,
        "extra": extra,
    }
    T.lib.tbsla_host_free(hx)
    T.lib.tbsla_host_free(hy)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference(a):
    """The reference arm: the reference's CSR Ax loop (MatrixCSR.cpp:209-233,
    schedule(static) over all host cores) on the same workload.  The matrix
    and x come from the oracle's restatement of the library's generator, so
    this process loads only oracle code (never the GPU library)."""
    ws, rank, local = dist()
    if rank != 0:
        return
    import oracle

    n = a.n
    t0 = time.time()
    rp, ci, va = oracle.gen_powerlaw(n, 16.0, 2.0, 4096, 0.3, 1024, 1)
    x = oracle.gen_uniform(n, 0.0, 1.0, 1)
    t_gen = time.time() - t0
    nnz = int(rp[-1])
    arrays = {"rowptr": rp, "colidx": ci, "values": va}
    B = algorithmic_bytes(n, nnz, 8)
    kind, _, _ = cpu_reference_time(arrays, x, n, nnz, 0.0, reps_min=a.warmup, reps_max=a.warmup)
    kind, times, _ = cpu_reference_time(arrays, x, n, nnz, 0.0, reps_min=a.steps, reps_max=a.steps)
    sec = sum(times) / len(times)
    val = B / sec / 1e9
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": val,
        "unit": "GB/s",
        "n_gpus": ws,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": sec * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded generator (power-law rows, seed 1), no dataset",
        "config": {"workload": f"csr_spmv_powerlaw_n{n}_mean16_zipf2_max4096_local30pct_f64", "format": "CSR",
                   "n": n, "nnz": nnz, "bytes_per_step": B, "parallelism": "host cores (OpenMP)",
                   "generator": "oracle restatement of the library's power-law generator (identical arrays)",
                   "gen_s": round(t_gen, 2)},
        "cpu_baseline": {"value": val, "unit": "GB/s", "cores": os.cpu_count(), "kind": kind,
                         "sample": f"{a.steps} full CSR Ax steps of the workload after {a.warmup} warm-up"},
        "e2e": {"value": val, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_small(a):
    """The reference's CPU-runnable workload: n = 10^4 rows, column i plus 9
    uniform columns per row, U[-1,1) values, x U[0,1), seed 0, as COO, SCOO,
    CSR and ELL, and a 2000 x 2000 DENSE GEMV; 100 Ax per format as in the
    reference perf app (tbsla_perf.cpp:101-106).  Everything fits L2, so the
    time is launch and latency: per format, device microseconds per Ax over
    100 back-to-back launches on one stream and over the same 100 launches
    replayed from a CUDA graph (CUDA events), and per host call through
    tbsla_Ax with pinned buffers (x in, y out, synchronised).  CPU baseline:
    the oracle's restatement of each format's loop, one host thread."""
    import ctypes as C

    import numpy as np
    import torch

    import oracle
    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    n, reps = 10_000, 100
    csr = T.MatrixCSR()
    csr.fill_uniform_rows(n, 10, 0)
    a0 = csr.arrays()
    nnz = int(a0["rowptr"][-1])
    x = T.fill_uniform(n, 0.0, 1.0, 0)
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a0["rowptr"]))
    coo = T.MatrixCOO.from_arrays(n, n, rows, a0["colidx"], a0["values"])
    ell = T.MatrixELL(coo)
    dense = T.MatrixDENSE()
    dense.fill_dense_uniform(2000, 2000, 0)
    xd = T.fill_uniform(2000, 0.0, 1.0, 0)
    max_col = ell.info()["max_col"]
    # algorithmic bytes per Ax (values, indices, x once, y)
    cases = {"COO": (coo, x, nnz * 16 + 16 * n), "SCOO": (T.MatrixSCOO(coo), x, nnz * 16 + 16 * n),
             "CSR": (csr, x, nnz * 12 + 4 * (n + 1) + 16 * n), "ELL": (ell, x, n * max_col * 12 + 16 * n),
             "DENSE": (dense, xd, 8 * 2000 * 2000 + 16 * 2000)}
    ae = ell.arrays()
    ad = dense.arrays()
    cpu = {"COO": lambda: oracle.coo_ax(n, rows, a0["colidx"], a0["values"], x),
           "SCOO": lambda: oracle.scoo_ax(n, 0, 0, rows, a0["colidx"], a0["values"], x),
           "CSR": lambda: oracle.csr_ax(a0["rowptr"], a0["colidx"], a0["values"], x),
           "ELL": lambda: oracle.ell_ax(ae["values"], ae["columns"], n, max_col, x),
           "DENSE": lambda: oracle.dense_ax(ad["values"], 2000, 2000, xd)}
    s = torch.cuda.Stream()
    out = {}
    launches = 0
    clk = Clocks(local)
    clk.start()
    for name, (m, xv, B) in cases.items():
        m.upload()
        nr = m.info()["ln_row"] if name != "COO" else m.info()["n_row"]
        xt = torch.from_numpy(xv).cuda()
        yt = torch.zeros(nr, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            for _ in range(a.warmup):
                m.Ax_device(yt, xt, stream=s)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                m.Ax_device(yt, xt, stream=s)
            e1.record(s)
        s.synchronize()
        stream_us = e0.elapsed_time(e1) * 1e3 / reps
        launches += reps * m.kernel_launches()
        graph_us = None
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                for _ in range(reps):
                    m.Ax_device(yt, xt, stream=s)
            g.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                e0.record(s)
                g.replay()
                e1.record(s)
            s.synchronize()
            graph_us = e0.elapsed_time(e1) * 1e3 / reps
        except RuntimeError as err:  # a capture the library refused: report it
            graph_us = f"not captured: {err}"[:120]
        hx, hy = C.c_void_p(), C.c_void_p()
        T.check(T.lib.tbsla_host_alloc(C.byref(hx), len(xv) * 8))
        T.check(T.lib.tbsla_host_alloc(C.byref(hy), nr * 8))
        np.ctypeslib.as_array(C.cast(hx, C.POINTER(C.c_double)), shape=(len(xv),))[:] = xv
        for _ in range(a.warmup):
            T.check(T.lib.tbsla_Ax(m._h, hy, hx, 0))
        t0 = time.perf_counter()
        for _ in range(reps):
            T.check(T.lib.tbsla_Ax(m._h, hy, hx, 0))
        host_us = (time.perf_counter() - t0) * 1e6 / reps
        T.lib.tbsla_host_free(hx)
        T.lib.tbsla_host_free(hy)
        t0 = time.perf_counter()
        for _ in range(10):
            cpu[name]()
        cpu_us = (time.perf_counter() - t0) * 1e6 / 10
        out[name] = {"device_us": stream_us, "graph_us": graph_us, "host_call_us": host_us,
                     "GB/s_device": B / (stream_us * 1e-6) / 1e9, "bytes_per_ax": B, "cpu_oracle_us": cpu_us}
    clocks = clk.stop()
    csr_us = out["CSR"]["device_us"]
    line = {
        "metric": "SpMV time per Ax, 10^4-row matrix (CSR; every format in `formats`)", "value": csr_us,
        "unit": "us", "n_gpus": ws, "steps": reps, "warmup": a.warmup, "ms_per_step": csr_us * 1e-3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: the reference's own generator recipe (seed 0), no dataset",
        "config": {"workload": "spmv_uniform_rows_n10000_k10_all_formats_dense2000_f64", "n": n, "nnz": nnz,
                   "reps": reps, "l2": "resident (1.4 MB): launch and latency bound", "parallelism": "1 GPU"},
        "formats": out,
        "cpu_baseline": {"value": out["CSR"]["cpu_oracle_us"], "unit": "us", "cores": 1, "kind": "port",
                         "sample": "10 Ax of each format through the oracle's C loops"},
        "e2e": {"value": out["CSR"]["host_call_us"], "unit": "us", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n},
        "gpu_launches": launches, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_formats(a):
    """Every format past L2: the reference's row recipe (column i plus 9
    uniform columns per row, U[-1,1) values, x U[0,1), seed 0) at n = 2^22
    rows (41.9 M entries; x = 32 MiB stays in L2 once read, so each kernel
    streams its own arrays) as COO, SCOO, CSR and ELL, and a 32768 x 16384
    DENSE GEMV (4.3 GB), FP64, and the same GEMV with FP32 and BF16
    values (double-float arithmetic).  Per format: device time per Ax (CUDA
    events on the launching stream, L2 flushed before each step, median),
    algorithmic bytes / time against the measured HBM copy bandwidth, and a
    host call through tbsla_Ax with pinned buffers (x in, y out).  CPU
    baseline: the oracle's loop for each format (CSR on all host threads,
    the others on one)."""
    import ctypes as C

    import numpy as np
    import torch

    import oracle
    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    want = [f.strip().upper() for f in a.formats.split(",")]
    n = a.n
    dm, dk = 32768, 16384
    csr = T.MatrixCSR()
    csr.fill_uniform_rows(n, 10, 0)
    a0 = csr.arrays()
    nnz = int(a0["rowptr"][-1])
    x = T.fill_uniform(n, 0.0, 1.0, 0)
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a0["rowptr"]))
    builders = {
        "COO": lambda: T.MatrixCOO.from_arrays(n, n, rows, a0["colidx"], a0["values"]),
        "SCOO": lambda: T.MatrixSCOO(T.MatrixCOO.from_arrays(n, n, rows, a0["colidx"], a0["values"])),
        "CSR": lambda: csr,
        "ELL": lambda: T.MatrixELL(T.MatrixCOO.from_arrays(n, n, rows, a0["colidx"], a0["values"])),
    }
    # algorithmic bytes per Ax: the stored arrays once, x once, y once
    sparse_bytes = {"COO": nnz * 16 + 16 * n, "SCOO": nnz * 16 + 16 * n,
                    "CSR": nnz * 12 + 4 * (n + 1) + 16 * n, "ELL": nnz * 12 + 16 * n}
    peak, peak_kind = peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    out = {}
    launches = 0
    clk = Clocks(local)
    clk.start()
    dense = None
    for name in ("COO", "SCOO", "CSR", "ELL", "DENSE", "DENSE_F32", "DENSE_BF16"):
        if name not in want:
            continue
        if name.startswith("DENSE"):
            if dense is None:
                dense = T.MatrixDENSE()
                dense.fill_dense_uniform(dm, dk, 0)
            m = dense
            sv = {"DENSE": 8, "DENSE_F32": 4, "DENSE_BF16": 2}[name]
            m.set_precision({8: T.F64, 4: T.F32, 2: T.BF16}[sv])
            xv = T.fill_uniform(dk, 0.0, 1.0, 0)
            nr, B = dm, sv * dm * dk + 8 * dk + 8 * dm
        else:
            m = builders[name]()
            xv, nr, B = x, n, sparse_bytes[name]
            if name == "ELL":
                assert m.info()["max_col"] == 10
        m.upload()
        xt = torch.from_numpy(xv).cuda()
        yt = torch.zeros(nr, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        times = []
        with torch.cuda.stream(s):
            for step in range(a.warmup + a.steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                m.Ax_device(yt, xt, stream=s)
                e1.record(s)
                s.synchronize()
                if step >= a.warmup:
                    times.append(e0.elapsed_time(e1))
        launches += a.steps * m.kernel_launches()
        ms = statistics.median(times)
        hx, hy = C.c_void_p(), C.c_void_p()
        T.check(T.lib.tbsla_host_alloc(C.byref(hx), len(xv) * 8))
        T.check(T.lib.tbsla_host_alloc(C.byref(hy), nr * 8))
        np.ctypeslib.as_array(C.cast(hx, C.POINTER(C.c_double)), shape=(len(xv),))[:] = xv
        for _ in range(a.warmup):
            T.check(T.lib.tbsla_Ax(m._h, hy, hx, 0))
        host = []
        for _ in range(a.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            T.check(T.lib.tbsla_Ax(m._h, hy, hx, 0))
            host.append(time.perf_counter() - t0)
        T.lib.tbsla_host_free(hx)
        T.lib.tbsla_host_free(hy)
        cpu_s = None
        if a.cpu_seconds > 0 and name not in ("DENSE_F32", "DENSE_BF16"):
            if name == "DENSE":
                ad = m.arrays()
                run = lambda: oracle.dense_ax(ad["values"], dm, dk, xv, threads=True)  # noqa: E731
            elif name == "CSR":
                run = lambda: oracle.csr_ax(a0["rowptr"], a0["colidx"], a0["values"], x, threads=True)  # noqa: E731
            elif name == "ELL":
                ae = m.arrays()
                run = lambda: oracle.ell_ax(ae["values"], ae["columns"], n, 10, x)  # noqa: E731
            elif name == "COO":
                run = lambda: oracle.coo_ax(n, rows, a0["colidx"], a0["values"], x)  # noqa: E731
            else:
                run = lambda: oracle.scoo_ax(n, 0, 0, rows, a0["colidx"], a0["values"], x)  # noqa: E731
            t0 = time.perf_counter()
            run()
            cpu_s = time.perf_counter() - t0
        # FP64 instructions per entry: one fused multiply-add (ELL: a rounded
        # product and an add, for the reference's rounding; the narrow DENSE
        # forms none: double-float on the FP32 pipes); gathers: one x entry
        # per stored entry (DENSE reads x in order, from L1)
        entries = dm * dk if name.startswith("DENSE") else nnz
        f64 = 0 if name in ("DENSE_F32", "DENSE_BF16") else entries * (2 if name == "ELL" else 1)
        out[name] = {"device_ms": ms, "GB/s": B / (ms * 1e-3) / 1e9, "frac_of_peak": B / (ms * 1e-3) / 1e9 / peak,
                     "fp64_ops": f64, "gathers": 0 if name.startswith("DENSE") else nnz,
                     "bytes_per_ax": B, "host_call_ms": statistics.median(host) * 1e3,
                     "cpu_oracle_ms": None if cpu_s is None else cpu_s * 1e3,
                     "cpu_threads": (os.cpu_count() if name in ("CSR", "DENSE") else 1)}
        if name.startswith("DENSE"):
            out[name]["launches_per_ax"] = m.kernel_launches()
        del m, xt, yt
        torch.cuda.empty_cache()
    clocks = clk.stop()
    # Floors per Ax: HBM (algorithmic bytes at the measured copy bandwidth),
    # the FP64 pipe (2 lanes per cycle per SM: one warp instruction per 16
    # cycles) and the L1->L2 request rate of the x gathers (one request per
    # gather, about one per SM cycle), at the SM clock sampled during the run.
    f_sm = (clocks.get("sm_mhz") or 2070.0) * 1e6
    for v in out.values():
        fl = {"hbm": v["bytes_per_ax"] / (peak * 1e9) * 1e3, "fp64_pipe": v["fp64_ops"] / (SMS * 2 * f_sm) * 1e3,
              "gather_requests": v["gathers"] / (SMS * f_sm) * 1e3}
        bound = max(fl, key=fl.get)
        v["floors_ms"] = fl
        v["bound"] = bound
        v["frac_of_bound"] = fl[bound] / v["device_ms"]
    head = "CSR" if "CSR" in out else next(iter(out))
    h = out[head]
    line = {
        "metric": "SpMV HBM GB/s (% peak) per format, x L2-resident", "value": h["GB/s"], "unit": "GB/s",
        "n_gpus": ws, "steps": a.steps, "warmup": a.warmup, "ms_per_step": h["device_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: the reference's row recipe (seed 0) at n = 2^22, no dataset",
        "config": {"workload": f"spmv_uniform_rows_n{n}_k10_formats_dense{dm}x{dk}_f64", "n": n, "nnz": nnz,
                   "head_format": head, "l2": "flushed (256 MB write) before each step; arrays > L2",
                   "parallelism": "1 GPU"},
        "formats": out,
        "roofline": {"bound": "hbm", "achieved": h["GB/s"], "peak": peak, "unit": "GB/s",
                     "frac": h["GB/s"] / peak, "peak_source": peak_kind, "traffic": None},
        "cpu_baseline": {"value": (h["bytes_per_ax"] / (h["cpu_oracle_ms"] * 1e-3) / 1e9
                                   if h["cpu_oracle_ms"] else None), "unit": "GB/s",
                         "cores": h["cpu_threads"], "kind": "port",
                         "sample": f"one Ax of the {head} matrix through the oracle's loop"},
        "e2e": {"value": h["bytes_per_ax"] / (h["host_call_ms"] * 1e-3) / 1e9, "unit": "GB/s",
                "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n, "ms_per_step": h["host_call_ms"]},
        "gpu_launches": launches, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_pagerank(a):
    """The PageRank workload: preferential-attachment graph, n = 2^22 nodes,
    Zipf(2.1) out-degrees of mean 16, 5% dangling, seed 2; column-stochastic
    (make_stochastic on the device), FP32 values, beta 0.85, uniform teleport,
    stop at L1 change < 1e-10; then 32 personalised teleport vectors (100
    random nodes each) in one batched solve.  value: GB/s of algorithmic
    bytes over whole solves (host call to host result, wall clock)."""
    import numpy as np
    import torch

    import oracle
    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    n = a.n
    g = T.MatrixCSR()
    g.fill_pa_graph(n, 16.0, 2.1, 4096, 0.05, 2)
    nnz = g.get_nnz()
    s = np.zeros(n)
    g.make_stochastic(s)
    g.set_precision(T.F32)
    g.upload()
    b_it = nnz * 8 + 4 * (n + 1) + 16 * n  # FP32 values + int32 indices, x gathered once, y
    res = np.zeros(n)  # one host result buffer for every solve (touched once, here)
    for _ in range(a.warmup):
        g.page_rank(0.85, 1e-10, 3, out=res)
    clk = Clocks(local)
    clk.start()
    times = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        x, it, err, ok = g.page_rank(0.85, 1e-10, 1000, out=res)
        times.append(time.perf_counter() - t0)
    clocks = clk.stop()
    sec = statistics.mean(times)
    value = b_it * it / sec / 1e9
    # the same solves with the epilogue as a pass of its own over t = A x
    g.set_pagerank_fused(False)
    g.page_rank(0.85, 1e-10, 3, out=res)
    t_sep = []
    for _ in range(max(1, min(a.steps, 3))):
        t0 = time.perf_counter()
        _, it_sep, _, _ = g.page_rank(0.85, 1e-10, 1000, out=res)
        t_sep.append(time.perf_counter() - t0)
    g.set_pagerank_fused(True)
    separate = {"per_iteration_ms": statistics.median(t_sep) * 1e3 / it_sep, "iterations": it_sep,
                "note": "SpMV writes t = A x, then an epilogue pass (two launches per iteration)"}
    rng = np.random.default_rng(2)
    tele = np.zeros((n, 32))
    for k in range(32):
        tele[rng.choice(n, 100, replace=False), k] = 1.0 / 100
    tuned = None
    if a.autotune:
        from tbsla_gb300 import autotune as AT

        r = AT.tune_pagerank_batched(g, tele, T.F32)
        tuned = {"settings": r["settings"], "cached": r["cached"], "key": r["key"], "trials": r.get("trials")}
    xb = np.zeros((n, 32))  # one host result buffer for every batched solve (touched once, here)
    g.page_rank_batched(tele, 0.85, 1e-10, 3, out=xb)
    tbs = []
    clk_b = Clocks(local)
    clk_b.start()
    for _ in range(3):  # whole solves (1 GiB up, 1 GiB back): median of three
        t0 = time.perf_counter()
        X, itb, okb = g.page_rank_batched(tele, 0.85, 1e-10, 1000, out=xb)
        tbs.append(time.perf_counter() - t0)
    clocks_b = clk_b.stop()
    tb = statistics.median(tbs)
    b_itb = nnz * 8 + 4 * (n + 1) + 32 * 24 * n  # X gathered once, Y written, T read
    peak, peak_kind = peaks()
    # oracle on the same FP32-rounded values: equal iteration count, L1 gap;
    # its per-iteration time is the CPU baseline (one host thread)
    arr = g.arrays()
    v32 = arr["values"].astype(np.float32).astype(np.float64)
    t0 = time.perf_counter()
    xo, ito, erro = oracle.pagerank(arr["rowptr"], arr["colidx"], v32, 0.85, 1e-10, it, stop_early=False)
    to = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 values, f64 vectors and sums", "data": "synthetic: seeded PA graph (seed 2), no dataset",
        "config": {"workload": f"pagerank_pa_graph_n{n}_mean16_zipf2.1_dangling5pct_f32", "n": n, "nnz": nnz,
                   "beta": 0.85, "epsilon": 1e-10, "bytes_per_iteration": b_it,
                   "step": "one PageRank solve to 1e-10 (host call to the result in a reused host buffer, "
                           "wall clock)", "parallelism": "1 GPU"},
        "iterations": it, "converged": bool(ok), "last_l1_change": err,
        "per_iteration_ms": sec * 1e3 / it,
        "epilogue": "fused into the sliced-ELL SpMV (one launch per iteration)", "separate_epilogue": separate,
        "roofline": {"bound": "hbm", "achieved": value, "peak": peak, "unit": "GB/s", "frac": value / peak,
                     "peak_source": peak_kind, "traffic": None, "note": "whole solves incl. host set-up"},
        "l1_vs_oracle_equal_iterations": float(np.abs(x - xo).sum()),
        "cpu_baseline": {"value": b_it * ito / to / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                         "sample": f"oracle PageRank, {ito} iterations on the same FP32-rounded graph"},
        "batched": {"nvec": 32, "iterations": itb, "converged": bool(okb), "ms": tb * 1e3,
                    "ms_each": [t * 1e3 for t in tbs], "clocks": clocks_b, "autotune": tuned,
                    "arithmetic": "double-float (float pairs) products and sums (compensated, Dot2), FP64 reductions",
                    "GB/s": b_itb * itb / tb / 1e9, "bytes_per_iteration": b_itb},
        "clocks": clocks, "gpu_launches": a.steps * (it + 3),  # per solve: x_0 fill, one per iteration, sum + scale
    }
    print(json.dumps(line), flush=True)


def cg_systems(T):
    """The batched-CG workload: 64 SPD 7-point diffusion systems, n^3 grids
    with n cycling through 16, 24, ..., 96, coefficients exp(g) of a Gaussian
    field (sigma 1, correlation 8 cells), Dirichlet boundaries, RHS U[-1,1),
    seed 3."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np

    sizes = [16 + 8 * (i % 11) for i in range(64)]

    def make(i):
        m = T.MatrixCSR()
        m.fill_diffusion7(sizes[i], 1.0, 8.0, 3000 + i)
        return m

    with ThreadPoolExecutor(8) as pool:
        systems = list(pool.map(make, range(len(sizes))))
    rhs = np.concatenate([T.fill_uniform(sz ** 3, -1.0, 1.0, 4000 + i) for i, sz in enumerate(sizes)])
    return sizes, systems, rhs


def batched_cg_jacobi(T, reps: int = 3) -> dict:
    """One batched Jacobi-PCG solve of the 64-system workload (FP32 values,
    FP64 refinement every 50 iterations, 1e-8), median of `reps` host calls."""
    sizes, systems, rhs = cg_systems(T)
    bt = T.Batch(systems, T.F32)
    bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=1, refresh=50)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        x, its, rr, ok = bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=1, refresh=50)
        times.append(time.perf_counter() - t0)
    ms = statistics.median(times) * 1e3
    return {"ms": ms, "solves_per_s": len(sizes) / (ms * 1e-3), "iterations_max": int(its.max()),
            "all_converged": bool(ok), "max_rel_residual_fp64": float(rr.max()), "engine": bt.engine(),
            "workload": "batched_cg_diffusion7_64_systems_n16to96_grf_sigma1_corr8_f32_refresh50"}


def run_cg(a):
    """The batched-CG workload: 64 SPD 7-point diffusion systems, n^3 grids
    with n cycling through 16, 24, ..., 96, coefficients exp(g) of a Gaussian
    field (sigma 1, correlation 8 cells), Dirichlet boundaries, RHS U[-1,1),
    seed 3; FP32 values, FP64 residual refresh every 50 iterations, relative
    residual 1e-8.  value: wall time of one batched Jacobi-PCG solve (host
    call to host result); plain CG beside it."""
    import numpy as np
    import torch

    import oracle
    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    sizes, systems, rhs = cg_systems(T)
    N = np.array([sz ** 3 for sz in sizes])
    nnz = np.array([m.get_nnz() for m in systems])
    res = {}
    clk = Clocks(local)
    tuned = {}
    for pre, name in ((0, "cg"), (1, "jacobi_pcg")):
        bt = T.Batch(systems, T.F32)
        if a.autotune:
            from tbsla_gb300 import autotune as AT

            r = AT.tune_batch_cg(bt, rhs, T.F32, precond=pre)
            tuned[name] = {"settings": r["settings"], "cached": r["cached"], "key": r["key"], "trials": r.get("trials")}
        for _ in range(a.warmup):
            bt.cg(rhs, max_iterations=20, rel_tol=1e-8, precond=pre, refresh=50, graph_iters=10)
        if pre == 1:
            clk.start()
        times = []
        for _ in range(a.steps):
            t0 = time.perf_counter()
            x, its, rr, ok = bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=pre, refresh=50,
                                   graph_iters=10)
            times.append(time.perf_counter() - t0)
        # algorithmic bytes per iteration and row, persistent engine (FP32
        # iteration, A in 7 diagonal slots of FP32): q = A p reads the 7
        # slots (28 B), z and p_old once (8 B), writes p and q (8 B); the
        # update reads p, q, r and the correction d, writes r, d and z
        # (28 B), Jacobi adds D^-1 (4 B)
        per_it = N * (28 + 16 + 28 + (4 if pre else 0))
        eng = bt.engine()
        sec = statistics.mean(times)
        res[name] = {"ms": sec * 1e3, "solves_per_s": len(sizes) / sec, "iterations_max": int(its.max()), "engine": eng,
                     "iterations_mean": float(its.mean()), "all_converged": bool(ok),
                     "max_rel_residual_fp64": float(rr.max()),
                     "GB/s": float((per_it * its).sum()) / sec / 1e9}
        del bt
    clocks = clk.stop()
    # CPU baseline: the oracle's Jacobi-PCG on one 48^3 system (one thread)
    k = sizes.index(48)
    arr = systems[k].arrays()
    b48 = rhs[int(N[:k].sum()):int(N[:k + 1].sum())]
    dinv = 1.0 / np.array([arr["values"][arr["rowptr"][i]:arr["rowptr"][i + 1]][
        arr["colidx"][arr["rowptr"][i]:arr["rowptr"][i + 1]] == i].sum() for i in range(N[k])])
    t0 = time.perf_counter()
    _, ito, rro = oracle.cg(arr["rowptr"], arr["colidx"], arr["values"], b48, rel_tol=1e-8, diag_inv=dinv)
    to = time.perf_counter() - t0
    peak, peak_kind = peaks()
    j = res["jacobi_pcg"]
    line = {
        "metric": METRIC, "value": j["ms"], "unit": "ms", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": j["ms"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 values and iteration, f64 refinement", "data": "synthetic: seeded diffusion systems (seed 3)",
        "config": {"workload": "batched_cg_diffusion7_64_systems_n16to96_grf_sigma1_corr8_f32_refresh50",
                   "systems": len(sizes), "unknowns": int(N.sum()), "nnz": int(nnz.sum()), "rel_tol": 1e-8,
                   "step": "one batched Jacobi-PCG solve of all 64 systems (host call, wall clock)",
                   "parallelism": "1 GPU, one block-diagonal matrix, one persistent cooperative launch per solve"},
        "solvers": res, "autotune": tuned or None,
        "roofline": {"bound": "hbm", "achieved": j["GB/s"], "peak": peak, "unit": "GB/s",
                     "frac": j["GB/s"] / peak, "peak_source": peak_kind, "traffic": None},
        "cpu_baseline": {"value": to * 1e3, "unit": "ms", "cores": 1, "kind": "port",
                         "sample": f"oracle Jacobi-PCG on the one 48^3 system: {ito} iterations, "
                                   f"residual {rro:.2e}"},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


REFRESH_OPTIONS = (50, 400, 0)  # FP64 refinement every k iterations; 0: only when the recursion says converged


def learned_vs_jacobi(a, T, local: int) -> dict:
    """The learned-preconditioner workload: the network is trained on the
    GPU (one Adam step per system, lr 1e-3, 8 Gaussian probes) on diffusion
    systems with n in [32, 64] (seeds 1000..), then held-out 128^3 systems
    (seeds 9000.., RHS U[-1,1)) are solved in one batch by Jacobi-PCG and by
    PCG with M^-1 = L L^T from the network; FP32 values, FP64 refinement, to
    a 1e-8 FP64-verified relative residual, both in the persistent engine.
    The learned solver's timed region holds the network inference on the
    GPU (L written into the batch's factor storage) AND the solve; Jacobi's
    holds the building of D^-1 and its solve.  Wall clock of the host calls.

    Every refinement interval of REFRESH_OPTIONS is timed for both solvers
    (each refinement restarts the FP32 recursion from the FP64 true residual,
    and frequent restarts cost Jacobi, with its slower convergence, more
    than the learned solver); the ratio is each solver at its own fastest
    interval.  The ratio at the shared 50-iteration interval is reported
    beside it."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np

    def system(n, seed):
        m = T.MatrixCSR()
        m.fill_diffusion7(n, 1.0, 8.0, seed)
        return m

    rng = np.random.default_rng(5)
    sizes = rng.integers(32, 65, a.train_systems)
    net = T.MPNN(1)
    t0 = time.time()
    losses = []
    total = a.train_systems * a.epochs
    with ThreadPoolExecutor(4) as pool:
        # systems are regenerated each epoch (same seeds) rather than held
        def sub(k):
            return pool.submit(system, int(sizes[k % a.train_systems]), 1000 + k % a.train_systems)

        futs = [sub(k) for k in range(min(8, total))]
        for k in range(total):
            A = futs[k].result()
            if k + 8 < total:
                futs.append(sub(k + 8))
            losses.append(net.train_step(A, probes=8, seed=k, lr=1e-3))
            futs[k] = None
    t_train = time.time() - t0
    t0 = time.time()
    with ThreadPoolExecutor(8) as pool:
        held = list(pool.map(lambda k: system(a.eval_n, 9000 + k), range(a.eval_systems)))
    N = a.eval_n ** 3
    rhs = np.concatenate([T.fill_uniform(N, -1.0, 1.0, 9100 + k) for k in range(a.eval_systems)])
    bt = T.Batch(held, T.F32)
    t_setup = time.time() - t0
    fprec = T.BF16 if a.factor_prec == "bf16" else T.F32
    reps = max(1, min(a.steps, 3))

    def jacobi(refresh):
        return bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=1, refresh=refresh), 0.0

    def learned(refresh):
        t1 = time.perf_counter()
        bt.factor_mpnn(net, fprec)
        tf = time.perf_counter() - t1
        return bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=2, refresh=refresh), tf

    clk = Clocks(local)
    clk.start()
    runs = {"jacobi_pcg": {}, "learned_pcg": {}}
    fb_count = 0
    for refresh in REFRESH_OPTIONS:
        for name, fn in (("jacobi_pcg", jacobi), ("learned_pcg", learned)):
            fn(refresh)  # warm-up: the solve graph of this setting is captured, scratch allocated
            ts, tfs = [], []
            for _ in range(reps):
                t1 = time.perf_counter()
                (x, it, rr, ok), tf = fn(refresh)
                ts.append(time.perf_counter() - t1)
                tfs.append(tf)
            r = {"ms": statistics.median(ts) * 1e3, "iterations_mean": float(it.mean()),
                 "iterations_max": int(it.max()), "all_converged": bool(ok), "max_rel_residual_fp64": float(rr.max())}
            if name == "learned_pcg":
                fb, _ = bt.fallbacks()
                fb_count = max(fb_count, int((fb != 0).sum()))
                r["factor_ms"] = statistics.median(tfs) * 1e3
                r["solve_ms"] = r["ms"] - r["factor_ms"]
            runs[name][str(refresh)] = r
    clocks = clk.stop()
    eng = bt.engine()
    best = {k: min(v.items(), key=lambda kv: kv[1]["ms"]) for k, v in runs.items()}
    res = {k: dict(b[1], refresh=int(b[0])) for k, b in best.items()}
    res["learned_pcg"]["fallbacks"] = fb_count
    ratio = res["learned_pcg"]["ms"] / res["jacobi_pcg"]["ms"]
    ratio50 = runs["learned_pcg"]["50"]["ms"] / runs["jacobi_pcg"]["50"]["ms"]
    return {"ratio": ratio, "ratio_refresh50": ratio50, "solvers": res, "sweep": runs, "reps": reps,
            "engine": eng, "clocks": clocks,
            "timed": "learned: network inference on the GPU + solve; jacobi: D^-1 + solve (same batch); "
                     "each at its fastest refinement interval of " + str(list(REFRESH_OPTIONS)),
            "systems": a.eval_systems, "n": a.eval_n, "unknowns": a.eval_systems * N, "factor_storage": a.factor_prec,
            "train": {"systems": a.train_systems, "epochs": a.epochs, "adam_steps": total,
                      "seconds": round(t_train, 1), "loss_first_50": float(np.mean(losses[:50])),
                      "loss_last_50": float(np.mean(losses[-50:]))},
            "setup_s": round(t_setup, 1)}


def run_learned(a):
    """--workload learned: the learned-vs-Jacobi measurement on its own line.
    value: (network inference + learned-PCG solve) / (Jacobi-PCG solve)."""
    import torch

    import tbsla_gb300 as T

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    T.device_init(local)
    r = learned_vs_jacobi(a, T, local)
    line = {
        "metric": METRIC, "value": r["ratio"], "unit": "learned-PCG time / Jacobi-PCG time", "n_gpus": ws,
        "steps": r["reps"], "warmup": 1, "ms_per_step": r["solvers"]["learned_pcg"]["ms"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 weights / f32 network; f32 values and iteration, f64 refinement",
        "data": "synthetic: seeded diffusion systems (train seeds 1000.., held-out 9000..)",
        "config": {"workload": f"learned_pcg_mpnn3x32_train{a.train_systems}_n32to64_eval{a.eval_systems}x{a.eval_n}^3",
                   "unknowns_per_system": a.eval_n ** 3, "rel_tol": 1e-8, "factor_storage": a.factor_prec,
                   "step": r["timed"], "parallelism": "1 GPU, one persistent launch per solve"},
        "ratio_refresh50": r["ratio_refresh50"],
        "train": r["train"], "solvers": r["solvers"], "sweep": r["sweep"], "engine": r["engine"], "clocks": r["clocks"],
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "small":
        run_small(args)
    elif args.workload == "formats":
        run_formats(args)
    elif args.workload == "pagerank":
        run_pagerank(args)
    elif args.workload == "cg":
        run_cg(args)
    elif args.workload == "learned":
        run_learned(args)
    else:
        run_ours(args)
