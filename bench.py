"""Benchmark of the load-balanced CSR SpMV/SpMM path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--schedule S] [--value-dtype f32|bf16|f16]

Default workload: y = A x, merge-path schedule, FP32 values, on a 2^20 x 2^20
power-law matrix (Zipf 2.0 row lengths, min 1, cap 100,000, rescaled to
~16M nonzeros, columns uniform and sorted per row, values and x uniform in
[-1, 1], int32 indices, seed 1) -- synthetic, standing in for the
reference's SuiteSparse inputs.  A step is one SpMV over the whole matrix;
the L2 cache is flushed (512 MiB write, outside the timed kernel) before
every step.  The metric is achieved bandwidth in GB/s of the algorithmic
(compulsory) bytes:
    nnz*(value bytes + 4) + 4*(rows+1) + 4*cols + 4*rows (+ 4*rows of scales).

`value` is timed on the device with CUDA events around every SpMV launch
(inputs resident in HBM); `e2e` is the same metric through the C ABI call
with host buffers, the H2D copy of the matrix and x (pinned memory) and the
D2H copy of y inside the timed region.  `--impl reference` times the
reference's CPU SpMV loop (examples/spmv/helpers.hxx:106-112, restated in
oracle/oracle.c, rows split over every host core) on the same workload.

Under torchrun with N > 1 every rank runs an independent replica (SpMV of
one matrix does not shard on this pool); value is the sum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

L2_FLUSH_BYTES = 512 << 20


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_for(workload_key):
    """DRAM bytes per launch of the dominant kernel from a committed ncu
    summary (profiles/traffic.json), or None."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(workload_key)
    return None if v is None else float(v.get("dram_bytes_per_launch"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workloads
def make_workload(name, device, value_dtype):
    """Returns dict(off, idx, vals, x, rows, cols, desc) on `device` (FP32
    values; quantised later if value_dtype != f32)."""
    from edge_loops_gb300 import synth
    if name == "spmv_powerlaw":
        off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000,
                                                  exponent=2.0, cap=100_000, seed=1,
                                                  device=device)
        desc = ("SpMV power-law 2^20 x 2^20, Zipf 2.0 rows (min 1, cap 100000) rescaled to "
                "~16M nnz, uniform sorted columns, U[-1,1] values and x, seed 1")
    elif name == "spmv_uniform1k":
        off, idx, vals, x, cols = synth.uniform_rows(rows=1000, cols=1000, per_row=10, seed=0,
                                                     device=device)
        desc = "SpMV 1000 x 1000, 10 nnz/row, U[-1,1], seed 0"
    elif name == "spmv_stencil":
        off, idx, vals, x, cols = synth.stencil27(n=160, seed=2, device=device)
        desc = ("SpMV 27-point stencil on 160^3 (4,096,000 rows, 109,215,352 nnz), diag 26.5, "
                "off-diag U[-1,0], x U[-1,1], seed 2")
    else:
        raise SystemExit(f"unknown workload {name}")
    rows = off.numel() - 1
    return dict(off=off, idx=idx, vals=vals, x=x, rows=rows, cols=cols, desc=desc)


def value_bytes(dt):
    return 4 if dt == "f32" else 2


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world):
    import torch
    from edge_loops_gb300 import api, synth

    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    W = make_workload(args.workload, dev, args.value_dtype)
    A = api.CSR(W["off"], W["idx"], W["vals"], W["rows"], W["cols"])
    if args.value_dtype != "f32":
        tdt = torch.bfloat16 if args.value_dtype == "bf16" else torch.float16
        A = A.quantized(tdt, per_row_scale=True)
    x = W["x"]
    y = torch.empty(A.rows, dtype=torch.float32, device=dev)
    nbytes = synth.algorithmic_bytes(A.rows, A.cols, A.nnz, value_bytes(args.value_dtype),
                                     row_scale=A.row_scale is not None)
    ws = api.Workspace()
    opts = dict(items_per_thread=args.ipt) if args.ipt else {}
    if args.variant:
        opts["variant"] = args.variant
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def step():
        api.spmv(A, x, y, schedule=args.schedule, workspace=ws, **opts)

    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    flags = ws.errors()
    if flags:
        raise SystemExit(f"device error flags {flags:#x} during warm-up")

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]  # ms
    kern_ms = sum(times)
    if world > 1:
        t = torch.tensor([kern_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        kern_ms = float(t.item())
    flags = ws.errors()
    if flags:
        raise SystemExit(f"device error flags {flags:#x} in the timed region")
    ms_per_step = kern_ms / args.steps
    value = world * nbytes * args.steps / (kern_ms * 1e-3) / 1e9  # GB/s, all ranks

    # ---- correctness of the timed output (size-independent properties)
    check = verify(args, A, x, y, W)

    # ---- e2e through the C ABI with host buffers
    e2e = run_e2e(args, A, W, nbytes, dev)

    peak, peak_kind = measured_peaks()
    achieved = nbytes / (ms_per_step * 1e-3) / 1e9
    key = f"{args.workload}:{args.schedule}:{args.value_dtype}"
    traffic = traffic_for(key)
    line = {
        "metric": "SpMV achieved HBM bandwidth (algorithmic bytes / kernel time)",
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if args.value_dtype == "f32" else f"{args.value_dtype} values, f32 accumulate",
        "data": "synthetic (seeded generator; SuiteSparse not available)",
        "config": {
            "workload": W["desc"],
            "schedule": args.schedule,
            "rows": A.rows, "cols": A.cols, "nnz": A.nnz,
            "value_dtype": args.value_dtype,
            "algorithmic_bytes_per_step": nbytes,
            "l2": "flushed before every step (512 MiB write, outside the timed kernel)",
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 2),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "peak_source": peak_kind,
            "traffic": traffic,
        },
        "e2e": e2e,
        "gpu_launches": args.steps,
        "clocks": clocks,
        "check": check,
        "wall_s_timed_region": round(wall, 4),
    }
    if rank == 0 and args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(W, args, budget_s=args.cpu_budget)
    return line


def verify(args, A, x, y, W):
    """Parity of the benchmarked output: the oracle on the same input, in full
    (the CPU loop finishes in about a second at these sizes)."""
    import numpy as np
    import oracle
    off = W["off"].cpu().numpy()
    idx = W["idx"].cpu().numpy()
    xx = x.cpu().numpy()
    yy = y.cpu().numpy()
    if args.value_dtype == "f32":
        vals = W["vals"].cpu().numpy()
        scale = None
    else:
        vals = A.values.float().cpu().numpy()
        scale = A.row_scale.cpu().numpy()
    y64, yabs = oracle.spmv_f64(off, idx, vals, xx, row_scale=scale)
    u = 2.0 ** -24
    n = np.diff(off.astype(np.int64)) + 2
    bound = (n * u / (1 - n * u)) * yabs
    bad = int(np.sum(np.abs(yy - y64) > bound))
    comp, norm = oracle.error_metrics(yy, y64, yabs)
    out = {"rows_outside_fp32_bound": bad, "max_rel_err_vs_fp64_stored": comp,
           "normwise_err_vs_fp64_stored": norm}
    if args.value_dtype != "f32":
        y64o, yabso = oracle.spmv_f64(off, idx, W["vals"].cpu().numpy(), xx)
        c2, n2 = oracle.error_metrics(yy, y64o, yabso)
        out["max_rel_err_vs_fp64_fp32matrix"] = c2
        out["normwise_err_vs_fp64_fp32matrix"] = n2
    if bad:
        raise SystemExit(f"benchmarked y fails the oracle check: {out}")
    return out


def run_e2e(args, A, W, nbytes, dev):
    """Same metric through el_spmv with host inputs: per step H2D of offsets,
    indices, values and x from pinned memory, the SpMV, D2H of y."""
    import torch
    from edge_loops_gb300 import api
    h_off = A.offsets.cpu().pin_memory()
    h_idx = A.indices.cpu().pin_memory()
    h_val = A.values.cpu().pin_memory()
    h_x = W["x"].cpu().pin_memory()
    h_sc = A.row_scale.cpu().pin_memory() if A.row_scale is not None else None
    h_y = torch.empty(A.rows, dtype=torch.float32).pin_memory()
    d_off, d_idx, d_val = torch.empty_like(A.offsets), torch.empty_like(A.indices), \
        torch.empty_like(A.values)
    d_sc = torch.empty_like(A.row_scale) if h_sc is not None else None
    d_x = torch.empty_like(W["x"])
    d_y = torch.empty(A.rows, dtype=torch.float32, device=dev)
    B = api.CSR(d_off, d_idx, d_val, A.rows, A.cols, row_scale=d_sc)
    ws = api.Workspace()
    stream = torch.cuda.current_stream()
    h2d = sum(t.numel() * t.element_size() for t in (h_off, h_idx, h_val, h_x) if t is not None)
    if h_sc is not None:
        h2d += h_sc.numel() * 4
    d2h = h_y.numel() * 4

    def step():
        d_off.copy_(h_off, non_blocking=True)
        d_idx.copy_(h_idx, non_blocking=True)
        d_val.copy_(h_val, non_blocking=True)
        if h_sc is not None:
            d_sc.copy_(h_sc, non_blocking=True)
        d_x.copy_(h_x, non_blocking=True)
        api.spmv(B, d_x, d_y, schedule=args.schedule, workspace=ws)
        h_y.copy_(d_y, non_blocking=True)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    steps = max(5, min(args.steps, 50))
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(steps):
        step()
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / steps
    if ws.errors():
        raise SystemExit("device error flags in the e2e run")
    return {"value": round(nbytes / (ms * 1e-3) / 1e9, 2), "unit": "GB/s",
            "ms_per_step": round(ms, 4), "steps": steps,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(W, args, budget_s=15.0, threads=None):
    """The reference's CPU SpMV loop (oracle restatement, FP32, rows split
    over host threads) on the same workload, repeated for about budget_s."""
    import numpy as np
    import oracle
    from edge_loops_gb300 import synth
    threads = threads or os.cpu_count() or 1
    off = W["off"].cpu().numpy()
    idx = W["idx"].cpu().numpy()
    vals = W["vals"].cpu().numpy()
    x = W["x"].cpu().numpy()
    nbytes = synth.algorithmic_bytes(W["rows"], W["cols"], len(idx), 4)
    oracle.spmv_f32_mt(off, idx, vals, x, threads)  # warm-up
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or len(times) < 3:
        t0 = time.perf_counter()
        oracle.spmv_f32_mt(off, idx, vals, x, threads)
        times.append(time.perf_counter() - t0)
        if len(times) >= 2000:
            break
    med = statistics.median(times)
    return {"value": round(nbytes / med / 1e9, 3), "unit": "GB/s", "cores": threads,
            "kind": "port",
            "sample": (f"whole matrix (FP32 values), {len(times)} repetitions in "
                       f"~{budget_s:.0f} s, median; reference loop examples/spmv/"
                       f"helpers.hxx:106-112 restated in oracle/oracle.c, rows split "
                       f"over {threads} threads"),
            "ms_per_step": round(med * 1e3, 3)}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU SpMV loop on the host cores, on
    the same workload (FP32), one whole-matrix SpMV per step."""
    if rank != 0:
        return None
    import oracle
    from edge_loops_gb300 import synth
    oracle.build()
    W = make_workload(args.workload, "cpu", "f32")
    off = W["off"].numpy()
    idx = W["idx"].numpy()
    vals = W["vals"].numpy()
    x = W["x"].numpy()
    nbytes = synth.algorithmic_bytes(W["rows"], W["cols"], len(idx), 4)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.spmv_f32_mt(off, idx, vals, x, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.spmv_f32_mt(off, idx, vals, x, threads)
    dt = time.perf_counter() - t0
    value = nbytes * args.steps / dt / 1e9
    return {
        "impl": "reference",
        "metric": "SpMV achieved HBM bandwidth (algorithmic bytes / kernel time)",
        "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator; SuiteSparse not available)",
        "config": {"workload": W["desc"], "schedule": "reference CPU loop (serial per row)",
                   "rows": W["rows"], "cols": W["cols"], "nnz": int(len(idx)),
                   "value_dtype": "f32", "algorithmic_bytes_per_step": nbytes},
        "cpu_baseline": {
            "value": round(value, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": (f"whole matrix per step, {args.steps} steps after {args.warmup} "
                       f"warm-up; reference loop examples/spmv/helpers.hxx:106-112 restated "
                       f"in oracle/oracle.c, rows split over {threads} threads")},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spmv_powerlaw")
    ap.add_argument("--schedule", default="merge_path_flat")
    ap.add_argument("--value-dtype", default="f32", choices=["f32", "bf16", "f16"])
    ap.add_argument("--ipt", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0,
                    help="merge_path kernel: 0 warp-streaming, 1 CTA ring")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return

    import torch
    from edge_loops_gb300 import build as b
    b.build()
    import oracle
    oracle.build()
    if world > 1:
        torch.distributed.init_process_group(
            "nccl", device_id=torch.device("cuda", _env_int("LOCAL_RANK", 0)))
    line = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
