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
D2H copy of y inside the timed region (row blocks of --e2e-block-nnz
nonzeros, default the library's); `graph_replay` times 100 SpMVs captured
in one CUDA graph and replayed without L2 flushes between them; `secondary`
measures the 27-point stencil (FP32, BF16, FP16) and the 4096-matrix batch in
the same run.  Every output is checked against an FP64 evaluation.
`--impl reference` times the reference's CPU SpMV loop
(examples/spmv/helpers.hxx:106-112, restated in oracle/oracle.c, rows split
over every host core) on the same workload, and the reference's own
merge_path_flat CUDA kernel where its cubin was built.

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
        return self.summarize(self.lines)

    @staticmethod
    def summarize(lines):
        """Median SM clock, highest max clock and the throttle reasons seen
        Active, from nvidia-smi CSV lines in FIELDS order (others skipped)."""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
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


# ------------------------------------------------------------- FP64 checker
# The benchmark checks its own outputs with this plain FP64 evaluation
# (numpy, row blocks of a few million nonzeros); the CPU oracle package is
# used only by the CPU-baseline and reference legs.
def fp64_spmv(off, idx, vals, x, scale=None, chunk=1 << 24):
    """(y, sum_j |a_ij x_j|) in FP64 for a host CSR; vals any float dtype
    (16-bit values given as their float32 widening), scale per row or None."""
    import numpy as np
    off = np.asarray(off, dtype=np.int64)
    rows = len(off) - 1
    x64 = np.asarray(x, dtype=np.float64)
    y = np.zeros(rows)
    ya = np.zeros(rows)
    r0 = 0
    while r0 < rows:
        r1 = int(np.searchsorted(off, off[r0] + chunk, side="right")) - 1
        r1 = min(max(r1, r0 + 1), rows)
        n0, n1 = int(off[r0]), int(off[r1])
        row_of = np.repeat(np.arange(r1 - r0), np.diff(off[r0:r1 + 1]))
        prod = np.asarray(vals[n0:n1], dtype=np.float64) * x64[np.asarray(idx[n0:n1])]
        y[r0:r1] = np.bincount(row_of, prod, minlength=r1 - r0)
        ya[r0:r1] = np.bincount(row_of, np.abs(prod), minlength=r1 - r0)
        r0 = r1
    if scale is not None:
        sc = np.asarray(scale, dtype=np.float64)
        y *= sc
        ya *= np.abs(sc)
    return y, ya


def fp32_bound(off, yabs, extra=2):
    """|fp32 sum - exact| <= gamma_(n+extra) * sum |a x| for any summation
    order of a row's n products (each rounded once)."""
    import numpy as np
    u = 2.0 ** -24
    n = np.diff(np.asarray(off, dtype=np.int64)) + extra
    return (n * u / (1 - n * u)) * yabs


def rel_errors(y, y64, yabs):
    """(max_i |y_i - y64_i| / sum_j |a_ij x_j|, ||y - y64||_inf / ||y64||_inf)."""
    import numpy as np
    d = np.abs(np.asarray(y, dtype=np.float64) - y64)
    if not len(d):
        return 0.0, 0.0
    comp = float(np.max(d / np.where(yabs > 0, yabs, 1.0)))
    ninf = float(np.max(np.abs(y64)))
    return comp, float(np.max(d) / ninf) if ninf > 0 else float(np.max(d))


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
        A = A.quantized(tdt, per_row_scale=not args.no_row_scale)
    x = W["x"]
    y = torch.empty(A.rows, dtype=torch.float32, device=dev)
    nbytes = synth.algorithmic_bytes(A.rows, A.cols, A.nnz, value_bytes(args.value_dtype),
                                     row_scale=A.row_scale is not None)
    ws = api.Workspace()
    opts = dict(items_per_thread=args.ipt) if args.ipt else {}
    if args.variant:
        opts["variant"] = args.variant
    if args.row_weight:
        opts["row_weight"] = args.row_weight
    if args.nz_per_lane:
        opts["nz_per_lane"] = args.nz_per_lane
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
        from edge_loops_gb300.dist import max_over_ranks
        kern_ms = max_over_ranks(kern_ms, device=dev)
    flags = ws.errors()
    if flags:
        raise SystemExit(f"device error flags {flags:#x} in the timed region")
    ms_per_step = kern_ms / args.steps
    value = world * nbytes * args.steps / (kern_ms * 1e-3) / 1e9  # GB/s, all ranks

    # ---- correctness of the timed output (size-independent properties)
    check = verify(args, A, x, y, W)

    # ---- the same SpMV replayed back to back from a CUDA graph
    replay = graph_replay(step, stream, nbytes)
    if ws.errors():
        raise SystemExit("device error flags in the graph replay")

    # ---- e2e through the C ABI with host buffers
    e2e = run_e2e(args, A, W, nbytes, dev, world)

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
        "graph_replay": replay,
        "gpu_launches": args.steps,
        "clocks": clocks,
        "check": check,
        "wall_s_timed_region": round(wall, 4),
    }
    if rank == 0 and args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(W, args, budget_s=args.cpu_budget)
    if rank == 0 and args.secondary and args.workload == "spmv_powerlaw" and \
            args.schedule == "merge_path_flat" and args.value_dtype == "f32" and not args.variant:
        del A, x, y, W
        torch.cuda.empty_cache()
        line["secondary"] = run_secondary(args, dev)
    return line


def run_secondary(args, dev):
    """The other configurations of the target, measured in the same run as
    the headline (same timing rules: L2 flushed before every step, outside
    the CUDA events): the 27-point stencil on 160^3 with FP32, BF16 and FP16
    values (16-bit with per-row scales), with merge_path and with the schedule
    el_spmv_select picks for it, the 4096-matrix batch
    (measure_batched: BF16 and FP32 plans and the plain FP32 kernel once per
    matrix), and the SpMM on the ~8M-nonzero power-law matrix at n = 32 and
    128 (FP32 and BF16 B).  Every output is checked against FP64."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api, synth
    peak, kind = measured_peaks()
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    stream = torch.cuda.current_stream()
    steps = max(5, min(args.steps, 20))
    warm = max(3, min(args.warmup, 5))
    out = {"steps": steps, "warmup": warm, "peak_GBps": peak, "peak_source": kind}

    off, idx, vals, x, rows = synth.stencil27(n=160, seed=2, device=dev)
    A = api.CSR(off, idx, vals, rows, rows)
    o, i, v, xh = (t.cpu().numpy() for t in (off, idx, vals, x))
    y64, yabs = fp64_spmv(o, i, v, xh)
    ws = api.Workspace()
    # el_spmv_select's choice from the row statistics (the same for every
    # value type): thread_mapped's staged kernel on these short coherent rows
    sel_sched, sel_opts = api.select_schedule(A, workspace=ws)
    st = {"workload": "27-point stencil on 160^3 (4,096,000 rows, 109,215,352 nnz), diag 26.5, "
                      "off-diag U[-1,0], x U[-1,1], seed 2; merge_path, and under 'selected' "
                      "the schedule el_spmv_select picks",
          "selected_schedule": {"schedule": sel_sched, **sel_opts}}
    for dt in ("f32", "bf16", "f16"):
        Q = A if dt == "f32" else A.quantized(
            torch.bfloat16 if dt == "bf16" else torch.float16, per_row_scale=True)
        nb = synth.algorithmic_bytes(rows, rows, Q.nnz, 4 if dt == "f32" else 2,
                                     row_scale=Q.row_scale is not None)
        if dt == "f32":
            q64, qabs = y64, yabs
        else:
            q64, qabs = fp64_spmv(o, i, Q.values.float().cpu().numpy(), xh,
                                  Q.row_scale.cpu().numpy())
        for key, sched, opts in (("merge_path", "merge_path_flat", {}),
                                 ("selected", sel_sched, sel_opts)):
            y = torch.empty(rows, device=dev)
            ms = _time_device(lambda: api.spmv(Q, x, y, schedule=sched, workspace=ws, **opts),
                              steps, warm, flush, stream)
            if ws.errors():
                raise SystemExit(f"device error flags in the stencil {dt} SpMV ({key})")
            yy = y.cpu().numpy()
            bad = int(np.sum(np.abs(yy - q64) > fp32_bound(o, qabs)))
            comp, _ = rel_errors(yy, y64, yabs)
            if bad or comp > 1e-2:
                raise SystemExit(f"stencil {dt} ({key}): {bad} rows outside the FP32 bound, "
                                 f"err {comp}")
            gbps = nb / (ms * 1e-3) / 1e9
            r = {"us": round(ms * 1e3, 2), "GBps": round(gbps, 1),
                 "frac": round(gbps / peak, 4), "algorithmic_bytes": nb,
                 "rows_outside_fp32_bound": bad, "max_rel_err_vs_fp64_of_fp32_matrix": comp}
            tkey = "merge_path_flat" if key == "merge_path" else \
                sched + ("_staged" if opts.get("variant") == 1 else "")
            r["traffic"] = traffic_for(f"spmv_stencil:{tkey}:{dt}")
            if key == "merge_path":
                st[dt] = r
            else:
                st[dt]["selected"] = r
            del y
        del Q
    for dt in ("bf16", "f16"):
        st[dt]["time_vs_f32"] = round(st[dt]["us"] / st["f32"]["us"], 4)
        st[dt]["selected"]["time_vs_f32"] = round(
            st[dt]["selected"]["us"] / st["f32"]["selected"]["us"], 4)
    out["stencil160"] = st
    del A, off, idx, vals, x, ws
    torch.cuda.empty_cache()

    b = measure_batched(dev, steps, warm, flush, stream, ("bf16",))
    b["workload"] = ("4096 square CSRs, rows log-uniform [64, 65536], log-normal nnz/row "
                     "(mean 8, sigma 1), seed 4; one persistent launch per plan in a CUDA graph")
    for dt in ("f32", "bf16"):
        b[dt]["frac"] = round(b[dt]["GBps"] / peak, 4)
        b[dt]["traffic"] = traffic_for(f"spmv_batched:{dt}")
    out["batched4096"] = b
    torch.cuda.empty_cache()

    A = spmm_matrix(dev)
    sp = {"workload": "SpMM C = A B, A power-law 2^20 x 2^20 ~8M nnz (Zipf 2.0, cap 1e5, seed 3), "
                      "B 2^20 x n uniform [-1, 1]; merge_path; GB/s of the compulsory bytes "
                      "(A + B + C once), the gather model (a B row per nonzero) beside it"}
    for n, bdt in ((32, "f32"), (128, "f32"), (128, "bf16")):
        r = measure_spmm(A, n, bdt, "merge_path_flat", steps, warm, flush, stream)
        sp[f"n{n}_{bdt}"] = {"ms": round(r["ms"], 4), "GBps": round(r["GBps"], 1),
                             "frac": round(r["GBps"] / peak, 4),
                             "GBps_gather_model": round(r["GBps_gather_model"], 1),
                             "entries_outside_fp32_bound_of_2048_rows": r["entries_outside_fp32_bound"],
                             "traffic": traffic_for(f"spmm_powerlaw:merge_path_flat:{bdt}:{n}")}
    out["spmm_powerlaw8M"] = sp
    del A
    torch.cuda.empty_cache()
    return out


def graph_replay(step, stream, nbytes, reps=100, runs=5):
    """`reps` SpMVs captured in one CUDA graph and replayed back to back (no
    host launch cost, no L2 flush between them): the median over `runs`
    replays of the time per SpMV.  Reported beside the flushed per-step
    figure, which stays the headline."""
    import torch
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for _ in range(reps):
            step()
    graph.replay()
    torch.cuda.synchronize()
    ts = []
    for _ in range(runs):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        graph.replay()
        e.record(stream)
        torch.cuda.synchronize()
        ts.append(s.elapsed_time(e) / reps)
    ts.sort()
    ms = ts[len(ts) // 2]
    return {"reps": reps, "runs": runs, "ms_per_spmv": round(ms, 5),
            "GBps_per_gpu": round(nbytes / (ms * 1e-3) / 1e9, 2),
            "l2": "not flushed between the SpMVs of a replay"}


def verify(args, A, x, y, W):
    """Parity of the benchmarked output: FP64 on the same input, every row,
    within the order-free FP32 bound (of the stored values for 16-bit runs)
    and, for 16-bit values, the error against FP64 of the FP32 matrix."""
    import numpy as np
    off = W["off"].cpu().numpy()
    idx = W["idx"].cpu().numpy()
    xx = x.cpu().numpy()
    yy = y.cpu().numpy()
    if args.value_dtype == "f32":
        vals = W["vals"].cpu().numpy()
        scale = None
    else:
        vals = A.values.float().cpu().numpy()
        scale = A.row_scale.cpu().numpy() if A.row_scale is not None else None
    y64, yabs = fp64_spmv(off, idx, vals, xx, scale)
    bad = int(np.sum(np.abs(yy - y64) > fp32_bound(off, yabs)))
    comp, norm = rel_errors(yy, y64, yabs)
    out = {"rows_outside_fp32_bound": bad, "max_rel_err_vs_fp64_stored": comp,
           "normwise_err_vs_fp64_stored": norm}
    if args.value_dtype != "f32":
        y64o, yabso = fp64_spmv(off, idx, W["vals"].cpu().numpy(), xx)
        c2, n2 = rel_errors(yy, y64o, yabso)
        out["max_rel_err_vs_fp64_fp32matrix"] = c2
        out["normwise_err_vs_fp64_fp32matrix"] = n2
    if bad:
        raise SystemExit(f"benchmarked y fails the FP64 check: {out}")
    return out


def run_e2e(args, A, W, nbytes, dev, world=1):
    """The same metric through the C ABI with host buffers (pinned): per step
    the matrix, x and y cross the host link inside the timed region.
    `value`: el_spmv_host (row blocks copied on a second stream while the
    previous block is multiplied, y blocks copied back); also reported: the
    plain sequence of H2D copies, el_spmv and the D2H copy of y.  With
    several ranks every timing starts after a barrier, the slowest rank's
    time counts, and value and bytes are the whole job's."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api
    h_off = A.offsets.cpu().pin_memory()
    h_idx = A.indices.cpu().pin_memory()
    h_val = A.values.cpu().pin_memory()
    h_x = W["x"].cpu().pin_memory()
    h_sc = A.row_scale.cpu().pin_memory() if A.row_scale is not None else None
    h_y = torch.empty(A.rows, dtype=torch.float32).pin_memory()
    Ah = api.CSR(h_off, h_idx, h_val, A.rows, A.cols, row_scale=h_sc)
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

    def step_stream():
        api.spmv_host(Ah, h_x, h_y, schedule=args.schedule, workspace=ws,
                      block_nnz=args.e2e_block_nnz)

    def step_copy():
        d_off.copy_(h_off, non_blocking=True)
        d_idx.copy_(h_idx, non_blocking=True)
        d_val.copy_(h_val, non_blocking=True)
        if h_sc is not None:
            d_sc.copy_(h_sc, non_blocking=True)
        d_x.copy_(h_x, non_blocking=True)
        api.spmv(B, d_x, d_y, schedule=args.schedule, workspace=ws)
        h_y.copy_(d_y, non_blocking=True)

    def timed(step):
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        steps = max(5, min(args.steps, 50))
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()
        s.record(stream)
        for _ in range(steps):
            step()
        e.record(stream)
        torch.cuda.synchronize()
        if ws.errors():
            raise SystemExit("device error flags in the e2e run")
        ms = s.elapsed_time(e)
        if world > 1:
            from edge_loops_gb300.dist import max_over_ranks
            ms = max_over_ranks(ms, device=dev)
        return ms / steps, steps

    ms_copy, _ = timed(step_copy)
    ms, steps = timed(step_stream)
    # the streamed y against FP64 (block borders change the merge ranges, so
    # the check is the FP32 bound, not equality)
    off = W["off"].cpu().numpy()
    vals = A.values.float().cpu().numpy()
    y64, yabs = fp64_spmv(off, W["idx"].cpu().numpy(), vals, W["x"].cpu().numpy(),
                          None if h_sc is None else h_sc.numpy())
    bad = int(np.sum(np.abs(h_y.numpy().astype(np.float64) - y64) > fp32_bound(off, yabs)))
    if bad:
        raise SystemExit(f"el_spmv_host output fails the FP64 bound in {bad} rows")
    return {"value": round(world * nbytes / (ms * 1e-3) / 1e9, 2), "unit": "GB/s",
            "ms_per_step": round(ms, 4), "steps": steps,
            "h2d_bytes_per_step": int(world * h2d), "d2h_bytes_per_step": int(world * d2h),
            "api": "el_spmv_host (row blocks streamed, copies overlapped with the SpMV)",
            "block_nnz": args.e2e_block_nnz,
            "copy_then_spmv": {"value": round(world * nbytes / (ms_copy * 1e-3) / 1e9, 2),
                               "ms_per_step": round(ms_copy, 4)},
            "rows_outside_fp32_bound": bad}


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
    # the reference runs its CPU check single-threaded: time that too (bounded)
    one = []
    t_end = time.perf_counter() + max(2.0, budget_s / 5)
    while time.perf_counter() < t_end or len(one) < 3:
        t0 = time.perf_counter()
        oracle.spmv_f32(off, idx, vals, x)
        one.append(time.perf_counter() - t0)
        if len(one) >= 200:
            break
    med1 = statistics.median(one)
    return {"value": round(nbytes / med / 1e9, 3), "unit": "GB/s", "cores": threads,
            "single_thread": {"value": round(nbytes / med1 / 1e9, 3), "unit": "GB/s",
                              "ms_per_step": round(med1 * 1e3, 3), "repetitions": len(one)},
            "cpu_model": _cpu_model(),
            "kind": "port",
            "sample": (f"whole matrix (FP32 values), {len(times)} repetitions in "
                       f"~{budget_s:.0f} s, median; reference loop examples/spmv/"
                       f"helpers.hxx:106-112 restated in oracle/oracle.c, rows split "
                       f"over {threads} threads"),
            "ms_per_step": round(med * 1e3, 3)}


# Arm "CPU part" numbers of /proc/cpuinfo (implementer 0x41) by core name
_ARM_PARTS = {"0xd0c": "Neoverse-N1", "0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2",
              "0xd4f": "Neoverse-V2", "0xd83": "Neoverse-V3"}


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                low = line.lower()
                if low.startswith("model name") or low.startswith("cpu part"):
                    v = line.split(":", 1)[1].strip()
                    name = _ARM_PARTS.get(v.lower()) if low.startswith("cpu part") else None
                    return f"Arm {name} (part {v})" if name else v
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU SpMV loop on the host cores, on
    the same workload (FP32), one whole-matrix SpMV per step."""
    if rank != 0:
        return None
    import torch
    import oracle
    from edge_loops_gb300 import synth
    oracle.build()
    # the same matrix as the device arm: drawn by the same generator on the
    # GPU when there is one (torch's CPU and CUDA generators differ), then
    # moved to host memory; the timed loop runs on the host cores only
    gen_dev = "cuda" if torch.cuda.is_available() else "cpu"
    W = make_workload(args.workload, gen_dev, "f32")
    off = W["off"].cpu().numpy()
    idx = W["idx"].cpu().numpy()
    vals = W["vals"].cpu().numpy()
    x = W["x"].cpu().numpy()
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
                   "generated_on": gen_dev,
                   "rows": W["rows"], "cols": W["cols"], "nnz": int(len(idx)),
                   "value_dtype": "f32", "algorithmic_bytes_per_step": nbytes},
        "cpu_baseline": {
            "value": round(value, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": (f"whole matrix per step, {args.steps} steps after {args.warmup} "
                       f"warm-up; reference loop examples/spmv/helpers.hxx:106-112 restated "
                       f"in oracle/oracle.c, rows split over {threads} threads")},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_gpu_kernel": reference_gpu_kernel(W, nbytes, args),
    }


def reference_gpu_kernel(W, nbytes, args):
    """The reference's own merge_path_flat CUDA kernel on the same matrix
    (the cubin oracle/ref/build_ref.sh compiles from the reference's
    headers, launched as the reference's launcher launches it; y zeroed and
    the L2 flushed before every run, outside the CUDA events), reported
    beside the CPU loop.  None of this library's code runs here."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
        from oracle.ref import ref_gpu
        if not ref_gpu.available():
            return {"unavailable": "oracle/_ref/ref_kernels.cubin is not built here (it is "
                                   "compiled from the reference's sources where they exist)"}
        dev = torch.device("cuda", 0)
        off, idx, vals, x = (ref_gpu.pad(W[k].to(dev)) for k in ("off", "idx", "vals", "x"))
        rows, cols, nnz = W["rows"], W["cols"], int(W["idx"].numel())
        y = ref_gpu.pad(torch.zeros(rows, device=dev))
        R = ref_gpu.RefKernels()
        flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
        stream = torch.cuda.current_stream()
        steps = max(5, min(args.steps, 20))
        ts = []
        for k in range(steps + 3):
            flush.fill_(float(k))
            y.zero_()
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record(stream)
            R.launch("merge_path_flat", rows, cols, nnz, off, idx, vals, x, y, zero=False)
            e.record(stream)
            torch.cuda.synchronize()
            if k >= 3:
                ts.append(s.elapsed_time(e))
        ms = statistics.median(ts)
        return {"kernel": "loops::algorithms::spmv::__merge_path_flat<128, 5> (the reference's "
                          "CUDA kernel, compiled from its headers for sm_103a)",
                "us": round(ms * 1e3, 2), "GBps": round(nbytes / (ms * 1e-3) / 1e9, 2),
                "steps": steps}
    except Exception as e:  # the reference kernel is a side measurement
        return {"unavailable": f"{type(e).__name__}: {e}"[:200]}


# ------------------------------------------------------ SpMM and batched SpMV
def _time_device(step, steps, warmup, flush, stream):
    """Mean CUDA-event time (ms) of step() over `steps` runs, L2 flushed
    before each run outside the timed interval."""
    import torch
    for _ in range(warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / steps


def spmm_matrix(dev):
    """The SpMM workload's A: power-law 2^20 x 2^20 with ~8M nonzeros (Zipf
    2.0, cap 100000, seed 3)."""
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=8_000_000, exponent=2.0,
                                              cap=100_000, seed=3, device=dev)
    return api.CSR(off, idx, vals, off.numel() - 1, cols)


def measure_spmm(A, n, b_dtype, schedule, steps, warmup, flush, stream):
    """C = A B with B dense row-major cols x n (uniform [-1, 1], seed 33) of
    b_dtype: time per step (L2 flushed before each, outside the events),
    compulsory bytes (A + B + C once) and the gather model (A + a B row per
    nonzero + C), checked on 2048 sampled rows of C against FP64."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api
    dev = A.device
    g = torch.Generator(device=dev)
    g.manual_seed(33)
    B = torch.rand(A.cols, n, generator=g, device=dev) * 2 - 1
    B = B.to({"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[b_dtype])
    Cm = torch.empty(A.rows, n, device=dev)
    sb = B.element_size()
    compulsory = A.nnz * 8 + 4 * (A.rows + 1) + A.cols * n * sb + A.rows * n * 4
    gather = A.nnz * 8 + 4 * (A.rows + 1) + A.nnz * n * sb + A.rows * n * 4
    ws = api.Workspace()
    ms = _time_device(lambda: api.spmm(A, B, Cm, schedule=schedule, workspace=ws),
                      steps, warmup, flush, stream)
    if ws.errors():
        raise SystemExit("device error flags in SpMM")
    rng = np.random.default_rng(0)
    rows_s = np.sort(rng.choice(A.rows, 2048, replace=False))
    offh, idxh, valh = (t.cpu().numpy() for t in (A.offsets, A.indices, A.values))
    lens = offh[rows_s + 1] - offh[rows_s]
    sel = np.concatenate([np.arange(offh[r], offh[r + 1]) for r in rows_s])
    row_of = np.repeat(np.arange(len(rows_s)), lens)
    Bh = B.float().cpu().numpy()
    prod = valh[sel].astype(np.float64)[:, None] * Bh[idxh[sel]].astype(np.float64)
    C64 = np.zeros((len(rows_s), n))
    Ca = np.zeros((len(rows_s), n))
    np.add.at(C64, row_of, prod)
    np.add.at(Ca, row_of, np.abs(prod))
    got = Cm[torch.as_tensor(rows_s, device=dev)].cpu().numpy().astype(np.float64)
    so = np.concatenate([[0], np.cumsum(lens)])
    bad = int(np.sum(np.abs(got - C64) > fp32_bound(so, 1.0)[:, None] * Ca))
    if bad:
        raise SystemExit(f"SpMM output fails the FP64 bound in {bad} entries")
    return {"ms": ms, "compulsory_bytes": compulsory, "gather_model_bytes": gather,
            "GBps": compulsory / (ms * 1e-3) / 1e9,
            "GBps_gather_model": gather / (ms * 1e-3) / 1e9, "sampled_rows": 2048,
            "entries_outside_fp32_bound": bad}


def run_spmm(args):
    """SpMM C = A B (the SpMM workload): A power-law 2^20 x 2^20 with ~8M
    nonzeros (Zipf 2.0, cap 100000, seed 3), B dense row-major 2^20 x n."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    A = spmm_matrix(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    r = measure_spmm(A, args.n, args.b_dtype, args.schedule, args.steps, args.warmup, flush,
                     torch.cuda.current_stream())
    ms, ach = r["ms"], r["GBps"]
    peak, kind = measured_peaks()
    return {
        "metric": "SpMM achieved bandwidth (compulsory bytes / kernel time)",
        "value": round(ach, 2), "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": f"f32 values, {args.b_dtype} B, f32 accumulate",
        "data": "synthetic (seeded generator; SuiteSparse not available)",
        "config": {"workload": "SpMM power-law 2^20 x 2^20 ~8M nnz (Zipf 2.0, cap 1e5, seed 3),"
                               f" B 2^20 x {args.n} {args.b_dtype}",
                   "schedule": args.schedule, "n": args.n, "nnz": A.nnz,
                   "compulsory_bytes": r["compulsory_bytes"],
                   "gather_model_bytes": r["gather_model_bytes"],
                   "l2": "flushed before every step (512 MiB write, outside the timed kernel)"},
        "roofline": {"bound": "hbm", "achieved": round(ach, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_source": kind,
                     "achieved_gather_model": round(r["GBps_gather_model"], 2),
                     "traffic": traffic_for(f"spmm_powerlaw:{args.schedule}:{args.b_dtype}:{args.n}")},
        "gpu_launches": args.steps * ((args.n + 127) // 128),
        "check": {"sampled_rows": 2048, "entries_outside_fp32_bound": 0},
    }


def measure_batched(dev, steps, warmup, flush, stream, dtypes=("bf16",), row_scale=True,
                    per_matrix=True, count=4096):
    """The batched workload: 4096 square CSRs (rows log-uniform in [64,
    65536], log-normal row lengths with mean 8 and sigma 1, seed 4), one
    plan for FP32 values and one per 16-bit dtype in `dtypes` (values and
    per-row scales of every matrix quantized in one array each), each a
    CUDA-graph replay of one persistent launch per step; with per_matrix,
    also the plain FP32 merge-path kernel launched once per matrix (eagerly
    and captured in one CUDA graph), the comparison the batching target is
    defined against.  Every row of every matrix is checked against FP64:
    FP32 within the order-free bound, 16-bit within that bound of its stored
    values, and the max relative error against FP64 of the FP32 matrices is
    reported."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api, synth
    R, offc, idxc, valc, xc, rs, ns = synth.batched(count=count, seed=4, device=dev)
    items32, y32 = api.batched_items(R, offc, idxc, valc, xc, rs, ns)
    goff, gidx = synth.batch_as_one_csr(R, offc, idxc, rs, ns)
    o, i, v, xh = (t.cpu().numpy() for t in (goff, gidx, valc, xc))
    y64, yabs = fp64_spmv(o, i, v, xh)
    bound = fp32_bound(o, yabs)

    def total_bytes(items, vb, scaled):
        return sum(synth.algorithmic_bytes(A.rows, A.cols, A.nnz, vb, row_scale=scaled)
                   for A, _, _ in items)

    thr = lambda b, t: round(b / (t * 1e-3) / 1e9, 2)  # noqa: E731
    out = {"matrices": int(R.numel()), "rows_total": int(R.sum()), "nnz_total": int(idxc.numel())}
    b32 = total_bytes(items32, 4, False)
    plan32 = api.BatchPlan(items32)
    ms32 = _time_device(plan32.execute, steps, warmup, flush, stream)
    if plan32.errors():
        raise SystemExit("device error flags in the batched FP32 plan")
    y = y32.cpu().numpy().astype(np.float64)
    bad = int(np.sum(np.abs(y - y64) > bound))
    comp, _ = rel_errors(y, y64, yabs)
    if bad:
        raise SystemExit(f"batched FP32 plan outside the FP32 bound in {bad} rows")
    out["f32"] = {"ms": round(ms32, 4), "GBps": thr(b32, ms32), "algorithmic_bytes": b32,
                  "plan": plan32.info(), "rows_outside_fp32_bound": bad,
                  "max_rel_err_vs_fp64": comp}
    for dt in dtypes:
        tdt = torch.bfloat16 if dt == "bf16" else torch.float16
        Q = api.CSR(goff, gidx, valc, goff.numel() - 1, goff.numel() - 1).quantized(
            tdt, per_row_scale=row_scale)
        yq = torch.empty_like(y32)
        items = []
        for m, (r, r0, n0) in enumerate(zip(R.tolist(), rs.tolist(), ns.tolist())):
            nn = int(o[r0 + r] - o[r0])
            items.append((api.CSR(offc[r0 + m: r0 + m + r + 1], idxc[n0: n0 + nn],
                                  Q.values[n0: n0 + nn], r, r,
                                  row_scale=None if Q.row_scale is None else
                                  Q.row_scale[r0: r0 + r]),
                          xc[r0: r0 + r], yq[r0: r0 + r]))
        nb = total_bytes(items, 2, row_scale)
        plan = api.BatchPlan(items)
        ms = _time_device(plan.execute, steps, warmup, flush, stream)
        if plan.errors():
            raise SystemExit(f"device error flags in the batched {dt} plan")
        yy = yq.cpu().numpy().astype(np.float64)
        qv = Q.values.float().cpu().numpy()
        sc = None if Q.row_scale is None else Q.row_scale.cpu().numpy()
        yq64, yqabs = fp64_spmv(o, i, qv, xh, sc)
        badq = int(np.sum(np.abs(yy - yq64) > fp32_bound(o, yqabs)))
        compq, _ = rel_errors(yy, y64, yabs)
        if badq or compq > 1e-2:
            raise SystemExit(f"batched {dt} plan fails the check: {badq} rows, err {compq}")
        out[dt] = {"ms": round(ms, 4), "GBps": thr(nb, ms), "algorithmic_bytes": nb,
                   "plan": plan.info(), "rows_outside_fp32_bound_vs_stored": badq,
                   "max_rel_err_vs_fp64_of_fp32_matrices": compq,
                   "time_vs_fp32_plan": round(ms / ms32, 4)}
        plan.close()
        del plan, items, Q
    plan32.close()
    if per_matrix:
        ws = api.Workspace()

        def one_by_one():
            for A, x, yv in items32:
                api.spmv(A, x, yv, schedule="merge_path_flat", workspace=ws)

        one_by_one()  # sizes the workspace before capture
        ms_eager = _time_device(one_by_one, max(3, min(steps, 10)), 2, flush, stream)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            one_by_one()
        ms_graph = _time_device(graph.replay, steps, warmup, flush, stream)
        if ws.errors():
            raise SystemExit("device error flags in the per-matrix launches")
        out["plain_f32_per_matrix"] = {
            "graph_ms": round(ms_graph, 4), "graph_GBps": thr(b32, ms_graph),
            "eager_ms": round(ms_eager, 4), "launches": len(items32)}
        for dt in dtypes:
            out[dt]["speedup_vs_plain_f32_per_matrix_graph"] = round(ms_graph / out[dt]["ms"], 3)
            out[dt]["speedup_vs_plain_f32_per_matrix_eager"] = round(ms_eager / out[dt]["ms"], 3)
        out["f32"]["speedup_vs_plain_f32_per_matrix_graph"] = round(ms_graph / ms32, 3)
    return out


def run_batched(args):
    """Batched SpMV (the batched workload, measure_batched): the line's
    value is the plan of --value-dtype."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    dts = () if args.value_dtype == "f32" else (args.value_dtype,)
    r = measure_batched(dev, args.steps, args.warmup, flush, torch.cuda.current_stream(), dts,
                        row_scale=not args.no_row_scale, per_matrix=args.batch_count == 4096,
                        count=args.batch_count)
    me = r[args.value_dtype]
    peak, kind = measured_peaks()
    return {
        "metric": "batched SpMV achieved bandwidth (algorithmic bytes / graph time)",
        "value": me["GBps"], "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": me["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": f"{args.value_dtype} values, f32 accumulate",
        "data": "synthetic (seeded generator; SuiteSparse not available)",
        "config": {"workload": f"{args.batch_count} square CSRs, rows log-uniform [64, 65536], "
                               "log-normal nnz/row (mean 8, sigma 1), seed 4",
                   "rows_total": r["rows_total"], "nnz_total": r["nnz_total"],
                   "algorithmic_bytes_per_step": me["algorithmic_bytes"], "plan": me["plan"],
                   "l2": "flushed before every step (512 MiB write, outside the timed graph)"},
        "roofline": {"bound": "hbm", "achieved": me["GBps"], "peak": peak, "unit": "GB/s",
                     "frac": round(me["GBps"] / peak, 4), "peak_source": kind,
                     "traffic": traffic_for(f"spmv_batched:{args.value_dtype}" + (
                         "" if args.batch_count == 4096 else f":{args.batch_count}"))},
        "comparison": r,
        "gpu_launches": args.steps,
    }


def run_csr_build(args):
    """COO -> CSR on the GPU (el_csr_from_coo) for the power-law matrix's
    entries in random order: metric = COO bytes read + CSR bytes written per
    conversion time; checked entry by entry against the restated reference
    construction (a stable sort by (row, column), offsets by lower bound;
    container/csr.hxx:86-94) done with numpy."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api, synth

    def csr_from_coo_np(rows, ri, ci, vv):
        order = np.lexsort((ci, ri))  # stable
        offs = np.searchsorted(ri[order], np.arange(rows + 1), side="left").astype(np.int32)
        return offs, ci[order], vv[order]

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000, exponent=2.0,
                                              cap=100_000, seed=1, device=dev)
    rows, nnz = off.numel() - 1, idx.numel()
    row_of = torch.repeat_interleave(torch.arange(rows, device=dev, dtype=torch.int32),
                                     (off[1:] - off[:-1]).to(torch.int64))
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    perm = torch.randperm(nnz, generator=g, device=dev)
    ri, ci, vv = row_of[perm].contiguous(), idx[perm].contiguous(), vals[perm].contiguous()
    ws = api.Workspace()
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    out = {}
    def step():
        out["A"] = api.csr_from_coo(rows, cols, ri, ci, vv, device=dev, workspace=ws)
    ms = _time_device(step, args.steps, args.warmup, flush, torch.cuda.current_stream())
    A = out["A"]
    o2, i2, v2 = csr_from_coo_np(rows, ri.cpu().numpy(), ci.cpu().numpy(), vv.cpu().numpy())
    ok = (np.array_equal(A.offsets.cpu().numpy(), o2) and np.array_equal(A.indices.cpu().numpy(), i2)
          and np.array_equal(A.values.cpu().numpy(), v2))
    if not ok:
        raise SystemExit("el_csr_from_coo differs from the numpy construction")
    nbytes = nnz * 12 + nnz * 8 + (rows + 1) * 4
    import time as _t
    t0 = _t.perf_counter()
    csr_from_coo_np(rows, ri.cpu().numpy(), ci.cpu().numpy(), vv.cpu().numpy())
    cpu_s = _t.perf_counter() - t0
    return {
        "metric": "COO->CSR construction bandwidth (COO read + CSR written / time)",
        "value": round(nbytes / (ms * 1e-3) / 1e9, 2), "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32 keys",
        "data": "synthetic (the power-law SpMV matrix's entries in random order)",
        "config": {"workload": "COO of the 2^20 x 2^20 power-law matrix (seed 1), shuffled",
                   "nnz": nnz, "rows": rows, "bytes_per_step": nbytes,
                   "includes": "range check (one host sync), radix sort, gather, offsets"},
        "check": {"equal_to_numpy_construction": ok},
        "cpu_baseline": {"value": round(nbytes / cpu_s / 1e9, 3), "unit": "GB/s", "cores": 1,
                         "kind": "port", "sample": "numpy stable lexsort + searchsorted, once"},
        "gpu_launches": 3 * args.steps,  # this library's kernels; the radix sort is CUB's
    }


def run_edge(args):
    """y = A x over an edge partition (el_spmv_edge) of the power-law
    matrix's COO: --edge pos:P:T (atoms of P nonzeros, tiles of T atoms) or
    coord:M0:K0:M1:K1.  Bytes per step: quark, row, column and value per
    nonzero (16 B), x and y once.  Checked against FP64 within the FP32
    order-free bound; the partition build is timed once beside it."""
    import numpy as np
    import torch
    from edge_loops_gb300 import api, edge, synth
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000, exponent=2.0,
                                              cap=100_000, seed=1, device=dev)
    A = api.CSR(off, idx, vals, off.numel() - 1, cols)
    coo = edge.COO.from_csr(A)
    spec = args.edge.split(":")
    sizes = [int(v) for v in spec[1:]]
    part = edge.Partitioner(coo, sort=False)  # already row-sorted
    ws = api.Workspace()
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)

    def build():
        if spec[0] == "coord":
            part.partition_atoms_coordinate_space(*sizes[:2])
            part.partition_tiles_coordinate_space(*sizes[2:])
        else:
            part.partition_atoms_position_space(sizes[0])
            part.partition_tiles_position_space(sizes[1])
    build_ms = _time_device(build, 3, 3, flush, torch.cuda.current_stream())
    y = torch.empty(A.rows, device=dev)
    ms = _time_device(lambda: edge.spmv_edge(coo, part, x, y, workspace=ws), args.steps,
                      args.warmup, flush, torch.cuda.current_stream())
    flags = api.workspace_errors(ws)
    o, i, v, xh = (t.cpu().numpy() for t in (off, idx, vals, x))
    y64, yabs = fp64_spmv(o, i, v, xh)
    bound = fp32_bound(o, yabs, extra=8)
    ok = flags == 0 and bool(np.all(np.abs(y.cpu().numpy().astype(np.float64) - y64) <= bound))
    if not ok:
        raise SystemExit("el_spmv_edge outside the FP32 bound of FP64")
    comp, _ = rel_errors(y.cpu().numpy(), y64, yabs)
    rows, nnz = A.rows, A.nnz
    nbytes = nnz * 16 + 4 * cols + 4 * rows
    peak, src = measured_peaks()
    import time as _t
    import oracle  # the CPU baseline: the reference's loop, restated
    t0 = _t.perf_counter()
    oracle.spmv_f32(o, i, v, xh)
    cpu_s = _t.perf_counter() - t0
    return {
        "metric": "edge-partitioned SpMV bandwidth (COO + quarks read, x, y / time)",
        "value": round(nbytes / (ms * 1e-3) / 1e9, 2), "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the 2^20 x 2^20 power-law matrix, seed 1, as a row-sorted COO)",
        "config": {"workload": "edge SpMV, power-law 2^20 x 2^20, %d nnz" % nnz,
                   "partition": args.edge, "tiles": part.get_num_tiles(),
                   "partition_build_ms": round(build_ms, 4), "bytes_per_step": nbytes,
                   "l2": "flushed between steps"},
        "check": {"within_fp32_bound_of_fp64": ok, "max_rel_err": comp},
        "roofline": {"bound": "hbm", "achieved": round(nbytes / (ms * 1e-3) / 1e9, 2),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(nbytes / (ms * 1e-3) / 1e9 / peak, 4), "peak_source": src,
                     "traffic": traffic_for(f"spmv_edge:{args.edge}")},
        "cpu_baseline": {"value": round(nbytes / cpu_s / 1e9, 3), "unit": "GB/s", "cores": 1,
                         "kind": "port", "sample": "the reference's CPU SpMV loop on the CSR, once"},
        "gpu_launches": args.steps,
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
    ap.add_argument("--row-weight", type=int, default=0,
                    help="merge_path: merge items per row end in the warp split (0 = default)")
    ap.add_argument("--nz-per-lane", type=int, default=0, choices=[0, 8, 16],
                    help="merge_path: nonzeros per lane of the tile walk (0 = the library's choice)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-row-scale", action="store_true",
                    help="16-bit values without per-row scales")
    ap.add_argument("--n", type=int, default=128, help="SpMM: columns of B")
    ap.add_argument("--batch-count", type=int, default=4096,
                    help="spmv_batched: matrices in the batch (the workload has 4096; fewer "
                         "for profiler captures)")
    ap.add_argument("--b-dtype", default="f32", choices=["f32", "bf16", "f16"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false",
                    help="default workload: skip the stencil and batched configurations")
    ap.add_argument("--e2e-block-nnz", type=int, default=0,
                    help="e2e: nonzeros per streamed row block (0: the library's default)")
    ap.add_argument("--edge", default="pos:256:1",
                    help="spmv_edge partition: pos:P:T or coord:M0:K0:M1:K1")
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
    if world > 1:
        torch.distributed.init_process_group(
            "nccl", device_id=torch.device("cuda", _env_int("LOCAL_RANK", 0)))
    try:
        if args.workload in ("spmm_powerlaw", "spmv_batched", "csr_build", "spmv_edge"):
            line = {"spmm_powerlaw": run_spmm, "spmv_batched": run_batched,
                    "csr_build": run_csr_build, "spmv_edge": run_edge}[args.workload](args)
        else:
            line = run_ours(args, rank, world)
        if rank == 0:
            print(json.dumps(line))
    finally:
        if world > 1:
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
