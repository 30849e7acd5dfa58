"""Times the reference's own SpMV kernels (oracle/ref/ref_gpu.py) beside this
library's schedules on the bench matrices, on one GPU (TEST INFRASTRUCTURE:
a measurement run by hand, not part of the library or of bench.py).

    python oracle/ref/time_ref_gpu.py [--workload spmv_powerlaw|spmv_stencil] [--reps N]

Every kernel runs on the same CSR, x and y; the L2 cache is flushed (512 MiB
write) before every run, outside the CUDA events that time it; the figure
is the median.  Each result is checked against the FP64 oracle with the
FP32 order-free bound (rows outside it are counted, not fatal: the
reference's work_oriented kernel has a race at block boundaries).
Prints one JSON line per kernel.
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def main():
    import numpy as np
    import torch

    import oracle
    from edge_loops_gb300 import api, synth
    from oracle.ref import ref_gpu

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="spmv_powerlaw")
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    if args.workload == "spmv_stencil":
        off, idx, vals, x, cols = synth.stencil27(n=160, seed=2, device=dev)
    else:
        off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000,
                                                  exponent=2.0, cap=100_000, seed=1, device=dev)
    rows, nnz = off.numel() - 1, idx.numel()
    A = api.CSR(off, idx, vals, rows, cols)
    nbytes = synth.algorithmic_bytes(rows, cols, nnz, 4)
    o, i, v, xh = (t.cpu().numpy() for t in (off, idx, vals, x))
    y64, yabs = oracle.spmv_f64(o, i, v, xh)
    lens = np.diff(o).astype(np.float64)
    bound = (lens + 2) * 2.0 ** -24 / (1 - (lens + 2) * 2.0 ** -24) * yabs
    R = ref_gpu.RefKernels()
    P = [ref_gpu.pad(t) for t in (off, idx, vals, x)]
    ws = api.Workspace()
    flush = torch.empty((512 << 20) // 4, device=dev)
    y = ref_gpu.pad(torch.empty(rows, device=dev))

    def timed(fn, reps, pre=None):
        for _ in range(2):
            flush.fill_(1.0)
            if pre:
                pre()
            fn()
        torch.cuda.synchronize()
        ts = []
        for k in range(reps):
            flush.fill_(float(k))
            if pre:
                pre()
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e))
        ts.sort()
        return ts[len(ts) // 2]

    def report(impl, sched, ms, note=""):
        got = y.cpu().numpy().astype(np.float64)
        bad = int(np.sum(np.abs(got - y64) > bound))
        print(json.dumps({"impl": impl, "schedule": sched, "workload": args.workload,
                          "rows": rows, "nnz": nnz, "ms": round(ms, 5),
                          "GBps": round(nbytes / (ms * 1e-3) / 1e9, 1),
                          "rows_outside_fp32_bound": bad, "note": note}), flush=True)

    for sched in ref_gpu.SCHEDULES:
        reps = 3 if sched in ("thread_mapped", "original") else args.reps
        # y is zeroed before each run, outside the timed interval (the
        # reference's callers hand it a zeroed y)
        ms = timed(lambda: R.launch(sched, rows, cols, nnz, *P, y, zero=False),
                   reps, pre=lambda: y.zero_())
        report("reference", sched, ms, "kernel only; y zeroed before the timed interval")
    for sched in ("merge_path_flat", "thread_mapped", "group_mapped", "work_oriented"):
        reps = 3 if sched == "thread_mapped" else args.reps
        ms = timed(lambda: api.spmv(A, x, y, schedule=sched, workspace=ws), reps)
        report("edge_loops_gb300", sched, ms)


if __name__ == "__main__":
    main()
