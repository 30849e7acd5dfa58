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
    ap.add_argument("--spmm", type=int, default=0,
                    help="n > 0: SpMM C = A B, B 2^20 x n, on the ~8M-nnz power-law matrix")
    args = ap.parse_args()
    if args.spmm:
        return spmm(args)
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
    # the schedule el_spmv_select picks (the staged thread_mapped kernel on
    # short coherent rows such as the stencil's)
    sel, opts = api.select_schedule(A, workspace=ws)
    ms = timed(lambda: api.spmv(A, x, y, schedule=sel, workspace=ws, **opts), args.reps)
    report("edge_loops_gb300", sel + "".join(f" {k}={v}" for k, v in opts.items()), ms,
           "the schedule el_spmv_select picks")


def spmm(args):
    """The reference's SpMM (thread_mapped) beside this library's three SpMM
    schedules on the bench's SpMM matrix (power-law 2^20 x 2^20, ~8M nnz,
    seed 3; B uniform [-1, 1], seed 33); 2048 sampled rows of C checked."""
    import numpy as np
    import torch

    import oracle
    from edge_loops_gb300 import api, synth
    from oracle.ref import ref_gpu
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=8_000_000, exponent=2.0,
                                              cap=100_000, seed=3, device=dev)
    rows, nnz, n = off.numel() - 1, idx.numel(), args.spmm
    A = api.CSR(off, idx, vals, rows, cols)
    g = torch.Generator(device=dev)
    g.manual_seed(33)
    B = torch.rand(cols, n, generator=g, device=dev) * 2 - 1
    Cm = torch.empty(rows, n, device=dev)
    compulsory = nnz * 8 + 4 * (rows + 1) + cols * n * 4 + rows * n * 4
    R = ref_gpu.RefKernels()
    P = [ref_gpu.pad(t) for t in (off, idx, vals)]
    ws = api.Workspace()
    flush = torch.empty((512 << 20) // 4, device=dev)
    rng = np.random.default_rng(0)
    rows_s = np.sort(rng.choice(rows, 2048, replace=False))
    offh, idxh, valh = off.cpu().numpy(), idx.cpu().numpy(), vals.cpu().numpy()
    lens = offh[rows_s + 1] - offh[rows_s]
    so = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    sel = np.concatenate([np.arange(offh[r], offh[r + 1]) for r in rows_s])
    C64, Ca = oracle.spmm_f64(so, idxh[sel], valh[sel], B.cpu().numpy())
    nn = (np.diff(so.astype(np.int64)) + 2)[:, None]
    bound = (nn * 2.0 ** -24 / (1 - nn * 2.0 ** -24)) * Ca

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        ts = []
        for k in range(reps):
            flush.fill_(float(k))
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e))
        ts.sort()
        return ts[len(ts) // 2]

    def report(impl, sched, ms):
        got = Cm[torch.as_tensor(rows_s, device=dev)].cpu().numpy().astype(np.float64)
        bad = int(np.sum(np.abs(got - C64) > bound))
        print(json.dumps({"impl": impl, "schedule": "spmm " + sched, "workload": "spmm_powerlaw",
                          "n": n, "rows": rows, "nnz": nnz, "ms": round(ms, 5),
                          "GBps": round(compulsory / (ms * 1e-3) / 1e9, 1),
                          "sampled_entries_outside_fp32_bound": bad}), flush=True)

    ms = timed(lambda: R.spmm(rows, cols, nnz, *P, B, Cm), 3)
    report("reference", "thread_mapped", ms)
    for sched, reps in (("merge_path_flat", args.reps), ("group_mapped", 3), ("thread_mapped", 3)):
        ms = timed(lambda: api.spmm(A, B, Cm, schedule=sched, workspace=ws), reps)
        report("edge_loops_gb300", sched, ms)


if __name__ == "__main__":
    main()
