"""Refits the schedule-selection cost model of csrc/select.cu on this GPU.

    python -m edge_loops_gb300.tune_select [--out sweep.csv] [--quick]

Times merge_path and thread_mapped with 1, 4 and 32 lanes per row (plus
group_mapped and work_oriented, for reference) on synthetic shapes --
uniform, log-normal (sigma 0.5, 1.0, 1.5) and Zipf(2) row lengths, 64 to 4M
rows, 1 to 256 nonzeros per row, L2 flushed before every run -- then fits
    merge_path          a + e (nnz + rows)/1e6
    thread_mapped, T    a + c max_row + d rows/1e3 + e nnz/1e6
by non-negative least squares on relative error, and prints the constants
(to paste into select.cu) with the selection quality of: always merge_path,
the library's built-in model (el_select_schedule) and the refit, as the
time of the chosen schedule over the best one per shape (geometric mean,
worst, shapes more than 1.2x off).
"""
import argparse
import csv
import ctypes as C
import math
import sys

import numpy as np
import torch

from . import _lib as L
from . import api, synth

CANDIDATES = [("merge_path", "merge_path_flat", {}),
              ("tm1", "thread_mapped", {"threads_per_row": 1}),
              ("tm4", "thread_mapped", {"threads_per_row": 4}),
              ("tm32", "thread_mapped", {"threads_per_row": 32})]
OTHERS = [("group", "group_mapped", {}), ("work", "work_oriented", {})]


def shapes(quick=False):
    out = []
    step = 4 if quick else 2
    for lg in range(6, 23, step):
        for per in (1, 4, 16, 64, 256):
            if (1 << lg) * per <= (1 << 27) and per <= (1 << lg):
                out.append(("uniform", 1 << lg, per))
        for mean in (4, 16):
            if (1 << lg) * mean <= (1 << 27):
                out.append(("powerlaw", 1 << lg, mean))
    for lg in range(10, 23, step):
        for mean in (4, 16, 64):
            for sigma in (0.5, 1.0, 1.5):
                if (1 << lg) * mean <= (1 << 27):
                    out.append(("lognormal%.1f" % sigma, 1 << lg, mean))
    return out


def make(fam, rows, per, g, dev):
    if fam == "powerlaw":
        return synth.power_law(rows=rows, cols=rows, target_nnz=rows * per, exponent=2.0,
                               cap=min(rows, 100_000), seed=rows + per, device=dev)
    if fam == "uniform":
        lens = torch.full((rows,), per, device=dev, dtype=torch.int64)
    else:
        sigma = float(fam[len("lognormal"):])
        mu = math.log(per) - sigma * sigma / 2
        lens = torch.exp(torch.randn(rows, generator=g, device=dev) * sigma + mu)
        lens = lens.round().clamp(1, rows).to(torch.int64)
    off = torch.zeros(rows + 1, device=dev, dtype=torch.int64)
    off[1:] = torch.cumsum(lens, 0)
    nnz = int(off[-1])
    row_of = torch.repeat_interleave(torch.arange(rows, device=dev), lens)
    cols = torch.randint(0, rows, (nnz,), generator=g, device=dev)
    idx = ((row_of * rows + cols).sort().values % rows).to(torch.int32)
    vals = torch.rand(nnz, generator=g, device=dev) * 2 - 1
    x = torch.rand(rows, generator=g, device=dev) * 2 - 1
    return off.to(torch.int32), idx, vals, x, rows


def time_us(fn, reps, flush):
    for _ in range(3):
        flush.fill_(1.0)
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
    return ts[len(ts) // 2] * 1e3


def sweep(quick, out_path):
    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty((512 << 20) // 4, device=dev)
    ws = api.Workspace()
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    data = []
    names = [c[0] for c in CANDIDATES + OTHERS]
    w = csv.writer(open(out_path, "w", newline="")) if out_path else None
    if w:
        w.writerow(["family", "rows", "nnz", "max"] + names)
    for fam, rows, per in shapes(quick):
        off, idx, vals, x, cols = make(fam, rows, per, g, dev)
        A = api.CSR(off, idx, vals, rows, cols)
        st = api.row_stats(A, workspace=ws)
        y = torch.empty(rows, device=dev)
        reps = 7 if A.nnz >= (1 << 24) else 15
        t = {}
        for name, sched, o in CANDIDATES + OTHERS:
            t[name] = time_us(lambda: api.spmv(A, x, y, schedule=sched, workspace=ws, **o),
                              reps, flush)
        feat = {"rows": rows, "nnz": A.nnz, "max": st["max_row_nnz"]}
        data.append((fam, feat, t))
        if w:
            w.writerow([fam, rows, A.nnz, st["max_row_nnz"]] + [round(t[n], 2) for n in names])
        print(fam, rows, A.nnz, st["max_row_nnz"],
              {k: round(v, 1) for k, v in t.items()}, flush=True)
        del A, off, idx, vals, x, y
        torch.cuda.empty_cache()
    return data


def fit(data):
    from scipy.optimize import nnls

    def solve(key, cols):
        A = np.array([[1.0] + [c(f) for c in cols] for _, f, _ in data])
        b = np.array([t[key] for _, _, t in data])
        x, _ = nnls(A / b[:, None], np.ones_like(b))
        return x
    model = {"merge_path": solve("merge_path", [lambda f: (f["nnz"] + f["rows"]) / 1e6])}
    for tpr in (1, 4, 32):
        model["tm%d" % tpr] = solve("tm%d" % tpr, [lambda f: f["max"], lambda f: f["rows"] / 1e3,
                                                   lambda f: f["nnz"] / 1e6])
    return model


def predict(model, f):
    a, e = model["merge_path"]
    est = {"merge_path": a + e * (f["nnz"] + f["rows"]) / 1e6}
    for tpr in (1, 4, 32):
        a, c, d, e = model["tm%d" % tpr]
        est["tm%d" % tpr] = a + c * f["max"] + d * f["rows"] / 1e3 + e * f["nnz"] / 1e6
    return min(est, key=est.get)


def builtin_choice(f):
    s, t = C.c_int32(), C.c_int32()
    L.check(L.lib().el_select_schedule(f["rows"], f["rows"], f["nnz"], f["max"], C.byref(s),
                                       C.byref(t), None), "el_select_schedule")
    return "merge_path" if s.value == L.EL_SCHED_MERGE_PATH_FLAT else "tm%d" % t.value


def quality(data, choose):
    loss = np.array([t[choose(f)] / min(t[c[0]] for c in CANDIDATES) for _, f, t in data])
    return {"geomean": round(float(np.exp(np.log(loss).mean())), 4),
            "worst": round(float(loss.max()), 3), "over_1.2x": int((loss > 1.2).sum()),
            "shapes": len(loss)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="CSV of the measured times")
    ap.add_argument("--quick", action="store_true", help="every other size")
    args = ap.parse_args(argv)
    data = sweep(args.quick, args.out)
    model = fit(data)
    print("fitted constants (a, c, d, e):")
    for k, v in model.items():
        print("  %-10s" % k, ", ".join("%.4g" % x for x in v))
    print("always merge_path:", quality(data, lambda f: "merge_path"))
    print("built-in model:   ", quality(data, builtin_choice))
    print("refit model:      ", quality(data, lambda f: predict(model, f)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
