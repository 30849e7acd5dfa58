"""Refits the schedule-selection cost model of csrc/select.cu on this GPU.

    python -m edge_loops_gb300.tune_select [--out sweep.csv] [--quick]

Times merge_path and thread_mapped with 1, 4 and 32 lanes per row, and
with one lane per row and the rows staged through shared memory (variant 1,
on shapes whose rows hold at most 27 nonzeros), plus group_mapped and
work_oriented for reference, on synthetic shapes -- uniform, log-normal
(sigma 0.5, 1.0, 1.5) and Zipf(2) row lengths, 64 to 4M rows, 1 to 256
nonzeros per row, and 27-point stencils on 16^3 to 128^3 grids, L2 flushed
before every run -- then fits
    merge_path          a + e (nnz + rows)/1e6
    thread_mapped, T    a + c max_row + d rows/1e3 + e nnz/1e6
    staged              the same form, on the shapes it applies to (rows of
                        at most 27 nonzeros, row coherence at least 0.5)
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
STAGED = ("tms", "thread_mapped", {"threads_per_row": 1, "variant": 1})
STAGED_MAX_ROW = 27  # every 32-row chunk fits the staging buffer
STAGED_COHERENCE = 0.5  # consecutive rows share their column pattern


def staged_applies(f):
    return f["max"] <= STAGED_MAX_ROW and f["coh"] >= STAGED_COHERENCE
OTHERS = [("group", "group_mapped", {}), ("work", "work_oriented", {})]


def shapes(quick=False):
    out = []
    step = 4 if quick else 2
    for lg in range(6, 23, step):
        for per in (1, 4, 16, 27, 64, 256):
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
    for n in ((16, 64, 128) if quick else (16, 32, 64, 100, 128)):
        out.append(("stencil", n ** 3, 27))
    return out


def make(fam, rows, per, g, dev):
    if fam == "stencil":
        n = round(rows ** (1 / 3))
        return synth.stencil27(n=n, seed=2, device=dev)
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
    names = [c[0] for c in CANDIDATES + [STAGED] + OTHERS]
    w = csv.writer(open(out_path, "w", newline="")) if out_path else None
    if w:
        w.writerow(["family", "rows", "nnz", "max", "coherence"] + names)
    for fam, rows, per in shapes(quick):
        off, idx, vals, x, cols = make(fam, rows, per, g, dev)
        A = api.CSR(off, idx, vals, rows, cols)
        st = api.row_stats(A, workspace=ws)
        y = torch.empty(rows, device=dev)
        reps = 7 if A.nnz >= (1 << 24) else 15
        t = {}
        staged = [STAGED] if st["max_row_nnz"] <= STAGED_MAX_ROW else []
        for name, sched, o in CANDIDATES + staged + OTHERS:
            t[name] = time_us(lambda: api.spmv(A, x, y, schedule=sched, workspace=ws, **o),
                              reps, flush)
        feat = {"rows": rows, "nnz": A.nnz, "max": st["max_row_nnz"],
                "coh": st["coherence"]}
        data.append((fam, feat, t))
        if w:
            w.writerow([fam, rows, A.nnz, st["max_row_nnz"], round(st["coherence"], 4)] +
                       [round(t[n], 2) if n in t else "" for n in names])
        print(fam, rows, A.nnz, st["max_row_nnz"], round(st["coherence"], 3),
              {k: round(v, 1) for k, v in t.items()}, flush=True)
        del A, off, idx, vals, x, y
        torch.cuda.empty_cache()
    return data


def fit(data):
    from scipy.optimize import nnls

    def solve(key, cols):
        rows = [(f, t) for _, f, t in data
                if key in t and (key != "tms" or staged_applies(f))]
        A = np.array([[1.0] + [c(f) for c in cols] for f, _ in rows])
        b = np.array([t[key] for _, t in rows])
        x, _ = nnls(A / b[:, None], np.ones_like(b))
        return x
    model = {"merge_path": solve("merge_path", [lambda f: (f["nnz"] + f["rows"]) / 1e6])}
    for key in ("tm1", "tm4", "tm32", "tms"):
        if any(key in t and (key != "tms" or staged_applies(f)) for _, f, t in data):
            model[key] = solve(key, [lambda f: f["max"], lambda f: f["rows"] / 1e3,
                                     lambda f: f["nnz"] / 1e6])
    return model


def predict(model, f):
    a, e = model["merge_path"]
    est = {"merge_path": a + e * (f["nnz"] + f["rows"]) / 1e6}
    for key in ("tm1", "tm4", "tm32", "tms"):
        if key not in model or (key == "tms" and not staged_applies(f)):
            continue
        a, c, d, e = model[key]
        est[key] = a + c * f["max"] + d * f["rows"] / 1e3 + e * f["nnz"] / 1e6
    return min(est, key=est.get)


def builtin_choice(f):
    """The library's own choice (el_select_schedule_stats) for features f."""
    st = L.ElRowStats()
    st.max_row_nnz = f["max"]
    st.coherence = f["coh"]
    s, o = C.c_int32(), api.make_opts()
    L.check(L.lib().el_select_schedule_stats(f["rows"], f["rows"], f["nnz"], C.byref(st),
                                             C.byref(s), C.byref(o), None),
            "el_select_schedule_stats")
    if s.value == L.EL_SCHED_MERGE_PATH_FLAT:
        return "merge_path"
    return "tms" if o.variant == 1 else "tm%d" % o.threads_per_row


def quality(data, choose):
    others = {c[0] for c in OTHERS}
    loss = np.array([t[choose(f)] / min(v for k, v in t.items() if k not in others)
                     for _, f, t in data])
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
