"""Autotuner for the batched SpMV plan: measures, per (rows, mean row length,
row-length variation) bucket, which kernel mode (1..32 lanes per row or the
nonzero-tiled walk) and work-item size run a group of matrices of that
bucket fastest, and writes the table el_batch_plan_create reads (JSON,
loaded by api.load_tuning_table).

    python -m edge_loops_gb300.tune_batch [--dtype bf16] [--out PATH]

Each probed bucket gets a group of synthetic matrices (fixed rows, log-normal
row lengths with the bucket's mean and spread, ~16M nonzeros in total) and a
second group twice as large; every (kernel mode, log2 rows + nonzeros per
work item) pair is timed on both as a CUDA-graph replay with L2 flushed
before each replay, and the choice is made on the difference: the marginal
cost of the bucket's matrices.  (A group timed alone ends with a tail of
about one work item per warp, which rewards small items; inside a whole
batch each warp runs dozens of items and the tail is shared, so the
marginal cost is what a bucket adds to a batch.)  A bucket gets an entry
only where a choice beats the plan's built-in rule by MARGIN.  The
bucket a group lands in is computed from its actual row statistics with the
same rule the plan uses; row buckets that were not probed take the entry of
the nearest probed row bucket with the same length and variation buckets.
"""
import argparse
import json
import math
import os
import time

import numpy as np
import torch

from . import _lib as L
from . import api, synth

TPRS = (1, 2, 4, 8, 16, 32, L.EL_BATCH_NZ_WALK)  # lanes per row, or the nonzero-tiled walk
CHUNKS = (10, 11, 12, 13, 14)  # log2(rows + nonzeros) per work item
ROW_BUCKETS = (6, 8, 10, 12, 14, 16)
LEN_BUCKETS = (1, 2, 3, 4, 5, 6, 7, 8)
SIGMAS = (0.1, 0.5, 1.0, 1.5)  # aims at variation buckets 0..3
BUILTIN = (L.EL_BATCH_NZ_WALK, 12)  # the plan's rule where the table has no entry
MARGIN = 0.05


def row_bucket(rows):
    b = 0
    while b < L.EL_BATCH_ROW_BUCKETS - 1 and (2 << b) <= rows:
        b += 1
    return b


def len_bucket(avg):
    if avg < 1.0:
        return 0
    b = 1
    while b < L.EL_BATCH_LEN_BUCKETS - 1 and avg >= float(1 << b):
        b += 1
    return b


def cv_bucket(cv):
    return 0 if cv < 0.25 else 1 if cv < 0.75 else 2 if cv < 1.5 else 3


def group_key(off_cat, rows, row_start):
    """Most common (rb, lb, cb) over the group's matrices, computed as the
    plan computes it (mean nnz/row, sqrt(E[len^2] - mean^2) / mean)."""
    off = off_cat.cpu().numpy().astype(np.int64)
    keys = {}
    for m, (r, rs) in enumerate(zip(rows.tolist(), row_start.tolist())):
        o = off[rs + m: rs + m + r + 1]
        lens = np.diff(o).astype(np.float64)
        avg = lens.sum() / r
        var = max(0.0, float((lens * lens).sum()) / r - avg * avg)
        cv = math.sqrt(var) / avg if avg > 0 else 0.0
        k = (row_bucket(r), len_bucket(avg), cv_bucket(cv))
        keys[k] = keys.get(k, 0) + 1
    return max(keys.items(), key=lambda kv: kv[1])[0]


def time_plan(plan, flush, reps=5):
    s = torch.cuda.current_stream()
    plan.execute()
    torch.cuda.synchronize()
    t = []
    for _ in range(reps):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(s)
        plan.execute()
        b.record(s)
        b.synchronize()
        t.append(a.elapsed_time(b))
    return float(np.median(t))


def tune(dtype="bf16", target_nnz=16_000_000, seed=100, verbose=True):
    dev = torch.device("cuda", torch.cuda.current_device())
    tdt = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[dtype]
    flush = torch.empty((512 << 20) // 4, device=dev)
    best = {}
    t0 = time.time()
    for rb in ROW_BUCKETS:
        r = int(round(1.41 * (1 << rb)))
        for lb in LEN_BUCKETS:
            mean = 1.41 * (1 << (lb - 1))
            if mean > r:
                continue
            for sg in SIGMAS:
                count = int(min(8192, max(16, target_nnz // max(1, int(r * mean)))))
                rows, off, idx, vals, x, rs, ns = synth.batched(
                    count=2 * count, rows_lo=r, rows_hi=r, mean_per_row=mean, sigma=sg,
                    seed=seed, device=dev)
                seed += 1
                key = group_key(off, rows, rs)
                items, y = api.batched_items(rows, off, idx, vals, x, rs, ns)
                if tdt != torch.float32:
                    items = [(A.quantized(tdt, per_row_scale=True), xx, yy)
                             for A, xx, yy in items]
                res = []
                for tpr in TPRS:
                    for cl in CHUNKS:
                        t = []
                        for part in (items[:count], items):
                            plan = api.BatchPlan(part, table=None, force_threads_per_row=tpr,
                                                 force_chunk_log2=cl)
                            if plan.info()["heavy_matrices"] == len(part):
                                plan.close()
                                break
                            t.append(time_plan(plan, flush))
                            plan.close()
                        if len(t) == 2:
                            res.append((t[1] - t[0], tpr, cl))
                if not res:
                    continue
                ms, tpr, cl = min(res)
                fastest = (tpr, cl, ms)
                # the built-in rule unless a choice beats it clearly: a bucket's
                # optimum measured alone moves by a few per cent inside a mixed
                # batch, so small gains are noise
                base = [t for t, tp, c in res if tp == BUILTIN[0] and c == BUILTIN[1]]
                if base and ms > (1.0 - MARGIN) * base[0]:
                    tpr, cl = BUILTIN
                prev = best.get(key)
                # two groups landing in one bucket: keep the choice of the
                # group nearer the bucket's centre (the first one probed)
                if prev is None:
                    best[key] = (tpr, cl, ms, fastest, base[0] if base else None)
                if verbose:
                    print(f"rows {r:6d} mean {mean:7.1f} sigma {sg:.1f} -> bucket {key}: "
                          f"tpr {tpr} chunk 2^{cl} marginal {ms:.4f} ms for {count} matrices "
                          f"(built-in {base[0] if base else float('nan'):.4f}) "
                          f"({time.time() - t0:.0f} s)", flush=True)
                del items, y
    # fill unprobed row buckets from the nearest probed one
    entries = {}
    probed_rb = sorted({k[0] for k in best})
    for (rb, lb, cb), (tpr, cl, *_rest) in best.items():
        if (tpr, cl) != BUILTIN:
            entries[f"{rb},{lb},{cb}"] = [tpr, cl]
    for rb in range(L.EL_BATCH_ROW_BUCKETS):
        if rb in probed_rb:
            continue
        near = min(probed_rb, key=lambda p: (abs(p - rb), p))
        for (prb, lb, cb), (tpr, cl, *_rest) in best.items():
            if prb == near and (tpr, cl) != BUILTIN:
                entries.setdefault(f"{rb},{lb},{cb}", [tpr, cl])
    # per probed bucket: the choice kept, the fastest (threads per row, chunk,
    # marginal ms) and the built-in rule's marginal ms on the same matrices
    return {"dtype": dtype, "device": torch.cuda.get_device_name(dev),
            "threads_per_row": list(TPRS), "chunk_log2": list(CHUNKS),
            "probed": {f"{k[0]},{k[1]},{k[2]}": {
                "chosen": [v[0], v[1]],
                "fastest": [v[3][0], v[3][1], round(v[3][2], 5)],
                "builtin_ms": None if v[4] is None else round(v[4], 5)}
                for k, v in sorted(best.items())},
            "entries": dict(sorted(entries.items(), key=lambda kv: tuple(
                int(t) for t in kv[0].split(","))))}


def dumps(table):
    """JSON text with one table entry per line."""
    out = ["{"]
    keys = list(table)
    for i, k in enumerate(keys):
        v = table[k]
        sep = "," if i + 1 < len(keys) else ""
        if isinstance(v, dict):
            out.append(f" {json.dumps(k)}: {{")
            items = list(v.items())
            for j, (kk, vv) in enumerate(items):
                out.append(f"  {json.dumps(kk)}: {json.dumps(vv)}" + ("," if j + 1 < len(items) else ""))
            out.append(" }" + sep)
        else:
            out.append(f" {json.dumps(k)}: {json.dumps(v)}" + sep)
    out.append("}")
    return "\n".join(out) + "\n"


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--dtype", default="bf16", choices=["f32", "bf16", "f16"])
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  "batch_tuning.json"))
    ap.add_argument("--target-nnz", type=int, default=16_000_000)
    args = ap.parse_args()
    if not torch.cuda.is_available():
        raise SystemExit("the tuner times kernels: it needs a GPU")
    table = tune(args.dtype, args.target_nnz)
    with open(args.out, "w") as f:
        f.write(dumps(table))
    print(f"wrote {len(table['entries'])} entries to {args.out}")


if __name__ == "__main__":
    main()
