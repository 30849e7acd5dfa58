"""Host logic of the two tuning tools (no GPU): tune_select's fit recovers
the constants of timings made by a known cost model and its choice is the
cheapest estimate; tune_batch's buckets follow the plan's bucket rules and
its table text round-trips through JSON."""
import json

import numpy as np
import pytest


def synthetic_sweep(consts, rng, n=60):
    """Timings of the candidates on random shapes, exactly as the cost model
    with `consts` predicts them; the staged kernel ("tms", where consts has
    it) is timed on short rows, as the model says where the rows are
    coherent and three times slower where they are not."""
    data = []
    for _ in range(n):
        rows = int(2 ** rng.uniform(6, 22))
        per = float(2 ** rng.uniform(0, 8))
        nnz = int(rows * per)
        mx = int(min(nnz, per * 2 ** rng.uniform(0, 10)))
        f = {"rows": rows, "nnz": nnz, "max": mx, "coh": float(rng.choice([0.0, 0.3, 0.9]))}
        a, e = consts["merge_path"]
        t = {"merge_path": a + e * (nnz + rows) / 1e6}
        for key in ("tm1", "tm4", "tm32", "tms"):
            if key not in consts or (key == "tms" and mx > 27):
                continue
            a, c, d, e = consts[key]
            t[key] = a + c * mx + d * rows / 1e3 + e * nnz / 1e6
            if key == "tms" and f["coh"] < 0.5:
                t[key] *= 3.0
        data.append(("synthetic", f, t))
    return data


def test_select_fit_recovers_a_known_model():
    pytest.importorskip("scipy")
    from edge_loops_gb300 import tune_select as ts
    consts = {"merge_path": (15.0, 4.0), "tm1": (7.0, 0.06, 0.004, 5.6),
              "tm4": (6.7, 0.044, 0.026, 3.2), "tm32": (6.7, 0.007, 0.2, 1.8)}
    data = synthetic_sweep(consts, np.random.default_rng(3))
    model = ts.fit(data)
    for k, v in consts.items():
        np.testing.assert_allclose(model[k], v, rtol=1e-6, atol=1e-9)
    q = ts.quality(data, lambda f: ts.predict(model, f))
    assert q["geomean"] == pytest.approx(1.0) and q["worst"] == pytest.approx(1.0)
    assert q["shapes"] == len(data)
    # always merge_path is worse on this data, and quality says so
    assert ts.quality(data, lambda f: "merge_path")["geomean"] > 1.0


def test_select_fit_of_the_staged_kernel_uses_only_the_shapes_it_applies_to():
    pytest.importorskip("scipy")
    from edge_loops_gb300 import tune_select as ts
    consts = {"merge_path": (15.0, 4.0), "tm1": (7.0, 0.06, 0.004, 5.6),
              "tm4": (6.7, 0.044, 0.026, 3.2), "tm32": (6.7, 0.007, 0.2, 1.8),
              "tms": (6.6, 0.0, 0.02, 1.5)}
    rng = np.random.default_rng(4)
    # short rows, so that many shapes carry a staged timing
    data = [d for d in synthetic_sweep(consts, rng, n=600) if d[1]["max"] <= 27][:80]
    assert sum(ts.staged_applies(f) for _, f, _ in data) >= 10
    assert any("tms" in t and not ts.staged_applies(f) for _, f, t in data)
    model = ts.fit(data)
    np.testing.assert_allclose(model["tms"], consts["tms"], rtol=1e-6, atol=1e-9)
    q = ts.quality(data, lambda f: ts.predict(model, f))
    assert q["geomean"] == pytest.approx(1.0) and q["worst"] == pytest.approx(1.0)
    # never the staged kernel where it does not apply
    assert all(ts.predict(model, f) != "tms" for _, f, _ in data if not ts.staged_applies(f))


def test_select_predict_takes_the_cheapest_estimate():
    from edge_loops_gb300 import tune_select as ts
    model = {"merge_path": (15.0, 4.0), "tm1": (7.0, 0.1, 0.0, 6.0),
             "tm4": (7.0, 0.05, 0.02, 3.0), "tm32": (7.0, 0.01, 0.2, 2.0)}
    assert ts.predict(model, {"rows": 1000, "nnz": 10000, "max": 10}).startswith("tm")
    assert ts.predict(model, {"rows": 1 << 20, "nnz": 16_000_000, "max": 100_000}) == \
        "merge_path"


def test_batch_buckets_and_table_text():
    from edge_loops_gb300 import _lib as L
    from edge_loops_gb300 import tune_batch as tb
    # rows: bucket b holds [2^b, 2^(b+1)), the last one everything above
    assert [tb.row_bucket(r) for r in (1, 2, 3, 4, 7, 8)] == [0, 1, 1, 2, 2, 3]
    assert tb.row_bucket(1 << 40) == L.EL_BATCH_ROW_BUCKETS - 1
    # mean row length: 0 below 1, then one bucket per power of two
    assert [tb.len_bucket(a) for a in (0.5, 1.0, 1.9, 2.0, 3.9, 4.0)] == [0, 1, 1, 2, 2, 3]
    assert tb.len_bucket(1e9) == L.EL_BATCH_LEN_BUCKETS - 1
    assert [tb.cv_bucket(c) for c in (0.0, 0.25, 0.74, 0.75, 1.49, 1.5, 9.0)] == \
        [0, 1, 1, 2, 2, 3, 3]
    table = {"threads_per_row": [1, 2], "entries": {"3,4,1": [64, 12], "0,1,0": [4, 10]},
             "note": "x"}
    assert json.loads(tb.dumps(table)) == table


def test_plan_default_table_is_the_validated_one():
    """The plan's default table is what the tuner's validation on a mixed
    batch kept (the recorded GB300 run kept no entry, so none is shipped
    and the built-in rule applies to every bucket)."""
    import os
    from conftest import REPO
    from edge_loops_gb300 import api
    rec = json.load(open(os.path.join(REPO, "tests", "data", "batch_tuning_gb300_bf16.json")))
    assert rec["validation"][0]["row_bucket"] is None  # the built-in rule's time comes first
    kept = {k: v for k, v in rec["entries"].items()}
    shipped = api.load_tuning_table()
    if kept:
        np.testing.assert_array_equal(shipped, api.tuning_table(kept))
    else:
        assert shipped is None
    # every recorded step that dropped a row bucket's candidates was not faster by 1 %
    base = rec["validation"][0]["ms"]
    for step in rec["validation"][1:-1]:
        assert step["kept"] or step["ms"] > 0.99 * base


def test_validation_keeps_only_row_buckets_that_speed_up_the_batch():
    """The tuner's greedy validation on a fake batch timer: a row bucket's
    candidates stay only when the batch gets >= 1 % faster with them on top
    of those already kept; the log ends with all candidates together."""
    from edge_loops_gb300 import tune_batch as tb
    entries = {"3,2,0": [4, 11], "3,3,1": [64, 10], "8,4,0": [64, 11], "12,5,2": [1, 12],
               "14,1,0": [32, 13]}
    effect = {3: -0.05, 8: +0.02, 12: -0.004, 14: -0.03}  # relative change per row bucket

    def time_of(ent):
        t = 1.0
        for rb in {int(k.split(",")[0]) for k in ent}:
            t *= 1.0 + effect[rb]
        return t

    kept, log = tb.select_entries(entries, time_of)
    assert set(kept) == {"3,2,0", "3,3,1", "14,1,0"}
    assert [s["row_bucket"] for s in log] == [None, 3, 8, 12, 14, "all candidates"]
    assert [s["kept"] for s in log[1:-1]] == [True, False, False, True]
    assert log[-1]["ms"] == pytest.approx(0.95 * 1.02 * 0.996 * 0.97, abs=1e-5)
    assert tb.select_entries({}, time_of) == ({}, [log[0], {"row_bucket": "all candidates",
                                                           "ms": 1.0, "kept": False}])
