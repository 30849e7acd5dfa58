"""Host-side parts of bench.py that need no GPU: the clock-sample summary
(throttle reasons must not be missed), the roofline denominator and DRAM
traffic lookups, and the CPU baseline's line on a small matrix."""
import json
import os

import pytest

from conftest import REPO


def _bench():
    import bench
    return bench


def test_clock_summary_reads_reasons_and_skips_junk():
    b = _bench()
    na = "Not Active"
    lines = [
        f"0, 2070, 2070, 800.1, 0x0000000000000000, {na}, {na}, {na}, {na}",
        f"0, 2055, 2070, 1390.0, 0x0000000000000004, {na}, {na}, {na}, Active",
        f"0, 1500, 2070, 1395.0, 0x0000000000000008, Active, {na}, {na}, {na}",
        "garbage line",
        "0, [N/A], 2070, 1.0, 0x0, a, b, c, d",
        "",
    ]
    s = b.ClockSampler.summarize(lines)
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert b.ClockSampler.summarize([]) == {"sm_mhz": None, "sm_max_mhz": None,
                                            "reasons": [], "samples": 0}


def test_peak_and_traffic_lookups():
    b = _bench()
    peak, kind = b.measured_peaks()
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        assert kind == "measured"
        assert peak == float(json.load(open(p))["hbm_gbs"])
    else:
        assert kind == "fallback"
    t = b.traffic_for("spmv_powerlaw:merge_path_flat:f32")
    assert t is not None and 1.0e8 < t < 2.0e8  # DRAM bytes of one 137 MB SpMV
    assert b.traffic_for("no such workload") is None


def test_cpu_baseline_line_on_a_small_matrix():
    pytest.importorskip("torch")
    b = _bench()
    from edge_loops_gb300 import synth
    off, idx, vals, x, cols = synth.uniform_rows(rows=1000, cols=1000, per_row=10, seed=0)
    W = dict(off=off, idx=idx, vals=vals, x=x, rows=1000, cols=cols)
    line = b.cpu_baseline(W, None, budget_s=0.05, threads=2)
    assert line["unit"] == "GB/s" and line["kind"] == "port" and line["cores"] == 2
    assert line["value"] > 0 and line["single_thread"]["value"] > 0
    assert "helpers.hxx:106-112" in line["sample"]


def test_fp64_checker_matches_the_oracle(oracle_mod):
    """bench.py checks its outputs with its own FP64 evaluation; it must agree
    with the oracle's FP64 loop (empty rows, row scales, row blocks that cut
    the matrix into several chunks)."""
    import numpy as np
    from conftest import random_csr
    b = _bench()
    rng = np.random.default_rng(4)
    off, idx, vals, x = random_csr(rng, rows=900, cols=700, max_len=40, empty_frac=0.25,
                                   long_rows=[(3, 600)])
    scale = np.exp2(rng.integers(-3, 4, size=900)).astype(np.float32)
    for sc in (None, scale):
        y, ya = b.fp64_spmv(off, idx, vals, x, sc, chunk=1000)
        y0, ya0 = oracle_mod.spmv_f64(off, idx, vals, x, row_scale=sc)
        np.testing.assert_allclose(y, y0, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(ya, ya0, rtol=1e-12, atol=1e-12)
    c, n = b.rel_errors(y0.astype(np.float32), y0, ya0)
    c0, n0 = oracle_mod.error_metrics(y0.astype(np.float32), y0, ya0)
    assert abs(c - c0) <= 1e-15 and abs(n - n0) <= 1e-15
