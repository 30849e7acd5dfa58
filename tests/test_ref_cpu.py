"""The oracle's restatement of the reference's CPU SpMV against the
reference's own cpu::reference (examples/spmv/helpers.hxx:97-115) compiled
from its sources (oracle/_ref/ref_cpu, built by oracle/ref/build_ref.sh
where the reference sources are present): y must be identical bit for bit,
on the chesapeake matrix, the 1000 x 1000 benchmark matrix, random shapes
with empty and long rows, and the full 16M-nonzero power-law benchmark
matrix."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden, random_csr

EXE = os.path.join(REPO, "oracle", "_ref", "ref_cpu")
pytestmark = pytest.mark.skipif(not os.path.exists(EXE),
                                reason="oracle/_ref/ref_cpu not built (needs the reference sources)")


def _run_ref(tmp_path, off, idx, vals, x):
    rows, cols, nnz = len(off) - 1, len(x), len(idx)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([rows, cols, nnz], dtype=np.int64).tofile(f)
        np.asarray(off, np.int32).tofile(f)
        np.asarray(idx, np.int32).tofile(f)
        np.asarray(vals, np.float32).tofile(f)
        np.asarray(x, np.float32).tofile(f)
    subprocess.run([EXE, str(inp), str(out)], check=True, timeout=300)
    return np.fromfile(out, dtype=np.float32)[:rows]


def _cases():
    g = load_golden("chesapeake.npz")
    yield "chesapeake", g["offsets"], g["indices"], g["values"], \
        np.random.default_rng(0).uniform(-1, 1, 39).astype(np.float32)
    from edge_loops_gb300 import synth
    o, i, v, x, _ = synth.uniform_rows(rows=1000, cols=1000, per_row=10, seed=0)
    yield "uniform1000", o.numpy(), i.numpy(), v.numpy(), x.numpy()
    rng = np.random.default_rng(8)
    for k in range(3):
        off, idx, vals, x = random_csr(rng, rows=2000, cols=2000, max_len=70, empty_frac=0.3,
                                       long_rows=[(5, 1900)])
        yield "random%d" % k, off, idx, vals, x


@pytest.mark.parametrize("name", ["chesapeake", "uniform1000", "random0", "random1", "random2"])
def test_oracle_equals_compiled_reference(tmp_path, oracle_mod, name):
    off, idx, vals, x = next(c[1:] for c in _cases() if c[0] == name)
    ref = _run_ref(tmp_path, off, idx, vals, x)
    got = oracle_mod.spmv_f32(off, idx, vals, x)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_oracle_equals_compiled_reference_power_law_16M(tmp_path, oracle_mod):
    from edge_loops_gb300 import synth
    o, i, v, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000, exponent=2.0,
                                       cap=100_000, seed=1)
    o, i, v, x = o.numpy(), i.numpy(), v.numpy(), x.numpy()
    ref = _run_ref(tmp_path, o, i, v, x)
    got = oracle_mod.spmv_f32(o, i, v, x)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
