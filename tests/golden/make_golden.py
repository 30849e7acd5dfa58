"""Regenerates the golden fixtures in this folder from the reference itself.

Run in a container that has the reference sources (it builds and runs
oracle/_ref/ref_fixtures, which is compiled from the reference's own
MatrixMarket loader, COO->CSR conversion, x generator and sample CSR):

    python tests/golden/make_golden.py [--ref /path/to/loops]

Outputs (committed):
  chesapeake.npz  CSR of datasets/chesapeake/chesapeake.mtx exactly as the
                  reference builds it (symmetric expansion, thrust sort), the
                  x the reference draws with seed 7 (integers in [1, 10], as
                  examples/spmv/merge_path.cu:33 asks for), and y = A x in
                  exact integer arithmetic (all values are 1.0, so every
                  summation order gives this y in float as well).
  sample.npz      util/sample.hxx:58-90 (4x4, 4 nonzeros) and its exact y for
                  x = [1, 2, 3, 4].
"""
import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def read_bin(path):
    with open(path, "rb") as f:
        rows, cols, nnz = np.frombuffer(f.read(24), dtype=np.int64)
        offsets = np.frombuffer(f.read(4 * (rows + 1)), dtype=np.int32).copy()
        indices = np.frombuffer(f.read(4 * nnz), dtype=np.int32).copy()
        values = np.frombuffer(f.read(4 * nnz), dtype=np.float32).copy()
        (xlen,) = np.frombuffer(f.read(8), dtype=np.int64)
        x = np.frombuffer(f.read(4 * xlen), dtype=np.float32).copy()
    return int(rows), int(cols), int(nnz), offsets, indices, values, x


def exact_spmv(offsets, indices, values, x):
    """y = A x with int64 arithmetic (values and x must be integers)."""
    v = values.astype(np.int64)
    xi = x.astype(np.int64)
    assert np.all(v == values) and np.all(xi == x)
    rows = len(offsets) - 1
    row_of = np.repeat(np.arange(rows), np.diff(offsets))
    y = np.zeros(rows, dtype=np.int64)
    np.add.at(y, row_of, v * xi[indices])
    return y


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("LOOPS_REF", "/root/reference"))
    args = ap.parse_args()
    env = dict(os.environ, LOOPS_REF=args.ref)
    subprocess.check_call([os.path.join(REPO, "oracle", "ref", "build_ref.sh")], env=env)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_fixtures")
    tmp = os.path.join(REPO, "oracle", "_ref")

    mtx = os.path.join(args.ref, "datasets", "chesapeake", "chesapeake.mtx")
    out = os.path.join(tmp, "chesapeake.bin")
    subprocess.check_call([exe, mtx, "7", out])
    rows, cols, nnz, off, idx, val, x = read_bin(out)
    y = exact_spmv(off, idx, val, x)
    np.savez(os.path.join(HERE, "chesapeake.npz"), rows=rows, cols=cols, nnz=nnz,
             offsets=off, indices=idx, values=val, x=x, y_exact=y, seed=7)
    print(f"chesapeake: {rows} x {cols} ({nnz})")

    out = os.path.join(tmp, "sample.bin")
    subprocess.check_call([exe, "--sample", out])
    rows, cols, nnz, off, idx, val, _ = read_bin(out)
    xs = np.arange(1, cols + 1, dtype=np.float32)
    y = exact_spmv(off, idx, val, xs)
    np.savez(os.path.join(HERE, "sample.npz"), rows=rows, cols=cols, nnz=nnz,
             offsets=off, indices=idx, values=val, x=xs, y_exact=y)
    print(f"sample: {rows} x {cols} ({nnz}) y={y.tolist()}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
