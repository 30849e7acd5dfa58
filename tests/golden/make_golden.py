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
  edge_partitions.npz
                  the reference's Partitioner (util/partitioner.hxx, run on
                  the host through oracle/_ref/ref_partition) on two shuffled
                  COOs: the row-sorted COO and the host-side tile / atom /
                  quark structure for each case in PARTITION_CASES, and which
                  of PARTITION_ERRORS it rejects.
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
    from oracle.ref import sources
    ap.add_argument("--ref", default=sources())
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

    make_partitions(os.path.join(REPO, "oracle", "_ref", "ref_partition"), tmp)
    return 0


# (matrix, mode, sizes): coordinate (M0, K0, M1, K1) / position (P, T)
PARTITION_CASES = [
    ("chesapeake", "coord", (4, 4, 2, 3)), ("chesapeake", "coord", (1, 39, 1, 1)),
    ("chesapeake", "coord", (39, 39, 1, 1)), ("chesapeake", "coord", (5, 7, 3, 2)),
    ("chesapeake", "coord", (3, 2, 5, 4)), ("chesapeake", "pos", (16, 4)),
    ("chesapeake", "pos", (7, 3)), ("chesapeake", "pos", (340, 1)),
    ("chesapeake", "pos", (1, 1000)),
    ("random", "coord", (16, 16, 3, 2)), ("random", "coord", (7, 5, 6, 9)),
    ("random", "coord", (300, 1, 1, 50)), ("random", "pos", (64, 3)),
    ("random", "pos", (100, 7)),
]
# sizes the reference rejects (it throws): M0 or K0 0 or above the matrix,
# M1 / K1 above the atom grid, nnz_per_atom 0 or above nnz
PARTITION_ERRORS = [
    ("chesapeake", "coord", (0, 4, 1, 1)), ("chesapeake", "coord", (40, 4, 1, 1)),
    ("chesapeake", "coord", (4, 40, 1, 1)), ("chesapeake", "coord", (4, 4, 11, 1)),
    ("chesapeake", "coord", (4, 4, 1, 0)), ("chesapeake", "pos", (0, 1)),
    ("chesapeake", "pos", (341, 1)),
]


def partition_matrices():
    """The COO inputs (shuffled, so the Partitioner's row sort matters):
    chesapeake's entries from the committed CSR, and a 300 x 200 random COO
    with repeated entries."""
    g = np.load(os.path.join(HERE, "chesapeake.npz"))
    off = g["offsets"]
    ri = np.repeat(np.arange(len(off) - 1), np.diff(off)).astype(np.int32)
    ci = g["indices"].astype(np.int32)
    perm = np.random.default_rng(5).permutation(len(ci))
    mats = {"chesapeake": (int(g["rows"]), int(g["cols"]), ri[perm], ci[perm],
                           g["values"][perm].astype(np.float32))}
    rng = np.random.default_rng(11)
    n = 3000
    rr = rng.integers(0, 300, n).astype(np.int32)
    cc = rng.integers(0, 200, n).astype(np.int32)
    rr[1::7], cc[1::7] = rr[0::7][: len(rr[1::7])], cc[0::7][: len(cc[1::7])]  # repeats
    mats["random"] = (300, 200, rr, cc, rng.uniform(-1, 1, n).astype(np.float32))
    return mats


def run_partition(exe, tmp, mat, mode, sizes):
    rows, cols, ri, ci, vv = mat
    inp, outp = os.path.join(tmp, "part_in.bin"), os.path.join(tmp, "part_out.bin")
    with open(inp, "wb") as f:
        np.array([rows, cols, len(ri)], dtype=np.int64).tofile(f)
        ri.tofile(f)
        ci.tofile(f)
        vv.tofile(f)
    r = subprocess.run([exe, inp, outp, mode] + [str(s) for s in sizes], capture_output=True)
    if r.returncode != 0:
        return None
    b = open(outp, "rb").read()
    pos = [0]

    def take(n, dt):
        k = n * np.dtype(dt).itemsize
        a = np.frombuffer(b[pos[0]:pos[0] + k], dtype=dt).copy()
        pos[0] += k
        return a

    _, _, nnz = (int(v) for v in take(3, np.int64))
    d = {"rows_sorted": take(nnz, np.int32), "cols_sorted": take(nnz, np.int32)}
    na, nt, ax, ay = (int(v) for v in take(4, np.int64))
    d.update(atoms_x=ax, atoms_y=ay, quarks=take(nnz, np.int32),
             atom_begin=take(na + 1, np.int32), atom_x=take(na, np.int32),
             atom_y=take(na, np.int32), tile_begin=take(nt + 1, np.int32))
    assert pos[0] == len(b)
    return d


def make_partitions(exe, tmp):
    """edge_partitions.npz: the reference Partitioner's host-side structure
    (flattened) for PARTITION_CASES, and which PARTITION_ERRORS it rejects."""
    mats = partition_matrices()
    out = {}
    for name, (rows, cols, ri, ci, vv) in mats.items():
        out[f"{name}_shape"] = np.array([rows, cols], dtype=np.int64)
        out[f"{name}_row"], out[f"{name}_col"], out[f"{name}_val"] = ri, ci, vv
    for i, (name, mode, sizes) in enumerate(PARTITION_CASES):
        d = run_partition(exe, tmp, mats[name], mode, sizes)
        assert d is not None, (name, mode, sizes)
        for k, v in d.items():
            out[f"case{i}_{k}"] = np.asarray(v)
        out[f"case{i}_matrix"], out[f"case{i}_mode"] = np.array(name), np.array(mode)
        out[f"case{i}_sizes"] = np.array(sizes, dtype=np.int64)
    out["num_cases"] = np.array(len(PARTITION_CASES))
    rejected = []
    for i, (name, mode, sizes) in enumerate(PARTITION_ERRORS):
        rejected.append(run_partition(exe, tmp, mats[name], mode, sizes) is None)
        out[f"error{i}_matrix"], out[f"error{i}_mode"] = np.array(name), np.array(mode)
        out[f"error{i}_sizes"] = np.array(sizes, dtype=np.int64)
    out["num_errors"] = np.array(len(PARTITION_ERRORS))
    out["errors_rejected"] = np.array(rejected)
    np.savez_compressed(os.path.join(HERE, "edge_partitions.npz"), **out)
    print(f"edge partitions: {len(PARTITION_CASES)} cases, rejected {sum(rejected)} of "
          f"{len(PARTITION_ERRORS)} bad sizes")


if __name__ == "__main__":
    sys.exit(main())
