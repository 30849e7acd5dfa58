"""Matrix ingest (the step before the path): the MatrixMarket reader against
the restated reference loader, on files the tests write, and the
reference's own golden CSR of datasets/chesapeake (written back out as a
symmetric pattern file, read and converted)."""
import os

import numpy as np
import pytest

from conftest import load_golden


def write_mtx(path, rows, cols, entries, field="real", symmetry="general", comments=True):
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {symmetry}\n")
        if comments:
            f.write("% written by the test\n%\n\n")
        f.write(f"{rows} {cols} {len(entries)}\n")
        for e in entries:
            if field == "pattern":
                f.write(f"{e[0] + 1} {e[1] + 1}\n")
            elif field == "integer":
                f.write(f"{e[0] + 1} {e[1] + 1} {int(e[2])}\n")
            else:
                f.write(f"{e[0] + 1}  {e[1] + 1}   {e[2]!r}\n")


def random_entries(rng, rows, cols, n, dup=0):
    ent = [(int(rng.integers(rows)), int(rng.integers(cols)), float(rng.uniform(-2, 2)))
           for _ in range(n)]
    ent += [ent[int(rng.integers(len(ent)))] for _ in range(dup)]
    return ent


def chesapeake_file(tmp_path):
    g = load_golden("chesapeake.npz")
    off, idx = g["offsets"], g["indices"]
    ent = []
    for r in range(len(off) - 1):
        for c in idx[off[r]:off[r + 1]]:
            if c <= r:
                ent.append((r, int(c), 1.0))
    rng = np.random.default_rng(5)
    ent = [ent[i] for i in rng.permutation(len(ent))]
    p = tmp_path / "chesapeake_pattern.mtx"
    write_mtx(p, len(off) - 1, len(off) - 1, ent, field="pattern", symmetry="symmetric")
    return p, g


@pytest.mark.parametrize("field,symmetry", [("real", "general"), ("integer", "general"),
                                            ("pattern", "symmetric"), ("real", "symmetric"),
                                            ("real", "skew-symmetric")])
def test_reader_matches_reference_loader(tmp_path, oracle_mod, field, symmetry):
    from edge_loops_gb300 import api
    rng = np.random.default_rng(hash((field, symmetry)) % 2**32)
    ent = random_entries(rng, 50, 70 if symmetry == "general" else 50, 400, dup=10)
    p = tmp_path / "m.mtx"
    write_mtx(p, 50, 70 if symmetry == "general" else 50, ent, field, symmetry)
    got = api.read_matrix_market(str(p))
    want = oracle_mod.matrix_market_coo(str(p))
    assert got[0] == want[0] and got[1] == want[1]
    for a, b in zip(got[2:], want[2:]):
        np.testing.assert_array_equal(a, b)


def test_reader_errors(tmp_path):
    from edge_loops_gb300 import _lib, api
    cases = {
        "missing": (None, _lib.EL_ERR_IO),
        "zero_based": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1.0\n",
                       _lib.EL_ERR_PARSE),
        "array": ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
                  _lib.EL_ERR_UNSUPPORTED),
        "complex": ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n",
                    _lib.EL_ERR_UNSUPPORTED),
        "truncated": ("%%MatrixMarket matrix coordinate real general\n3 3 4\n1 1 1\n2 2 2\n",
                      _lib.EL_ERR_PARSE),
        "outside": ("%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1\n",
                    _lib.EL_ERR_PARSE),
        "banner": ("hello\n1 1 1\n1 1 1\n", _lib.EL_ERR_PARSE),
    }
    for name, (text, status) in cases.items():
        p = tmp_path / f"{name}.mtx"
        if text is not None:
            p.write_text(text)
        with pytest.raises(_lib.ElError) as e:
            api.read_matrix_market(str(p))
        assert e.value.status == status, name


def test_chesapeake_golden_through_reader_and_oracle(tmp_path, oracle_mod):
    """Reader + restated CSR construction reproduce the CSR the reference's
    own loader and thrust sort built for chesapeake (the golden fixture)."""
    from edge_loops_gb300 import api
    p, g = chesapeake_file(tmp_path)
    rows, cols, ri, ci, vv = api.read_matrix_market(str(p))
    assert (rows, cols, len(ri)) == (39, 39, 340)
    off, idx, val = oracle_mod.csr_from_coo(rows, ri, ci, vv)
    np.testing.assert_array_equal(off, g["offsets"])
    np.testing.assert_array_equal(idx, g["indices"])
    np.testing.assert_array_equal(val, g["values"])


@pytest.mark.gpu
def test_csr_from_coo_on_gpu(cuda, oracle_mod, tmp_path):
    from edge_loops_gb300 import _lib, api
    import torch
    rng = np.random.default_rng(9)
    for rows, cols, n, dup in [(1000, 800, 20000, 500), (3, 5, 0, 0), (1, 1, 7, 3),
                               (70000, 100, 300000, 1000)]:
        ent = random_entries(rng, rows, cols, n, dup) if n else []
        ri = np.array([e[0] for e in ent], dtype=np.int32)
        ci = np.array([e[1] for e in ent], dtype=np.int32)
        vv = np.array([e[2] for e in ent], dtype=np.float32)
        A = api.csr_from_coo(rows, cols, ri, ci, vv, device=cuda)
        torch.cuda.synchronize()
        off, idx, val = oracle_mod.csr_from_coo(rows, ri, ci, vv)
        np.testing.assert_array_equal(A.offsets.cpu().numpy(), off)
        np.testing.assert_array_equal(A.indices.cpu().numpy(), idx)
        np.testing.assert_array_equal(A.values.cpu().numpy(), val)
    p, g = chesapeake_file(tmp_path)
    rows, cols, ri, ci, vv = api.read_matrix_market(str(p))
    A = api.csr_from_coo(rows, cols, ri, ci, vv, device=cuda)
    np.testing.assert_array_equal(A.offsets.cpu().numpy(), g["offsets"])
    np.testing.assert_array_equal(A.indices.cpu().numpy(), g["indices"])
    y = api.spmv(A, torch.as_tensor(g["x"], device=cuda))
    np.testing.assert_array_equal(y.cpu().numpy(), g["y_exact"].astype(np.float32))
    with pytest.raises(_lib.ElError) as e:
        api.csr_from_coo(3, 3, [0, 3], [0, 0], [1.0, 2.0], device=cuda)
    assert e.value.status == _lib.EL_ERR_MALFORMED_CSR
