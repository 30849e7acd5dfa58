"""COO matrices and the edge (nonzero) partitioner, the reference's coo_t
(include/loops/container/coo.hxx:30-167), Partitioner
(include/loops/util/partitioner.hxx:68-301) and the thread-mapped edge
schedule's SpMV (schedule_edge/thread_mapped.hxx:45-117,
examples/spmv/thread_mapped_edge.cu:16-34), over the C ABI.

The method names are the reference's.  The differences: the partition is
built on the GPU (the reference loops on the host), it is held as the
CSR-like arrays of el_edge_partition (quarks, atom_begin, atom_x, atom_y,
tile_begin) rather than pointer-carrying structs, atom and tile sizes are
given together (partition_tiles_* runs the C call, with the atom sizes that
partition_atoms_* recorded), and prepare_gpu() has nothing left to do.
"""
import ctypes as C

import torch

from . import _lib as L
from .api import CSR, _ptr, _stream, _ws


class COO:
    """A COO matrix in device memory: int32 row and column indices, float32
    values (coo_t with memory_space_t::device)."""

    def __init__(self, rows, cols, row_indices, col_indices, values):
        self.rows = int(rows)
        self.cols = int(cols)
        self.row_indices = row_indices
        self.col_indices = col_indices
        self.values = values

    @property
    def nnzs(self):  # the reference's field name
        return int(self.values.numel())

    @property
    def device(self):
        return self.values.device

    @classmethod
    def from_arrays(cls, rows, cols, row_indices, col_indices, values, device="cuda"):
        dev = torch.device(device)
        return cls(rows, cols,
                   torch.as_tensor(row_indices, dtype=torch.int32).to(dev).contiguous(),
                   torch.as_tensor(col_indices, dtype=torch.int32).to(dev).contiguous(),
                   torch.as_tensor(values, dtype=torch.float32).to(dev).contiguous())

    @classmethod
    def from_csr(cls, A, stream=None):
        """coo_t(csr_t) [coo.hxx:90-97]: row indices expanded from the
        offsets (el_csr_row_indices), the CSR's column indices and values."""
        if A.values.dtype != torch.float32 or A.row_scale is not None:
            raise ValueError("from_csr needs float32 values without row scales")
        ri = torch.empty(A.nnz, dtype=torch.int32, device=A.device)
        L.check(L.lib().el_csr_row_indices(_ptr(A.offsets), A.rows, A.nnz,
                                           _ptr(ri) if A.nnz else None, _stream(stream)),
                "el_csr_row_indices")
        return cls(A.rows, A.cols, ri, A.indices, A.values)

    def el(self):
        c = L.ElCoo()
        c.rows, c.cols, c.nnz = self.rows, self.cols, self.nnzs
        n = self.nnzs
        c.row_indices = self.row_indices.data_ptr() if n else None
        c.col_indices = self.col_indices.data_ptr() if n else None
        c.values = self.values.data_ptr() if n else None
        return c

    def _sort(self, by_column, stream, workspace):
        c = self.el()
        L.check(L.lib().el_coo_sort(_ws(workspace), C.byref(c), by_column, _stream(stream)),
                "el_coo_sort")

    def sort_by_row(self, stream=None, workspace=None):
        """In place, stable, by (row, column) [coo.hxx:104-110]."""
        self._sort(0, stream, workspace)

    def sort_by_column(self, stream=None, workspace=None):
        """In place, stable, by (column, row) [coo.hxx:116-122]."""
        self._sort(1, stream, workspace)

    def to_csr(self, stream=None, workspace=None):
        """csr_t(coo_t) [csr.hxx:86-94] (el_csr_from_coo)."""
        from .api import csr_from_coo
        return csr_from_coo(self.rows, self.cols, self.row_indices, self.col_indices,
                            self.values, device=self.device, stream=stream,
                            workspace=workspace)


class Partitioner:
    """Partitions the nonzeros (quarks) of a COO into atoms and the atoms
    into tiles [partitioner.hxx:68-301].  Like the reference, the
    constructor sorts A by row (in place) unless sort=False."""

    def __init__(self, A, sort=True, stream=None, workspace=None):
        self.A = A
        self.stream = stream
        self.workspace = workspace
        if sort:
            A.sort_by_row(stream=stream, workspace=workspace)
        self._atoms = None
        self.P = None
        self.arrays = None

    def partition_atoms_coordinate_space(self, M0, K0):
        """Atoms of M0 rows x K0 columns [:81-127] (the sizes are checked
        here, the partition is built by partition_tiles_coordinate_space)."""
        P = L.ElEdgePartition()
        L.check(L.lib().el_edge_partition_coordinate_plan(self.A.rows, self.A.cols,
                                                          self.A.nnzs, int(M0), int(K0), 1, 1,
                                                          C.byref(P)),
                "partition_atoms_coordinate_space")
        self._atoms = ("coordinate", int(M0), int(K0))

    def partition_atoms_position_space(self, nnzs_per_atom):
        """Atoms of nnzs_per_atom consecutive nonzeros [:178-206]."""
        P = L.ElEdgePartition()
        L.check(L.lib().el_edge_partition_position_plan(self.A.nnzs, int(nnzs_per_atom), 1,
                                                        C.byref(P)),
                "partition_atoms_position_space")
        self._atoms = ("position", int(nnzs_per_atom))

    def _alloc(self, P):
        dev = self.A.device
        arr = {
            "quarks": torch.empty(max(P.nnz, 0), dtype=torch.int32, device=dev),
            "atom_begin": torch.empty(P.num_atoms + 1, dtype=torch.int32, device=dev),
            "atom_x": torch.empty(P.num_atoms, dtype=torch.int32, device=dev),
            "atom_y": torch.empty(P.num_atoms, dtype=torch.int32, device=dev),
            "tile_begin": torch.empty(P.num_tiles + 1, dtype=torch.int32, device=dev),
        }
        P.quarks = arr["quarks"].data_ptr() if P.nnz else None
        P.atom_begin = arr["atom_begin"].data_ptr()
        P.atom_x = arr["atom_x"].data_ptr() if P.num_atoms else None
        P.atom_y = arr["atom_y"].data_ptr() if P.num_atoms else None
        P.tile_begin = arr["tile_begin"].data_ptr()
        return arr

    def partition_tiles_coordinate_space(self, M1, K1):
        """Tiles of M1 x K1 atoms [:129-176]."""
        if not self._atoms or self._atoms[0] != "coordinate":
            raise RuntimeError("partition_tiles_coordinate_space(): need to partition "
                               "work atoms (coordinate space) first")
        _, M0, K0 = self._atoms
        A = self.A
        P = L.ElEdgePartition()
        L.check(L.lib().el_edge_partition_coordinate_plan(A.rows, A.cols, A.nnzs, M0, K0,
                                                          int(M1), int(K1), C.byref(P)),
                "el_edge_partition_coordinate_plan")
        arr = self._alloc(P)
        c = A.el()
        L.check(L.lib().el_edge_partition_coordinate(_ws(self.workspace), C.byref(c), M0, K0,
                                                     int(M1), int(K1), C.byref(P),
                                                     _stream(self.stream)),
                "el_edge_partition_coordinate")
        self.P, self.arrays = P, arr

    def partition_tiles_position_space(self, num_atoms_per_tile):
        """Tiles of num_atoms_per_tile consecutive atoms [:208-226]."""
        if not self._atoms or self._atoms[0] != "position":
            raise RuntimeError("partition_tiles_position_space(): need to partition "
                               "work atoms (position space) first")
        P = L.ElEdgePartition()
        L.check(L.lib().el_edge_partition_position_plan(self.A.nnzs, self._atoms[1],
                                                        int(num_atoms_per_tile), C.byref(P)),
                "el_edge_partition_position_plan")
        arr = self._alloc(P)
        L.check(L.lib().el_edge_partition_position(self._atoms[1], int(num_atoms_per_tile),
                                                   C.byref(P), _stream(self.stream)),
                "el_edge_partition_position")
        self.P, self.arrays = P, arr

    def prepare_gpu(self):
        """The partition already lives in device memory [:228-258]."""
        if self.P is None:
            raise RuntimeError("prepare_gpu(): need to partition work atoms and tiles first")

    def get_work_tiles(self):
        """The partition's device arrays: quarks, atom_begin, atom_x, atom_y,
        tile_begin."""
        self.prepare_gpu()
        return self.arrays

    def get_num_tiles(self):
        self.prepare_gpu()
        return int(self.P.num_tiles)


def spmv_edge(A, partitioner, x, y=None, track=False, stream=None, workspace=None):
    """y = A x over the partition's tiles (el_spmv_edge); with track=True
    also returns quark_tile (the tile that processed each nonzero, the
    reference's Tracker under its one-thread-per-tile launch)."""
    P = partitioner.P
    if P is None:
        raise RuntimeError("partition the matrix first")
    if y is None:
        y = torch.empty(A.rows, dtype=torch.float32, device=A.device)
    qt = torch.empty(A.nnzs, dtype=torch.int32, device=A.device) if track else None
    c = A.el()
    L.check(L.lib().el_spmv_edge(_ws(workspace), C.byref(c), C.byref(P), _ptr(x), _ptr(y),
                                 _ptr(qt) if (track and A.nnzs) else None, _stream(stream)),
            "el_spmv_edge")
    return (y, qt) if track else y


__all__ = ["COO", "Partitioner", "spmv_edge", "CSR"]
