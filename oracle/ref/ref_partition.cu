// ref_partition.cu -- fixture generator for the edge partitioner, built
// against the reference's own Partitioner (util/partitioner.hxx:68-301) and
// host COO (container/coo.hxx) -- test infrastructure, never part of the
// product.  Host code only: the device half of the Partitioner
// (prepare_gpu) is not called.
//
//   ref_partition <in.bin> <out.bin> coord M0 K0 M1 K1
//   ref_partition <in.bin> <out.bin> pos nnz_per_atom atoms_per_tile
//
// in.bin : int64 rows, cols, nnz; int32 row[nnz]; int32 col[nnz];
//          float val[nnz]
// out.bin: int64 rows, cols, nnz; int32 row[nnz]; int32 col[nnz] (the COO
//          after the Partitioner's sort_by_row); int64 num_atoms,
//          num_tiles, atoms_x, atoms_y; int32 quarks[nnz] (tile by tile,
//          atom by atom); int32 atom_begin[num_atoms + 1]; int32
//          atom_x[num_atoms]; int32 atom_y[num_atoms]; int32
//          tile_begin[num_tiles + 1] -- the host-side WorkTile / WorkAtom
//          structure flattened, quark ranges read from the atoms' pointers.
//
// The Partitioner keeps its structure in private members with no host
// accessor, so they are opened to this driver by redefining `private`
// around that one header.
#include <loops/error.hxx>
#include <loops/range.hxx>
#include <loops/container/formats.hxx>
#include <loops/container/vector.hxx>
#include <loops/container/coo.hxx>
#include <loops/memory.hxx>

#define private public
#include <loops/util/partitioner.hxx>
#undef private

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace loops;
using quarks_t = std::size_t;

static void put64(FILE* f, long long v) {
  int64_t x = v;
  std::fwrite(&x, 8, 1, f);
}
static void put32(FILE* f, long long v) {
  int32_t x = (int32_t)v;
  std::fwrite(&x, 4, 1, f);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s in.bin out.bin coord M0 K0 M1 K1 | pos P T\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  int64_t hdr[3];
  if (std::fread(hdr, 8, 3, f) != 3) return 1;
  const size_t nnz = (size_t)hdr[2];
  coo_t<int, float, memory_space_t::host> A(hdr[0], hdr[1], nnz);
  std::vector<int32_t> buf(nnz);
  std::vector<float> vb(nnz);
  if (std::fread(buf.data(), 4, nnz, f) != nnz) return 1;
  for (size_t i = 0; i < nnz; ++i) A.row_indices[i] = buf[i];
  if (std::fread(buf.data(), 4, nnz, f) != nnz) return 1;
  for (size_t i = 0; i < nnz; ++i) A.col_indices[i] = buf[i];
  if (std::fread(vb.data(), 4, nnz, f) != nnz) return 1;
  for (size_t i = 0; i < nnz; ++i) A.values[i] = vb[i];
  std::fclose(f);

  Partitioner<int, float, quarks_t> part(A);  // sorts A by row
  try {
    if (std::strcmp(argv[3], "coord") == 0 && argc == 8) {
      part.partition_atoms_coordinate_space(std::strtoull(argv[4], nullptr, 10),
                                            std::strtoull(argv[5], nullptr, 10));
      part.partition_tiles_coordinate_space(std::strtoull(argv[6], nullptr, 10),
                                            std::strtoull(argv[7], nullptr, 10));
    } else if (std::strcmp(argv[3], "pos") == 0 && argc == 6) {
      part.partition_atoms_position_space(std::strtoull(argv[4], nullptr, 10));
      part.partition_tiles_position_space(std::strtoull(argv[5], nullptr, 10));
    } else {
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "partition error: %s\n", e.what());
    return 4;
  }
  const bool coord = std::strcmp(argv[3], "coord") == 0;

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 1;
  put64(o, (long long)A.rows);
  put64(o, (long long)A.cols);
  put64(o, (long long)A.nnzs);
  for (size_t i = 0; i < nnz; ++i) put32(o, A.row_indices[i]);
  for (size_t i = 0; i < nnz; ++i) put32(o, A.col_indices[i]);
  put64(o, (long long)part.num_atoms);
  put64(o, (long long)part.num_tiles);
  put64(o, coord ? (long long)part.num_atoms_x : 0);
  put64(o, coord ? (long long)part.num_atoms_y : 0);
  std::vector<long long> quarks, atom_begin(1, 0), ax, ay, tile_begin(1, 0);
  for (size_t t = 0; t < part.num_tiles; ++t) {
    const auto& tile = part.work_tiles[t];
    for (auto* a = tile.begin(); a != tile.end(); ++a) {
      for (const quarks_t* q = a->begin(); q != a->end(); ++q) quarks.push_back((long long)*q);
      atom_begin.push_back((long long)quarks.size());
      ax.push_back((long long)a->get_x_idx());
      ay.push_back((long long)a->get_y_idx());
    }
    tile_begin.push_back((long long)ax.size());
  }
  for (long long v : quarks) put32(o, v);
  for (long long v : atom_begin) put32(o, v);
  for (long long v : ax) put32(o, v);
  for (long long v : ay) put32(o, v);
  for (long long v : tile_begin) put32(o, v);
  std::fclose(o);
  return 0;
}
