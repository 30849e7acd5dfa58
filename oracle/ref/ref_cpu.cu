// ref_cpu.cu -- the reference's own CPU SpMV, cpu::reference
// (examples/spmv/helpers.hxx:97-115), compiled from the reference's sources
// by oracle/ref/build_ref.sh, to pin the oracle's restatement of it
// (oracle/oracle.c) bit for bit.  Thrust's device system is set to CPP, so
// the reference's "device" CSR and vectors are thrust vectors in host
// memory and the program runs without a GPU; the loop itself is the
// reference's, unchanged.  Test infrastructure only.
//
//   in : int64 rows, cols, nnz; int32 offsets[rows+1]; int32 indices[nnz];
//        float values[nnz]; float x[cols]
//   out: float y[cols]  (cpu::reference returns x.size() entries; rows <= cols)
#include <cstdio>
#include <vector>

#include "helpers.hxx"

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  long long hdr[3];
  if (std::fread(hdr, sizeof(long long), 3, f) != 3) return 2;
  const long long rows = hdr[0], cols = hdr[1], nnz = hdr[2];
  if (rows < 0 || cols < rows || nnz < 0) return 2;
  std::vector<int> off(rows + 1), idx(nnz);
  std::vector<float> val(nnz), xh(cols);
  if (std::fread(off.data(), 4, rows + 1, f) != (size_t)(rows + 1)) return 2;
  if (nnz && std::fread(idx.data(), 4, nnz, f) != (size_t)nnz) return 2;
  if (nnz && std::fread(val.data(), 4, nnz, f) != (size_t)nnz) return 2;
  if (cols && std::fread(xh.data(), 4, cols, f) != (size_t)cols) return 2;
  std::fclose(f);

  loops::csr_t<int, int, float> A(rows, cols, nnz);
  thrust::copy(off.begin(), off.end(), A.offsets.begin());
  thrust::copy(idx.begin(), idx.end(), A.indices.begin());
  thrust::copy(val.begin(), val.end(), A.values.begin());
  loops::vector_t<float> x(cols);
  thrust::copy(xh.begin(), xh.end(), x.begin());

  auto y = cpu::reference(A, x);

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(y.data(), 4, y.size(), o);
  std::fclose(o);
  return 0;
}
