// ref_fixtures.cu -- fixture generator built against the reference's own
// host-side headers (test infrastructure; never part of the product).
//
// It drives the reference's MatrixMarket loader (container/market.hxx:99-227),
// its host COO -> CSR conversion (container/csr.hxx:138-146, coo.hxx:104-145,
// detail/convert.hxx:69-78), its x generator
// (util/generate.hxx:54-79) and its 4x4 sample CSR (util/sample.hxx:58-90),
// and writes what they produce as raw little-endian arrays:
//
//   ref_fixtures <file.mtx> <seed> <out.bin>   -> CSR + x of the .mtx file
//   ref_fixtures --sample <out.bin>            -> sample::csr() (host)
//
// Layout of out.bin: int64 rows, cols, nnz; int32 offsets[rows+1];
// int32 indices[nnz]; float values[nnz]; int64 xlen; float x[xlen].
#include <loops/error.hxx>
#include <loops/container/container.hxx>
#include <loops/container/csr.hxx>
#include <loops/container/coo.hxx>
#include <loops/util/generate.hxx>
#include <loops/util/sample.hxx>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace loops;

template <typename csr_host_t>
static int write_csr(const char* path, const csr_host_t& csr,
                     const std::vector<float>& x) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return 1;
  int64_t hdr[3] = {(int64_t)csr.rows, (int64_t)csr.cols, (int64_t)csr.nnzs};
  std::fwrite(hdr, sizeof(int64_t), 3, f);
  for (size_t i = 0; i < csr.rows + 1; ++i) {
    int32_t v = csr.offsets[i];
    std::fwrite(&v, 4, 1, f);
  }
  for (size_t i = 0; i < csr.nnzs; ++i) {
    int32_t v = csr.indices[i];
    std::fwrite(&v, 4, 1, f);
  }
  for (size_t i = 0; i < csr.nnzs; ++i) {
    float v = csr.values[i];
    std::fwrite(&v, 4, 1, f);
  }
  int64_t xlen = (int64_t)x.size();
  std::fwrite(&xlen, sizeof(int64_t), 1, f);
  if (xlen) std::fwrite(x.data(), 4, x.size(), f);
  std::fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 3 && std::strcmp(argv[1], "--sample") == 0) {
    auto csr = sample::csr<memory_space_t::host, int, int, float>();
    return write_csr(argv[2], csr, std::vector<float>());
  }
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <file.mtx> <seed> <out.bin> | --sample <out.bin>\n", argv[0]);
    return 2;
  }
  matrix_market_t<int, int, float> mtx;
  csr_t<int, int, float, memory_space_t::host> csr(mtx.load(argv[1]));
  unsigned seed = (unsigned)std::strtoul(argv[2], nullptr, 10);
  // examples/spmv/merge_path.cu:33 draws x with the integer distribution in
  // [1, 10]; here with a fixed seed instead of the clock.
  vector_t<float, memory_space_t::host> xh(csr.cols);
  generate::random::uniform_distribution(xh.begin(), xh.end(), 1, 10, seed);
  std::vector<float> x(xh.begin(), xh.end());
  return write_csr(argv[3], csr, x);
}
