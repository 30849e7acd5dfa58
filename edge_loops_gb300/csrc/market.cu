// market.cu -- el_read_matrix_market: a MatrixMarket coordinate file into a
// host COO, with the reference loader's semantics
// [include/loops/container/market.hxx:99-227]:
//   * banner "%%MatrixMarket matrix coordinate <field> <symmetry>", field
//     real, integer or pattern (pattern entries get the value 1.0), values
//     read as double and stored as float;
//   * 1-based indices in the file (an index 0 is an error), stored 0-based;
//   * "symmetric" files: every off-diagonal entry (i, j) is followed by its
//     mirror (j, i) with the same value, diagonal entries are kept once;
//     other symmetries (general, skew-symmetric, hermitian) are read as
//     written, as the reference does.
// Unlike the reference, failures return a status instead of exiting, and
// sizes beyond int32 are rejected before anything is allocated.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "el_internal.h"

namespace el {
namespace {

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// next line that is neither blank nor a comment; false at end of file
bool next_line(FILE* f, std::string& line) {
  char buf[4096];
  while (fgets(buf, sizeof buf, f)) {
    line.assign(buf);
    while (!line.empty() && line.back() != '\n' && !feof(f) && fgets(buf, sizeof buf, f))
      line.append(buf);  // lines longer than the buffer
    size_t i = 0;
    while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
    if (i == line.size() || line[i] == '%') continue;
    return true;
  }
  return false;
}

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_read_matrix_market(const char* path, el_coo* out) {
  if (!path || !out) return fail(EL_ERR_NULL_POINTER, "path or out is NULL");
  std::memset(out, 0, sizeof(*out));
  File file;
  file.f = fopen(path, "r");
  if (!file.f) return fail(EL_ERR_IO, "cannot open %s", path);
  char banner[1024];
  if (!fgets(banner, sizeof banner, file.f))
    return fail(EL_ERR_PARSE, "%s: empty file", path);
  char w[5][128] = {{0}};
  if (sscanf(banner, "%127s %127s %127s %127s %127s", w[0], w[1], w[2], w[3], w[4]) != 5 ||
      lower(w[0]) != "%%matrixmarket" || lower(w[1]) != "matrix")
    return fail(EL_ERR_PARSE, "%s: not a MatrixMarket matrix banner", path);
  const std::string format = lower(w[2]), field = lower(w[3]), symmetry = lower(w[4]);
  if (format != "coordinate")
    return fail(EL_ERR_UNSUPPORTED, "%s: only coordinate files are supported", path);
  const bool pattern = field == "pattern";
  if (!pattern && field != "real" && field != "integer")
    return fail(EL_ERR_UNSUPPORTED, "%s: field '%s' not supported", path, w[3]);
  if (symmetry != "general" && symmetry != "symmetric" && symmetry != "skew-symmetric" &&
      symmetry != "hermitian")
    return fail(EL_ERR_PARSE, "%s: unknown symmetry '%s'", path, w[4]);
  const bool mirror = symmetry == "symmetric";

  std::string line;
  if (!next_line(file.f, line)) return fail(EL_ERR_PARSE, "%s: no size line", path);
  long long rows = -1, cols = -1, entries = -1;
  if (sscanf(line.c_str(), "%lld %lld %lld", &rows, &cols, &entries) != 3 || rows < 0 ||
      cols < 0 || entries < 0)
    return fail(EL_ERR_PARSE, "%s: bad size line '%s'", path, line.c_str());
  if (rows >= (1LL << 31) - 1 || cols >= (1LL << 31) - 1 || entries >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "%s: sizes exceed int32", path);

  std::vector<int32_t> ri, ci;
  std::vector<float> vv;
  ri.reserve((size_t)entries);
  ci.reserve((size_t)entries);
  vv.reserve((size_t)entries);
  long long off_diag = 0;
  for (long long k = 0; k < entries; ++k) {
    if (!next_line(file.f, line))
      return fail(EL_ERR_PARSE, "%s: %lld of %lld entries", path, k, entries);
    const char* p = line.c_str();
    char* end = nullptr;
    const long long i = strtoll(p, &end, 10);
    if (end == p) return fail(EL_ERR_PARSE, "%s: entry %lld: '%s'", path, k, p);
    p = end;
    const long long j = strtoll(p, &end, 10);
    if (end == p) return fail(EL_ERR_PARSE, "%s: entry %lld: '%s'", path, k, line.c_str());
    p = end;
    double v = 1.0;
    if (!pattern) {
      v = strtod(p, &end);
      if (end == p) return fail(EL_ERR_PARSE, "%s: entry %lld has no value", path, k);
    }
    if (i == 0 || j == 0) return fail(EL_ERR_PARSE, "%s: zero-based index in entry %lld", path, k);
    if (i < 1 || i > rows || j < 1 || j > cols)
      return fail(EL_ERR_PARSE, "%s: entry %lld (%lld, %lld) outside %lld x %lld", path, k, i,
                  j, rows, cols);
    ri.push_back((int32_t)(i - 1));
    ci.push_back((int32_t)(j - 1));
    vv.push_back((float)v);
    if (i != j) ++off_diag;
  }
  const long long nnz = mirror ? entries + off_diag : entries;
  if (nnz >= (1LL << 31)) return fail(EL_ERR_OVERFLOW, "%s: %lld nonzeros exceed int32", path, nnz);
  out->rows = rows;
  out->cols = cols;
  out->nnz = nnz;
  const size_t n = (size_t)(nnz > 0 ? nnz : 1);
  out->row_indices = static_cast<int32_t*>(std::malloc(n * sizeof(int32_t)));
  out->col_indices = static_cast<int32_t*>(std::malloc(n * sizeof(int32_t)));
  out->values = static_cast<float*>(std::malloc(n * sizeof(float)));
  if (!out->row_indices || !out->col_indices || !out->values) {
    el_coo_free(out);
    return fail(EL_ERR_OUT_OF_MEMORY, "%s: host allocation", path);
  }
  long long q = 0;
  for (size_t k = 0; k < ri.size(); ++k) {
    out->row_indices[q] = ri[k];
    out->col_indices[q] = ci[k];
    out->values[q] = vv[k];
    ++q;
    if (mirror && ri[k] != ci[k]) {  // the mirrored entry right after it
      out->row_indices[q] = ci[k];
      out->col_indices[q] = ri[k];
      out->values[q] = vv[k];
      ++q;
    }
  }
  return EL_OK;
}

extern "C" void el_coo_free(el_coo* coo) {
  if (!coo) return;
  std::free(coo->row_indices);
  std::free(coo->col_indices);
  std::free(coo->values);
  coo->row_indices = coo->col_indices = nullptr;
  coo->values = nullptr;
  coo->rows = coo->cols = coo->nnz = 0;
}
