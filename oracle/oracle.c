/*
 * oracle.c -- CPU restatement of the `loops` CSR SpMV/SpMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (edge_loops_gb300/,
 * include/) links, loads or calls this file.  It is used by tests/ as the
 * parity checker, by __graft_entry__.smoke() as the checker of one small
 * launch, and by bench.py's CPU-baseline leg (the timed CPU arm).
 *
 * Every function restates a piece of the reference and cites the file:line
 * it follows (paths relative to the reference project root):
 *
 *   oracle_spmv_f32          examples/spmv/helpers.hxx:106-112  (cpu::reference)
 *   oracle_spmv_f32_mt       same loop, rows split over host threads
 *   oracle_spmv_f64_q        same loop in FP64 over the exactly dequantised values
 *   oracle_spmm_f32          algorithms/spmm/thread_mapped.cuh:41-52 loop order
 *   oracle_spmm_f64_q        same, FP64
 *   oracle_mp_search         util/search.hxx:34-60 (search::_binary_search)
 *   oracle_merge_path_tile_coords
 *                            schedule/merge_path_flat.hxx:108-138
 *                            (generate_search_coordinates)
 *   oracle_merge_path_thread_coords
 *                            schedule/merge_path_flat.hxx:321-385 (setup::init)
 *   oracle_merge_path_walk   brute-force sequential merge of row-ends and
 *                            nonzeros (pins the search independently)
 *   oracle_work_oriented_coords
 *                            schedule/work_oriented.hxx:141-167 (setup::init)
 *   oracle_group_mapped_map  schedule/group_mapped.hxx:146-235 (partition,
 *                            atom_accessor, tile_accessor, tile_id, atom_id)
 *
 * Built with -ffp-contract=off so that `sum += v * x` rounds the product and
 * the sum separately, exactly as the reference's C++ loop is written.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <math.h>
#include <pthread.h>

/* ---------------------------------------------------------------- dtypes -- */
/* value dtype codes shared with include/edge_loops.h: 0 f32, 1 bf16, 2 f16 */

static double bf16_to_double(uint16_t h) {
  uint32_t u = ((uint32_t)h) << 16;
  float f;
  memcpy(&f, &u, 4);
  return (double)f;
}

static double f16_to_double(uint16_t h) {
  int sign = (h >> 15) & 1;
  int exp = (h >> 10) & 0x1f;
  int man = h & 0x3ff;
  double v;
  if (exp == 0)
    v = ldexp((double)man, -24); /* subnormal: man * 2^-24 */
  else if (exp == 31)
    v = man ? NAN : INFINITY;
  else
    v = ldexp((double)(man | 0x400), exp - 25);
  return sign ? -v : v;
}

static double load_value(const void* vals, int dtype, int64_t i) {
  if (dtype == 0) return (double)((const float*)vals)[i];
  if (dtype == 1) return bf16_to_double(((const uint16_t*)vals)[i]);
  return f16_to_double(((const uint16_t*)vals)[i]);
}

/* ------------------------------------------------------------------ SpMV -- */

/* examples/spmv/helpers.hxx:106-112: serial row loop, float accumulation in
 * nonzero order, y[row] overwritten. */
void oracle_spmv_f32(int64_t rows, const int32_t* offsets,
                     const int32_t* indices, const float* values,
                     const float* x, float* y) {
  for (int64_t row = 0; row < rows; ++row) {
    float sum = 0;
    for (int32_t nz = offsets[row]; nz < offsets[row + 1]; ++nz)
      sum += values[nz] * x[indices[nz]];
    y[row] = sum;
  }
}

/* The same loop with the rows split into contiguous blocks, one per host
 * thread (used only as the multi-core CPU baseline; results are identical to
 * oracle_spmv_f32 because each row is still summed serially). */
typedef struct {
  int64_t r0, r1;
  const int32_t* offsets;
  const int32_t* indices;
  const float* values;
  const float* x;
  float* y;
} spmv_job_t;

static void* spmv_job(void* p) {
  spmv_job_t* j = (spmv_job_t*)p;
  for (int64_t row = j->r0; row < j->r1; ++row) {
    float sum = 0;
    for (int32_t nz = j->offsets[row]; nz < j->offsets[row + 1]; ++nz)
      sum += j->values[nz] * j->x[j->indices[nz]];
    j->y[row] = sum;
  }
  return NULL;
}

int oracle_spmv_f32_mt(int64_t rows, const int32_t* offsets,
                       const int32_t* indices, const float* values,
                       const float* x, float* y, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  spmv_job_t jobs[256];
  /* split rows so that every thread gets about the same number of nonzeros */
  int64_t nnz = offsets[rows];
  int64_t r = 0;
  for (int t = 0; t < threads; ++t) {
    int64_t target = (nnz * (t + 1)) / threads;
    int64_t r1 = r;
    if (t == threads - 1) {
      r1 = rows;
    } else {
      int64_t lo = r, hi = rows;
      while (lo < hi) { /* first row whose start offset reaches target */
        int64_t mid = lo + (hi - lo) / 2;
        if (offsets[mid] < target) lo = mid + 1; else hi = mid;
      }
      r1 = lo;
    }
    jobs[t].r0 = r; jobs[t].r1 = r1; jobs[t].offsets = offsets;
    jobs[t].indices = indices; jobs[t].values = values; jobs[t].x = x;
    jobs[t].y = y;
    r = r1;
  }
  int started = 0;
  for (int t = 0; t < threads; ++t) {
    if (pthread_create(&tid[t], NULL, spmv_job, &jobs[t]) != 0) {
      spmv_job(&jobs[t]);
      tid[t] = 0;
    } else {
      started++;
    }
  }
  for (int t = 0; t < threads; ++t)
    if (tid[t]) pthread_join(tid[t], NULL);
  return started;
}

/* FP64 restatement of the same loop over the exactly dequantised stored
 * values (value * row_scale[row] when a scale is given).  Also returns, per
 * row, sum_j |a_ij * x_j|, the denominator of the componentwise error bound.
 * yabs may be NULL. */
void oracle_spmv_f64_q(int64_t rows, const int32_t* offsets,
                       const int32_t* indices, const void* values, int dtype,
                       const float* row_scale, const float* x, double* y,
                       double* yabs) {
  for (int64_t row = 0; row < rows; ++row) {
    double sum = 0, asum = 0;
    double s = row_scale ? (double)row_scale[row] : 1.0;
    for (int32_t nz = offsets[row]; nz < offsets[row + 1]; ++nz) {
      double p = load_value(values, dtype, nz) * s * (double)x[indices[nz]];
      sum += p;
      asum += fabs(p);
    }
    y[row] = sum;
    if (yabs) yabs[row] = asum;
  }
}

/* ------------------------------------------------------------------ SpMM -- */

/* algorithms/spmm/thread_mapped.cuh:41-52: for each row, for each column of
 * B, a float sum over the row's nonzeros.  B is row-major cols x n with
 * leading dimension ldb, C row-major rows x n with leading dimension ldc
 * (matrix.cuh:27-35 uses ld == n). */
void oracle_spmm_f32(int64_t rows, const int32_t* offsets,
                     const int32_t* indices, const float* values,
                     const float* B, int64_t n, int64_t ldb, float* C,
                     int64_t ldc) {
  for (int64_t row = 0; row < rows; ++row)
    for (int64_t col = 0; col < n; ++col) {
      float sum = 0;
      for (int32_t nz = offsets[row]; nz < offsets[row + 1]; ++nz)
        sum += values[nz] * B[(int64_t)indices[nz] * ldb + col];
      C[row * ldc + col] = sum;
    }
}

/* FP64 SpMM over dequantised values and a B given as f32 (b_dtype 0) or
 * bf16 (b_dtype 1) or f16 (b_dtype 2). cabs may be NULL. */
void oracle_spmm_f64_q(int64_t rows, const int32_t* offsets,
                       const int32_t* indices, const void* values, int dtype,
                       const float* row_scale, const void* B, int b_dtype,
                       int64_t n, int64_t ldb, double* C, double* cabs) {
  for (int64_t row = 0; row < rows; ++row) {
    double s = row_scale ? (double)row_scale[row] : 1.0;
    for (int64_t col = 0; col < n; ++col) {
      double sum = 0, asum = 0;
      for (int32_t nz = offsets[row]; nz < offsets[row + 1]; ++nz) {
        double p = load_value(values, dtype, nz) * s *
                   load_value(B, b_dtype, (int64_t)indices[nz] * ldb + col);
        sum += p;
        asum += fabs(p);
      }
      C[row * n + col] = sum;
      if (cabs) cabs[row * n + col] = asum;
    }
  }
}

/* ------------------------------------------------------------ merge path -- */

/* util/search.hxx:34-60.  Merge of list a (row-end offsets, a_len entries)
 * with list b (the counting sequence b0, b0+1, ...; b_len entries) cut at
 * `diagonal`.  x is thrust::lower_bound over the counting range
 * [max(diag-b_len,0), min(diag,a_len)) with predicate a[i] <= b[diag-i-1];
 * the result is {min(x, a_len), diag - x}.  All arithmetic is the
 * reference's int arithmetic. */
void oracle_mp_search(int64_t diagonal, const int32_t* a, int64_t a_len,
                      int64_t b0, int64_t b_len, uint32_t* out_x,
                      uint32_t* out_y) {
  int x_min = (int)diagonal - (int)b_len;
  if (x_min < 0) x_min = 0;
  int x_max = (int)diagonal < (int)a_len ? (int)diagonal : (int)a_len;
  /* thrust::lower_bound (sequential): first position where the predicate
   * is false; an empty or inverted range returns its first element. */
  int64_t first = x_min;
  int64_t len = (int64_t)x_max - (int64_t)x_min;
  while (len > 0) {
    int64_t half = len / 2;
    int64_t mid = first + half;
    int32_t bval = (int32_t)(b0 + (diagonal - mid - 1));
    if (a[mid] <= bval) {
      first = mid + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  *out_x = (uint32_t)(first < a_len ? first : a_len);
  *out_y = (uint32_t)(diagonal - first);
}

/* schedule/merge_path_flat.hxx:108-138: the start coordinate of every merge
 * tile (plus the end of the last one) at diagonal k * items_per_tile, over
 * a = offsets + 1 (row ends) and b = 0..nnz-1.  out holds 2*(num_tiles+1)
 * uint32 (x, y pairs). Returns num_tiles. */
int64_t oracle_merge_path_tile_coords(int64_t rows, int64_t nnz,
                                      const int32_t* offsets,
                                      int64_t items_per_tile, uint32_t* out) {
  int64_t total = rows + nnz;
  int64_t tiles = (total + items_per_tile - 1) / items_per_tile;
  for (int64_t t = 0; t <= tiles; ++t) {
    int64_t diag = t * items_per_tile;
    oracle_mp_search(diag, offsets + 1, rows, 0, nnz, &out[2 * t],
                     &out[2 * t + 1]);
  }
  return tiles;
}

/* schedule/merge_path_flat.hxx:321-385, for every block of the launch in
 * algorithms/spmv/merge_path_flat.cuh:102-127: threads 0/1 search the tile
 * start/end diagonals; the block gathers the tile's row-end offsets
 * (item < tile_num_tiles + items_per_thread, index clamped to rows-1) into
 * shared memory; each thread searches local diagonal tid*items_per_thread in
 * that array against the counting sequence starting at the tile's first
 * nonzero.  Writes, per (tile, thread), the LOCAL coordinate the reference
 * thread starts from: out[2*(tile*tpb+tid)+{0,1}].  Returns num_tiles. */
int64_t oracle_merge_path_thread_coords(int64_t rows, int64_t nnz,
                                        const int32_t* offsets, int64_t tpb,
                                        int64_t ipt, uint32_t* out,
                                        int32_t* scratch /* tpb*ipt+ipt+1 */) {
  int64_t items = tpb * ipt;
  int64_t total = rows + nnz;
  int64_t tiles = (total + items - 1) / items;
  const int32_t* end_offsets = offsets + 1;
  for (int64_t t = 0; t < tiles; ++t) {
    uint32_t sx, sy, ex, ey;
    oracle_mp_search(t * items, end_offsets, rows, 0, nnz, &sx, &sy);
    oracle_mp_search((t + 1) * items, end_offsets, rows, 0, nnz, &ex, &ey);
    int64_t tile_num_tiles = (int64_t)ex - (int64_t)sx;
    int64_t tile_num_atoms = (int64_t)ey - (int64_t)sy;
    for (int64_t item = 0; item < tile_num_tiles + ipt; ++item) {
      int64_t off = (int64_t)sx + item;
      if (off > rows - 1) off = rows - 1;
      scratch[item] = end_offsets[off];
    }
    for (int64_t tid = 0; tid < tpb; ++tid) {
      uint32_t x, y;
      oracle_mp_search(tid * ipt, scratch, tile_num_tiles, (int64_t)sy,
                       tile_num_atoms, &x, &y);
      out[2 * (t * tpb + tid)] = x;
      out[2 * (t * tpb + tid) + 1] = y;
    }
  }
  return tiles;
}

/* Independent pin of the search: walk the whole merge of row ends and
 * nonzeros item by item (a row end is taken when the next nonzero index is
 * not below the row's end offset) and record the coordinate reached at each
 * diagonal k*step, k = 0..floor(total/step), plus the final one. out must
 * hold 2*(total/step+2) uint32.  Returns the number of coordinates
 * written. */
int64_t oracle_merge_path_walk(int64_t rows, int64_t nnz,
                               const int32_t* offsets, int64_t step,
                               uint32_t* out) {
  int64_t x = 0, y = 0, d = 0, k = 0;
  int64_t total = rows + nnz;
  for (;;) {
    if (d % step == 0 || d == total) {
      out[2 * k] = (uint32_t)x;
      out[2 * k + 1] = (uint32_t)y;
      k++;
    }
    if (d == total) break;
    if (x < rows && (y >= nnz || y >= offsets[x + 1]))
      x++;
    else
      y++;
    d++;
  }
  return k;
}

/* schedule/work_oriented.hxx:141-167: with num_threads threads, every
 * thread gets work_per_thread = ceil((rows+nnz)/num_threads) merge items;
 * thread tid searches diagonals min(wpt*tid, total) and
 * min(that + wpt, total).  out[4*tid + {0,1,2,3}] = st.x, st.y, en.x, en.y
 * (int64). */
void oracle_work_oriented_coords(int64_t rows, int64_t nnz,
                                 const int32_t* offsets, int64_t num_threads,
                                 int64_t* out) {
  int64_t total = rows + nnz;
  int64_t wpt = (total + num_threads - 1) / num_threads;
  for (int64_t tid = 0; tid < num_threads; ++tid) {
    int64_t upper = wpt * tid < total ? wpt * tid : total;
    int64_t lower = upper + wpt < total ? upper + wpt : total;
    uint32_t x, y;
    oracle_mp_search(upper, offsets + 1, rows, 0, nnz, &x, &y);
    out[4 * tid] = x;
    out[4 * tid + 1] = y;
    oracle_mp_search(lower, offsets + 1, rows, 0, nnz, &x, &y);
    out[4 * tid + 2] = x;
    out[4 * tid + 3] = y;
  }
}

/* schedule/group_mapped.hxx:146-235 with THREADS_PER_TILE == tpt and a
 * block of tpb threads: tile (group) g of tpt consecutive rows takes its
 * row lengths' exclusive scan; virtual atom v (strided by tpt) maps to the
 * local row upper_bound(scan, v) - 1 and to the nonzero
 * offsets[row] + v - scan[local].  For every group, in group order and then
 * virtual-atom order, writes the (row, nz) each virtual atom maps to.
 * Returns the number of atoms written (== nnz for a well-formed CSR). */
int64_t oracle_group_mapped_map(int64_t rows, const int32_t* offsets,
                                int64_t tpt, int32_t* atom_row,
                                int32_t* atom_nz, int32_t* scan /* tpt */) {
  int64_t w = 0;
  for (int64_t g0 = 0; g0 < rows; g0 += tpt) {
    int64_t length = rows - g0 < tpt ? rows - g0 : tpt; /* get_length */
    int32_t agg = 0;
    for (int64_t k = 0; k < tpt; ++k) {
      int32_t n = 0;
      if (g0 + k < rows) n = offsets[g0 + k + 1] - offsets[g0 + k];
      scan[k] = agg;
      agg += n;
    }
    for (int32_t v = 0; v < agg; ++v) {
      /* thrust::upper_bound over scan[0..length) */
      int64_t lo = 0, hi = length;
      while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (v < scan[mid]) hi = mid; else lo = mid + 1;
      }
      int64_t local = lo - 1;
      if (local >= length) continue; /* is_valid_accessor */
      int64_t row = g0 + local;
      atom_row[w] = (int32_t)row;
      atom_nz[w] = offsets[row] + v - scan[local];
      w++;
    }
  }
  return w;
}
