/*
 * edge_loops.h -- C ABI of the GB300-native load-balanced CSR SpMV/SpMM path.
 *
 * This header is the drop-in boundary for the `loops` library's SpMV/SpMM
 * hot path.  The reference exposes that path as C++ function templates with
 * no ABI; each entry point below replaces one of them (file:line of the
 * reference project in brackets):
 *
 *   el_spmv(.., EL_SCHED_THREAD_MAPPED, ..)
 *       loops::algorithms::spmv::thread_mapped / original
 *       [include/loops/algorithms/spmv/thread_mapped.cuh:68-91,
 *        include/loops/algorithms/spmv/original.cuh:59-76]
 *   el_spmv(.., EL_SCHED_GROUP_MAPPED, ..)
 *       loops::algorithms::spmv::group_mapped
 *       [include/loops/algorithms/spmv/group_mapped.cuh:73-105]
 *   el_spmv(.., EL_SCHED_WORK_ORIENTED, ..)
 *       loops::algorithms::spmv::work_oriented
 *       [include/loops/algorithms/spmv/work_oriented.cuh:88-111]
 *   el_spmv(.., EL_SCHED_MERGE_PATH_FLAT, ..)
 *       loops::algorithms::spmv::merge_path_flat
 *       [include/loops/algorithms/spmv/merge_path_flat.cuh:96-139]
 *   el_spmm(..)
 *       loops::algorithms::spmm::thread_mapped
 *       [include/loops/algorithms/spmm/thread_mapped.cuh:67-90]
 *   el_merge_path_partition / el_merge_path_thread_coords
 *       loops::schedule::merge_path::generate_search_coordinates and
 *       setup<merge_path_flat>::init
 *       [include/loops/schedule/merge_path_flat.hxx:108-138, :321-385]
 *   el_work_oriented_partition
 *       setup<work_oriented>::init [include/loops/schedule/work_oriented.hxx:150-167]
 *   el_read_matrix_market / el_csr_from_coo
 *       matrix_market_t::load and csr_t(coo_t)
 *       [include/loops/container/market.hxx:99-227, csr.hxx:86-94]
 *   el_coo_sort / el_csr_row_indices
 *       coo_t::sort_by_row, sort_by_column and coo_t(csr_t)
 *       [include/loops/container/coo.hxx:90-122]
 *   el_edge_partition_* / el_spmv_edge
 *       Partitioner and the thread-mapped edge schedule
 *       [include/loops/util/partitioner.hxx:68-301,
 *        include/loops/schedule_edge/thread_mapped.hxx:45-117]
 * and adds entry points the reference does not have: el_spmv_host (matrix,
 * x and y in host memory, streamed), el_spmv_static_scratch (no device
 * allocation), the batched plan (el_batch_plan_*), schedule selection
 * (el_spmv_select, el_select_schedule, el_select_schedule_stats,
 * el_csr_row_stats),
 * el_quantize_values and el_csr_validate.  include/edge_loops_device.cuh holds the device-side
 * load-balanced loop API for user kernels (the reference's schedule::setup).
 *
 * Conventions (differences from the reference are deliberate and listed):
 *   - Every call is asynchronous on the given stream (the reference ends
 *     each entry point with cudaStreamSynchronize).  Pointers are device
 *     pointers on the current device (host pointers where a call says so).
 *     Inputs are borrowed.
 *   - y (or C) is OVERWRITTEN; it need not be zeroed first (the reference's
 *     atomic schedules require a zeroed y; overwriting a zeroed y gives the
 *     same result).
 *   - No call throws across the ABI or exits the process; each returns an
 *     el_status.  el_last_error_string() describes the last failure on the
 *     calling thread.
 *   - Kernels never read or write outside the arrays the el_csr describes,
 *     whatever the offsets and indices contain: a malformed CSR gives wrong
 *     numbers and sets a device error flag (read it with
 *     el_workspace_errors), never a fault.  el_csr_validate checks a CSR
 *     completely and synchronously.
 *   - Values may be stored as FP32, BF16 or FP16; accumulation is always
 *     FP32.  x and y are FP32.
 */
#ifndef EDGE_LOOPS_H_
#define EDGE_LOOPS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ABI-identical to cudaStream_t (NULL = the legacy default stream). */
typedef struct CUstream_st* el_stream_t;

#define EL_VERSION 100 /* 1.0.0 */

typedef enum el_status {
  EL_OK = 0,
  EL_ERR_INVALID_ARGUMENT = 1, /* bad size, dtype, schedule option */
  EL_ERR_NULL_POINTER = 2,     /* a required pointer is NULL */
  EL_ERR_OVERFLOW = 3,         /* rows+nnz >= 2^31 - 2^16 (int32 merge
                                  path with headroom for tile arithmetic) */
  EL_ERR_UNSUPPORTED = 4,      /* e.g. the reference's unimplemented
                                  `bucketing` schedule */
  EL_ERR_MALFORMED_CSR = 5,    /* el_csr_validate found a defect */
  EL_ERR_CUDA = 6,             /* a CUDA runtime call failed */
  EL_ERR_OUT_OF_MEMORY = 7,    /* workspace allocation failed */
  EL_ERR_DEVICE = 8,           /* a kernel reported an error flag */
  EL_ERR_IO = 9,               /* a file could not be opened or read */
  EL_ERR_PARSE = 10            /* a MatrixMarket file is malformed */
} el_status;

/* Value storage types.  Accumulation is FP32 for all of them. */
typedef enum el_dtype { EL_F32 = 0, EL_BF16 = 1, EL_F16 = 2 } el_dtype;

/* Schedules.  Values 0-4 are the reference's
 * loops::schedule::algorithms_t [include/loops/schedule.hxx:23-29]. */
typedef enum el_schedule {
  EL_SCHED_MERGE_PATH_FLAT = 0,
  EL_SCHED_WORK_ORIENTED = 1,
  EL_SCHED_THREAD_MAPPED = 2,
  EL_SCHED_GROUP_MAPPED = 3,
  EL_SCHED_BUCKETING = 4, /* declared by the reference, never implemented:
                             returns EL_ERR_UNSUPPORTED */
  EL_SCHED_AUTO = 5       /* new: the selection model without row
                             statistics (merge_path but for tiny inputs);
                             el_spmv_select picks with them */
} el_schedule;

/* Device error flags (bit set), reported by el_workspace_errors and
 * el_csr_validate. */
#define EL_FLAG_INDEX_RANGE 0x1u  /* a column index outside [0, cols) */
#define EL_FLAG_OFFSETS 0x2u      /* offsets not monotone / outside [0,nnz] */
#define EL_FLAG_NNZ_MISMATCH 0x4u /* offsets[0] != 0 or offsets[rows] != nnz */
#define EL_FLAG_TIMEOUT 0x8u      /* a bounded device wait ran out */

/* A CSR matrix [include/loops/container/csr.hxx:32-95] as borrowed device
 * pointers.  With row_scale != NULL, A[i][j] = row_scale[i] * values[ij]
 * (per-row scales let BF16/FP16 storage keep each row in range; powers of
 * two keep the product exact). */
typedef struct el_csr {
  int64_t rows;
  int64_t cols;
  int64_t nnz;
  const int32_t* offsets; /* rows + 1 */
  const int32_t* indices; /* nnz column indices */
  const void* values;     /* nnz values of value_dtype */
  int32_t value_dtype;    /* el_dtype */
  int32_t reserved0;
  const float* row_scale; /* rows, or NULL */
} el_csr;

/* Tuning knobs; zero means "the schedule's default".  Initialise with
 * el_spmv_opts_default. */
typedef struct el_spmv_opts {
  int32_t threads_per_block; /* thread/group_mapped block size */
  int32_t items_per_thread;  /* merge_path variants 1 and 2: merge items per
                                thread and tile (1..16, tile = 256 x this);
                                variant 0 and work_oriented: unused */
  int32_t threads_per_row;   /* thread_mapped: 1,2,4,8,16,32 lanes per row */
  int32_t group_rows;        /* group_mapped: rows per group: 32 (one warp
                                per group, the reference's warp_mapped) or
                                threads_per_block (block_mapped) */
  int64_t num_threads;       /* work_oriented: threads of the even split,
                                a multiple of 128 (the reference uses
                                2 x SMs x 128); 0 = the resident blocks'
                                threads, or one per 256 merge items when
                                that is more (at most 16 x SMs x 128), and
                                none with fewer than 32 merge items */
  int32_t compensated;       /* 1: Neumaier / two-sum compensated FP32 sums */
  int32_t max_ctas;          /* cap on persistent grids (0 = resident) */
  int32_t wait_limit_us;     /* bound on every device-side wait (0 = 2 s) */
  int32_t test_hooks;        /* testing only, 0 in normal use: bit 0 makes
                                merge_path ranges skip publishing their row
                                carries, so a range that needs one waits until
                                wait_limit_us and reports EL_FLAG_TIMEOUT */
  int32_t variant;           /* merge_path kernel (same results within the
                                FP32 bound, deterministic):
                                0 = warp ranges walked in tiles of 256
                                    nonzeros, 8 per lane, vector loads;
                                1 = CTA ring: producer warps stream the range
                                    into shared memory with bulk copies;
                                2 = warp ranges walked in tiles of 256 merge
                                    items, lane t from the split point of
                                    diagonal 8t (the reference's per-thread
                                    split).
                                thread_mapped with one lane per row (y
                                bit-identical either way):
                                0 = each lane reads its row straight from
                                    the CSR arrays;
                                1 = a warp copies its 32 rows' indices and
                                    values into shared memory (TMA bulk
                                    copies, the next 32 rows in flight) and
                                    each lane walks its row from
                                    there: faster on short rows (the whole
                                    32-row chunk fits when no row holds more
                                    than 27 nonzeros; a chunk that does not
                                    is read as in 0, in its turn, which makes
                                    long rows slower than in 0).  Needs 16-byte
                                    aligned indices and values, else 0 runs.
                                    el_spmv_select sets it where it pays. */
  int32_t row_weight;        /* merge_path (variant 0): the warp ranges split
                                the merge of row ends and nonzeros with a
                                row end counted as this many nonzeros, so
                                ranges of short rows hold fewer items; 0 =
                                the library default, 1 = the reference's
                                equal split */
  int32_t nz_per_lane;       /* merge_path (variant 0): nonzeros per lane of the
                                tile walk, 8 (tiles of 256) or 16 (tiles of 512);
                                0 = 16 for 16-bit values on matrices with at
                                least 24 nonzeros per row on average and 2^20
                                nonzeros in all, else 8.  Same results within
                                the FP32 bound (the summation order changes) */
  int32_t reserved[3];
} el_spmv_opts;

typedef struct el_workspace el_workspace;

/* ---- library ---------------------------------------------------------- */
int el_version(void);
const char* el_status_string(el_status s);
const char* el_last_error_string(void);
void el_spmv_opts_default(el_spmv_opts* opts);

/* ---- workspaces --------------------------------------------------------
 * A workspace holds the small device state of the persistent schedules
 * (tile tickets, cross-CTA carries, the error flags).  Calls that pass
 * ws == NULL use a library-owned workspace per (device, stream).  A
 * workspace must not be used by two streams at the same time. */
el_status el_workspace_create(int device, el_workspace** out);
el_status el_workspace_destroy(el_workspace* ws);
/* Synchronises `stream`, returns the device error flags of `ws` (or of the
 * library workspace of this device/stream when ws == NULL) and clears them
 * when clear != 0. */
el_status el_workspace_errors(el_workspace* ws, el_stream_t stream,
                              uint32_t* flags, int clear);

/* ---- SpMV / SpMM ------------------------------------------------------ */
/* y = A x.  x has A->cols floats, y has A->rows floats. */
el_status el_spmv(el_workspace* ws, const el_csr* A, int32_t schedule,
                  const el_spmv_opts* opts, const float* x, float* y,
                  el_stream_t stream);

/* y = A x with the CSR arrays, row scales, x and y in HOST memory (no
 * counterpart in the reference).  The rows are cut into blocks of about
 * block_nnz nonzeros (0 = nnz / 2 clamped to [2^22, 2^27]); each block is
 * copied to device staging memory of the workspace on a copy stream while
 * the previous block is multiplied on `stream`, and its y rows are copied
 * back.  Pinned host memory gives full link speed; the device holds x, y
 * and two blocks at a time, so the matrix may exceed device memory.  The
 * host offsets must start at 0, end at nnz and not decrease between blocks
 * (EL_ERR_MALFORMED_CSR).  Asynchronous on `stream`: y is complete, and the
 * host arrays may be reused, once the stream has been synchronised.  Same
 * results as el_spmv within the FP32 bound (block borders change the merge
 * ranges). */
el_status el_spmv_host(el_workspace* ws, const el_csr* A, int32_t schedule,
                       const el_spmv_opts* opts, const float* x, float* y,
                       int64_t block_nnz, el_stream_t stream);

/* ---- matrix ingest (the step before the path) ------------------------ */
/* A matrix in coordinate form: nnz (row, column, value) entries, 0-based. */
typedef struct el_coo {
  int64_t rows, cols, nnz;
  int32_t* row_indices;
  int32_t* col_indices;
  float* values;
} el_coo;

/* Reads a MatrixMarket coordinate file (real / integer / pattern; general,
 * symmetric -- mirrored entries added --, skew-symmetric, hermitian read as
 * written) into host arrays allocated with malloc, released by
 * el_coo_free.  Replaces the reference's matrix_market_t::load
 * (include/loops/container/market.hxx:99-227), returning EL_ERR_IO /
 * EL_ERR_PARSE / EL_ERR_UNSUPPORTED instead of exiting. */
el_status el_read_matrix_market(const char* path, el_coo* out);
void el_coo_free(el_coo* coo);

/* CSR from a COO whose arrays are in device memory: entries sorted by
 * (row, column) -- stable, so duplicates keep their order and are all kept,
 * as the reference keeps them --, offsets (rows + 1), indices and values
 * (nnz each) written to caller-allocated device arrays.  Replaces
 * csr_t(coo_t) (include/loops/container/csr.hxx:86-94).  An entry outside
 * the matrix gives EL_ERR_MALFORMED_CSR (checked first: synchronises
 * `stream` once); the rest is asynchronous. */
el_status el_csr_from_coo(el_workspace* ws, const el_coo* coo, int32_t* offsets,
                          int32_t* indices, float* values, el_stream_t stream);

/* Sorts a COO whose arrays are in device memory, in place, by (row, column)
 * (by_column = 0) or (column, row) (by_column = 1), stable.  Replaces
 * coo_t::sort_by_row / sort_by_column
 * (include/loops/container/coo.hxx:104-122).  An entry outside the matrix
 * gives EL_ERR_MALFORMED_CSR before anything is written (synchronises
 * `stream` once). */
el_status el_coo_sort(el_workspace* ws, el_coo* coo, int32_t by_column,
                      el_stream_t stream);

/* The row index of every nonzero of a CSR (nnz entries, device memory):
 * the row indices of coo_t(csr_t) (include/loops/container/coo.hxx:90-97),
 * whose column indices and values are the CSR's own arrays. */
el_status el_csr_row_indices(const int32_t* offsets, int64_t rows, int64_t nnz,
                             int32_t* row_indices, el_stream_t stream);

/* ---- edge (nonzero) partitioner -----------------------------------------
 * The reference's Partitioner (include/loops/util/partitioner.hxx:68-301)
 * and the SpMV over its tiles (schedule_edge/thread_mapped.hxx,
 * examples/spmv/thread_mapped_edge.cu).  A quark is one nonzero (its
 * position in the COO), an atom a set of quarks, a tile a set of atoms.
 *
 *   coordinate space: atom (ax, ay) = the nonzeros of rows [ax M0, ax M0 +
 *     M0) and columns [ay K0, ay K0 + K0) in COO order; atoms row-major over
 *     the atoms_x x atoms_y grid; tile (tx, ty) = atom rows [tx M1, ..) and
 *     atom columns [ty K1, ..), tiles row-major, atoms in atom order.
 *   position space: atom i = quarks [i P, i P + P), tile t = atoms
 *     [t T, t T + T) (the last ones shorter).
 *
 * The partition is held as CSR-like arrays in device memory that the caller
 * allocates from the counts the *_plan call fills in:
 *   quarks[nnz]                 the quarks, tile by tile, atom by atom;
 *   atom_begin[num_atoms + 1]   atom a (in tile order) = quarks
 *                               [atom_begin[a], atom_begin[a + 1]);
 *   atom_x, atom_y[num_atoms]   the atom's grid coordinates (the
 *                               reference's x_idx / y_idx; 0 in position
 *                               space);
 *   tile_begin[num_tiles + 1]   tile t = atoms [tile_begin[t],
 *                               tile_begin[t + 1]).
 * A tile's quarks are therefore one contiguous range of `quarks`.  Sort the
 * COO by row first (el_coo_sort), as the reference's Partitioner does, for
 * its quark numbering.  The reference's argument rules hold: sizes > 0,
 * M0 <= rows, K0 <= cols, M1 <= atoms_x, K1 <= atoms_y, 0 < nnz_per_atom
 * <= nnz; atoms_per_tile must be > 0 (the reference divides by it). */
typedef struct el_edge_partition {
  int64_t nnz, num_atoms, num_tiles;
  int64_t atoms_x, atoms_y; /* the atom grid (coordinate space), else 0 */
  int32_t* quarks;
  int32_t* atom_begin;
  int32_t* atom_x;
  int32_t* atom_y;
  int32_t* tile_begin;
} el_edge_partition;

/* Fill P's counts (the arrays are left alone). */
el_status el_edge_partition_coordinate_plan(int64_t rows, int64_t cols,
                                            int64_t nnz, int64_t M0, int64_t K0,
                                            int64_t M1, int64_t K1,
                                            el_edge_partition* P);
el_status el_edge_partition_position_plan(int64_t nnz, int64_t nnz_per_atom,
                                          int64_t atoms_per_tile,
                                          el_edge_partition* P);
/* Fill P's arrays; P's counts must be the plan's for these arguments.  The
 * coordinate partition checks every entry is inside the matrix first
 * (EL_ERR_MALFORMED_CSR; synchronises `stream` once) and uses the
 * workspace's staging memory; the position partition is asynchronous. */
el_status el_edge_partition_coordinate(el_workspace* ws, const el_coo* A,
                                       int64_t M0, int64_t K0, int64_t M1,
                                       int64_t K1, el_edge_partition* P,
                                       el_stream_t stream);
el_status el_edge_partition_position(int64_t nnz_per_atom,
                                     int64_t atoms_per_tile,
                                     el_edge_partition* P, el_stream_t stream);
/* y = A x over the tiles of P, a warp per tile (the reference runs a thread
 * per tile); FP32, y overwritten, partial sums added atomically so the
 * summation order varies from run to run.  With quark_tile != NULL,
 * quark_tile[q] = the tile that processed quark q (the reference's Tracker
 * records the thread, which is the tile under its one-thread-per-tile
 * launch).  Quarks, rows or columns outside the arrays are skipped and
 * raise EL_FLAG_INDEX_RANGE in the workspace's flags (el_workspace_errors). */
el_status el_spmv_edge(el_workspace* ws, const el_coo* A,
                       const el_edge_partition* P, const float* x, float* y,
                       int32_t* quark_tile, el_stream_t stream);

/* ---- schedule selection ------------------------------------------------
 * The predictor the reference's paper fits to its per-matrix timings
 * (plots/data/heuristics.csv), here a cost model of this library's kernels
 * on GB300: estimated times of merge_path and of thread_mapped with 1, 4
 * and 32 lanes per row from (rows, nnz, longest row), and with the row
 * coherence also of one lane per row staged through shared memory.
 * EL_SCHED_AUTO in el_spmv cannot see the longest row without a
 * synchronisation, so it applies the model with the longest row taken as
 * nnz (the worst case):
 * merge_path, the choice that is never far off, except for matrices of a
 * few hundred nonzeros; callers that multiply by the same matrix
 * repeatedly call el_spmv_select once and reuse its choice (no cost per
 * call). */
typedef struct el_row_stats {
  int64_t max_row_nnz;
  int64_t empty_rows;
  double mean_row_nnz;
  double cv;        /* standard deviation / mean of the row lengths */
  double coherence; /* new: on about 2^16 sampled rows r, the fraction of the
                       first (up to 32) column pairs (col(r, j), col(r+1, j))
                       that step by 0, 1 or 2 -- near 1 on banded and stencil
                       matrices, near 0 on scattered columns */
} el_row_stats;

/* Row statistics of A's offsets, and the coherence from the indices of
 * sampled rows (one kernel; synchronises `stream`). */
el_status el_csr_row_stats(el_workspace* ws, const el_csr* A, el_row_stats* out,
                           el_stream_t stream);
/* The cost model without the coherence (the staged kernel is not weighed):
 * schedule (EL_SCHED_MERGE_PATH_FLAT or EL_SCHED_THREAD_MAPPED), lanes per
 * row for thread_mapped (else 0), and the estimated time in microseconds
 * (may be NULL).  Host only. */
el_status el_select_schedule(int64_t rows, int64_t cols, int64_t nnz,
                             int64_t max_row_nnz, int32_t* schedule,
                             int32_t* threads_per_row, double* est_us);
/* The cost model with all of el_row_stats: also weighs thread_mapped's
 * staged kernel (variant 1), where no row holds more than 27 nonzeros and
 * the coherence is at least 0.5.  Writes the schedule and, for
 * thread_mapped, opts->threads_per_row and opts->variant (other fields are
 * left alone).  Host only. */
el_status el_select_schedule_stats(int64_t rows, int64_t cols, int64_t nnz,
                                   const el_row_stats* stats, int32_t* schedule,
                                   el_spmv_opts* opts, double* est_us);
/* el_csr_row_stats + el_select_schedule_stats. */
el_status el_spmv_select(el_workspace* ws, const el_csr* A, int32_t* schedule,
                         el_spmv_opts* opts, el_stream_t stream);

/* C = A B.  B is row-major A->cols x n (leading dimension ldb >= n) of
 * b_dtype (FP32 / BF16 / FP16); C is row-major FP32 A->rows x n (ldc >= n).
 * Schedules: THREAD_MAPPED (the reference's), GROUP_MAPPED (a warp per
 * row, lanes across columns) and MERGE_PATH_FLAT. */
el_status el_spmm(el_workspace* ws, const el_csr* A, int32_t schedule,
                  const el_spmv_opts* opts, const void* B, int32_t b_dtype,
                  int64_t n, int64_t ldb, float* C, int64_t ldc,
                  el_stream_t stream);

/* Checks offsets[0] == 0, offsets monotone, offsets[rows] == nnz and every
 * index in [0, cols).  Synchronous.  *flags gets the EL_FLAG_* bits found;
 * returns EL_ERR_MALFORMED_CSR when any is set. */
el_status el_csr_validate(const el_csr* A, el_stream_t stream,
                          uint32_t* flags);

/* ---- partitions (exposed so split points can be checked bit for bit) --
 * Number of merge tiles of tpb * ipt items over rows + nnz items. */
int64_t el_merge_path_num_tiles(int64_t rows, int64_t nnz, int32_t tpb,
                                int32_t ipt);
/* Start coordinate (row, nonzero) of every merge tile plus the end of the
 * last one: 2 * (num_tiles + 1) uint32 in device memory. */
el_status el_merge_path_partition(const int32_t* offsets, int64_t rows,
                                  int64_t nnz, int32_t tpb, int32_t ipt,
                                  uint32_t* coords, el_stream_t stream);
/* For every tile and thread, the tile-local coordinate the thread starts
 * its items_per_thread steps from: 2 * num_tiles * tpb uint32. */
el_status el_merge_path_thread_coords(const int32_t* offsets, int64_t rows,
                                      int64_t nnz, int32_t tpb, int32_t ipt,
                                      uint32_t* coords, el_stream_t stream);
/* work_oriented even share over num_threads threads: per thread the start
 * and end coordinate, 4 * num_threads int64 (st.row, st.nz, en.row, en.nz). */
el_status el_work_oriented_partition(const int32_t* offsets, int64_t rows,
                                     int64_t nnz, int64_t num_threads,
                                     int64_t* coords, el_stream_t stream);

/* Testing only (no counterpart in the reference): while `ranges` is not
 * NULL, every launch of the default merge-path kernel (el_spmv with
 * EL_SCHED_MERGE_PATH_FLAT and variant 0, el_spmv_static_scratch) made from
 * the calling host thread writes, for each of its warp ranges g < capacity,
 * six int64 to ranges[6 g .. 6 g + 5]: the range's first and end merge
 * diagonal, then the (row, nonzero) coordinates the kernel itself computed
 * for them -- first row, first nonzero, end row, end nonzero.  With a row
 * weight of 1 these are the reference's merge-path split points
 * (util/search.hxx:34-60) at those diagonals.  `ranges` is device memory of
 * 6 * capacity int64; NULL switches the trace off. */
el_status el_debug_range_trace(int64_t* ranges, int64_t capacity);

/* ---- batched SpMV (no counterpart in the reference) --------------------
 * Thousands of independent CSR matrices, each with its own x and y, run in
 * ONE persistent launch that the plan captures in a CUDA graph.  A plan
 * computes row-length statistics of every matrix on the device, picks per
 * matrix a kernel mode (the nonzero-tiled warp walk of the merge-path
 * kernel, or 1..32 lanes per row) and a work-item size from a tuning table
 * indexed by (rows, mean row length, row-length variation) buckets, cuts
 * every matrix into work items of whole rows at merge-path diagonals (about
 * 2^chunk rows + nonzeros each) and keeps the work list on the device.
 * Matrices with a row longer than EL_BATCH_MAX_ROW_NNZ run as their own
 * merge-path launches inside the same graph.  All matrices of a plan share
 * one value dtype. */
typedef struct el_batch_item {
  el_csr A;
  const float* x;
  float* y;
} el_batch_item;

#define EL_BATCH_ROW_BUCKETS 21 /* floor(log2(rows)), clamped to [0, 20] */
#define EL_BATCH_LEN_BUCKETS 11 /* mean nnz/row: < 1, [1,2), [2,4), ... , >= 512 */
#define EL_BATCH_CV_BUCKETS 4   /* row-length std/mean: < .25, < .75, < 1.5, >= 1.5 */
#define EL_BATCH_TABLE_SIZE \
  (EL_BATCH_ROW_BUCKETS * EL_BATCH_LEN_BUCKETS * EL_BATCH_CV_BUCKETS)
/* table index = (row_bucket * EL_BATCH_LEN_BUCKETS + len_bucket) *
 * EL_BATCH_CV_BUCKETS + cv_bucket; entry = threads_per_row (1..32, or
 * EL_BATCH_NZ_WALK) | log2(rows + nonzeros per work item) << 8, or 0 for
 * the built-in rule (nonzero-tiled walk, 2^12). */
#define EL_BATCH_NZ_WALK 64
#define EL_BATCH_MAX_ROW_NNZ 16384

typedef struct el_batch_opts {
  const int32_t* table;          /* EL_BATCH_TABLE_SIZE entries or NULL */
  int32_t use_graph;             /* 1: capture in a CUDA graph (default 1 via
                                    el_batch_opts_default) */
  int32_t force_threads_per_row; /* > 0: this (1..32 or EL_BATCH_NZ_WALK) for
                                    every matrix (tuning) */
  int32_t force_chunk_log2;      /* > 0: this for every matrix (tuning) */
  int32_t max_ctas;              /* cap on the persistent grid (0 = resident) */
  int32_t reserved[8];
} el_batch_opts;

typedef struct el_batch_plan el_batch_plan;

void el_batch_opts_default(el_batch_opts* opts);
/* items: host array of `count` matrices.  Synchronises `stream` (it reads
 * the statistics back); the inputs must stay valid while the plan lives. */
el_status el_batch_plan_create(const el_batch_item* items, int32_t count,
                               const el_batch_opts* opts, el_stream_t stream,
                               el_batch_plan** out);
/* One y = A x for every matrix of the plan, asynchronous on `stream`. */
el_status el_batch_plan_execute(el_batch_plan* plan, el_stream_t stream);
/* Work items, matrices per kernel mode (tpr_counts[7]: 1,2,4,8,16,32 lanes
 * per row, nonzero-tiled walk) and matrices run as separate merge-path
 * launches. */
el_status el_batch_plan_info(const el_batch_plan* plan, int64_t* work_items,
                             int32_t* tpr_counts, int32_t* heavy);
/* Synchronises `stream` and returns (and optionally clears) the EL_FLAG_*
 * bits raised by the plan's kernels. */
el_status el_batch_plan_errors(el_batch_plan* plan, el_stream_t stream,
                               uint32_t* flags, int clear);
el_status el_batch_plan_destroy(el_batch_plan* plan);

/* ---- SpMV without device allocation (no counterpart in the reference) --
 * y = A x with the default merge-path kernel, for callers that may not
 * allocate device memory once they are running: processes whose device
 * memory is all reserved up front by their own allocator (inference
 * servers, frameworks with a caching allocator, where a cudaMalloc would
 * fail or bypass the budget), real-time loops that forbid allocation (and
 * the device-wide synchronisation cudaMalloc/cudaFree bring) after start-up,
 * and plugins hosted by an application that owns the device allocator.
 * Every other entry point may allocate a workspace on first use; this one
 * never calls cudaMalloc, cudaFree or any allocating routine.
 *
 * Its scratch (range tickets, error flags and one carry slot per warp
 * range) is a fixed array in the library's device image: 64 KiB + 64 B,
 * present on every GPU that loads the library until the process exits.
 * Each call looks the array's device address up (cudaGetSymbolAddress);
 * the first call on a device, and the first after a cudaDeviceReset, also
 * loads the library's device image there, so make that call before any
 * stream capture.  All calls on a device share the array: calls that may
 * overlap on the GPU (other streams, other host threads) race and give
 * wrong results; serialise them.  Each call clears the array's counters
 * and flags itself.
 *
 * num_ranges: warp ranges the work is split into, 0 = one per resident
 * warp (at most EL_STATIC_MAX_RANGES); a larger value is rejected with
 * EL_ERR_INVALID_ARGUMENT.  With flags != NULL the call synchronises
 * `stream`, stores the EL_FLAG_* bits the kernel raised and returns
 * EL_ERR_DEVICE if any is set; with flags == NULL it is asynchronous, and
 * the bits stay readable with el_spmv_static_scratch_errors until the next
 * call clears them.
 * Values FP32 / BF16 / FP16 with optional row scales; FP32 accumulation. */
#define EL_STATIC_MAX_RANGES 4096
el_status el_spmv_static_scratch(const el_csr* A, const float* x, float* y,
                                 int32_t num_ranges, uint32_t* flags,
                                 el_stream_t stream);
/* Synchronises `stream` and returns the EL_FLAG_* bits the last
 * el_spmv_static_scratch call on the current device raised (clearing them
 * when clear != 0).  Allocates nothing. */
el_status el_spmv_static_scratch_errors(el_stream_t stream, uint32_t* flags,
                                        int clear);

/* ---- mixed precision -------------------------------------------------- */
/* Converts FP32 values to BF16 / FP16 (round to nearest even).  With
 * row_scale != NULL, each row is first divided by a power of two chosen so
 * that the row's largest magnitude lands in [1, 2) for BF16 or in
 * [2^14, 2^15) for FP16 (the top of its range, so the row's small entries
 * stay clear of FP16 subnormals), and the power is written to
 * row_scale[row] (exact: dequantised = out * row_scale). */
el_status el_quantize_values(const int32_t* offsets, int64_t rows,
                             int64_t nnz, const float* values, int32_t dtype,
                             void* out_values, float* row_scale,
                             el_stream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* EDGE_LOOPS_H_ */
