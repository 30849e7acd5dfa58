// spmv_schedules.cuh -- the thread_mapped, group_mapped and work_oriented
// SpMV schedules for sm_103a.  All three overwrite y and are deterministic.
#pragma once

#include "el_internal.h"

namespace el {

struct BasicArgs {
  long long rows, cols, nnz;
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  WsHeader* hdr;
};

__device__ __forceinline__ void row_bounds(const BasicArgs& a, long long row,
                                           long long* b, long long* e) {
  long long lo = __ldg(a.offsets + row), hi = __ldg(a.offsets + row + 1);
  if (lo < 0 || hi > a.nnz || hi < lo) {
    raise_flag(a.hdr, EL_FLAG_OFFSETS, (unsigned)row);
    lo = lo < 0 ? 0 : (lo > a.nnz ? a.nnz : lo);
    hi = hi < lo ? lo : (hi > a.nnz ? a.nnz : hi);
  }
  *b = lo;
  *e = hi;
}

__device__ __forceinline__ float scaled(const BasicArgs& a, long long row,
                                        float v) {
  return a.row_scale ? v * __ldg(a.row_scale + row) : v;
}

// acc += the products of nonzeros b, b + S, b + 2S, ... < e, added in that
// order (each product rounded, then the sum: no fused multiply-add).  The
// nonzeros go in batches of W, software-pipelined: a batch's x gathers are
// in flight together with the next batch's index and value loads.  A column
// outside [0, cols) contributes 0, loads nothing and sets `bad` (the caller
// raises the flag once).
template <typename VT, int S, bool COMP, int W = 8>
__device__ __forceinline__ void accumulate(const BasicArgs& a, long long b, long long e,
                                           Acc<COMP>& acc, bool& bad) {
  if (b >= e) return;
  const VT* __restrict__ vals = reinterpret_cast<const VT*>(a.values);
  const unsigned long long cols = (unsigned long long)a.cols;
  int c[W];
  float v[W];
  unsigned in = 0;  // bit k: nonzero nz + k S is inside [b, e)
  long long nz = b;
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const bool t = nz + k * S < e;
    in |= (unsigned)t << k;
    c[k] = t ? __ldg(a.indices + nz + k * S) : 0;
    v[k] = t ? to_f32(vals[nz + k * S]) : 0.f;
  }
  for (;;) {
    float xv[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const bool t = (in >> k) & 1u;
      const bool ok = (unsigned)c[k] < cols;
      bad |= t && !ok;
      xv[k] = t && ok ? __ldg(a.x + c[k]) : 0.f;
      if (!ok) v[k] = 0.f;
    }
    const long long nn = nz + W * S;
    int c2[W];
    float v2[W];
    unsigned in2 = 0;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const bool t = nn + k * S < e;
      in2 |= (unsigned)t << k;
      c2[k] = t ? __ldg(a.indices + nn + k * S) : 0;
      v2[k] = t ? to_f32(vals[nn + k * S]) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < W; ++k)
      if ((in >> k) & 1u) acc.add(__fmul_rn(v[k], xv[k]));
    if (!in2) break;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      c[k] = c2[k];
      v[k] = v2[k];
    }
    in = in2;
    nz = nn;
  }
}

// ------------------------------------------------------------ thread_mapped
// The reference's thread_mapped / original schedule
// [include/loops/schedule/thread_mapped.hxx:147-160,
//  include/loops/algorithms/spmv/thread_mapped.cuh:26-55]: rows in a grid-
// stride loop, each summed in nonzero order.  TPR > 1 generalises it to
// TPR lanes per row (lane k takes nonzeros k, k+TPR, ...; lanes combine in
// a fixed xor tree).  With TPR == 1 every row is the reference CPU loop's
// exact sequence of FP32 roundings (no fused multiply-add).
template <typename VT, int TPR, bool COMP>
__global__ void __launch_bounds__(256, 5)
    thread_mapped_spmv_kernel(const BasicArgs a) {
  const int lane = threadIdx.x & 31;
  const int sub = lane % TPR;
  constexpr int RPW = 32 / TPR;  // rows per warp per step
  const long long warp_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp_id * RPW; base < a.rows; base += nwarps * RPW) {
    const long long row = base + lane / TPR;
    Acc<COMP> acc;
    if (row < a.rows) {
      long long b, e;
      row_bounds(a, row, &b, &e);
      bool bad = false;
      if (TPR == 1) {
        accumulate<VT, 1, COMP, 8>(a, b, e, acc, bad);
      } else {
        // a lane sees few nonzeros of a row: a plain strided loop
        const VT* __restrict__ vals = reinterpret_cast<const VT*>(a.values);
        for (long long nz = b + sub; nz < e; nz += TPR) {
          const int col = __ldg(a.indices + nz);
          const bool ok = (unsigned)col < (unsigned long long)a.cols;
          bad |= !ok;
          acc.add(ok ? __fmul_rn(to_f32(vals[nz]), __ldg(a.x + col)) : 0.f);
        }
      }
      if (bad) raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)row);
    }
#pragma unroll
    for (int d = TPR / 2; d > 0; d >>= 1) {
      Acc<COMP> o;
      o.set(__shfl_xor_sync(kFullMask, acc.s, d),
            __shfl_xor_sync(kFullMask, acc.comp(), d));
      if ((sub & d) == 0) {
        acc.add(o);
      } else {
        o.add(acc);
        acc = o;
      }
    }
    if (sub == 0 && row < a.rows) a.y[row] = scaled(a, row, acc.value());
  }
}

// ------------------------------------------------- thread_mapped, staged
// The same schedule and summation order as thread_mapped_spmv_kernel with
// one lane per row (y bit-identical to it), for matrices whose rows are
// short: read straight from the CSR arrays, lane l's index and value loads
// stride by its row length, so each load instruction touches 32 lines.
// Here a warp copies the indices and values of its chunk of 32 rows into
// shared memory with two bulk copies by the TMA engine (cp.async.bulk, one
// mbarrier per buffer, L2 evict-first; two buffers per warp: the next chunk
// is in flight while this one is summed), and each lane then walks its row
// from there.  The x gathers keep the row-aligned order
// (lane l reads x near row r0 + l), which on banded matrices puts a gather
// instruction's 32 addresses on one or two lines.  Warp gw takes chunks
// gw, gw + nw, gw + 2 nw, ... (nw warps in the grid).
//
// A chunk whose nonzeros do not fit a buffer of CAP (long rows), or whose
// offsets fail the range checks, is summed straight from global memory as
// the unstaged kernel does, in its turn.  Every chunk fits when no row holds
// more than kStagedMaxRow nonzeros, which is when el_spmv_select picks this
// kernel.  Requires indices and values 16-byte aligned (checked by the
// launcher).
template <typename VT>
struct TmStage {
  static constexpr int kCap = 880;   // nonzeros per buffer
  static constexpr int kWarps = 4;   // per CTA: 4 CTAs of FP32 buffers per SM
  static constexpr int kIdxBytes = kCap * 4;
  static constexpr int kValBytes = (kCap * (int)sizeof(VT) + 15) / 16 * 16;
  static constexpr int kBuf = kIdxBytes + kValBytes;
  static constexpr int kSmem = kWarps * 2 * kBuf;
  static constexpr int kValPerUnit = 16 / (int)sizeof(VT);
  static constexpr int kBatch = 16;  // nonzeros of a row gathered together
};
// 32 rows of this many nonzeros, their start rounded down to 16 bytes, fit.
constexpr int kStagedMaxRow = 27;
static_assert(((32 * kStagedMaxRow + 3 + 3) / 4) * 16 <= TmStage<float>::kIdxBytes, "cap");
static_assert(((32 * kStagedMaxRow + 7 + 7) / 8) * 16 <= TmStage<__nv_bfloat16>::kValBytes,
              "cap");

// A lane's row in one chunk: raw offsets (checked when staged) and its
// scale, loaded a chunk ahead.
struct TmRows {
  int lo, hi;
  float scale;
};

// One row summed straight from global memory (the unstaged kernel's walk).
template <typename VT, bool COMP>
__device__ __forceinline__ void tm_direct_row(const BasicArgs& a, long long row) {
  Acc<COMP> acc;
  bool bad = false;
  long long b, e;
  row_bounds(a, row, &b, &e);
  accumulate<VT, 1, COMP, 8>(a, b, e, acc, bad);
  if (bad) raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)row);
  a.y[row] = scaled(a, row, acc.value());
}

// Four resident CTAs per SM (the FP32 buffers' limit): the bound lets the
// compiler use up to 128 registers, which it spends on keeping a batch's
// loads in flight (on the stencil 144 against 162 µs with the registers
// left to its own heuristic).
template <typename VT, bool COMP>
__global__ void __launch_bounds__(32 * TmStage<VT>::kWarps, 4)
    thread_mapped_staged_kernel(const BasicArgs a) {
  using S = TmStage<VT>;
  constexpr int W = S::kBatch;
  extern __shared__ __align__(16) unsigned char tm_smem[];
  __shared__ __align__(8) uint64_t s_bar[S::kWarps][2];  // one per buffer
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned char* const wbase = tm_smem + (size_t)w * 2 * S::kBuf;
  uint64_t pol = 0;  // the matrix streams: evict first, x keeps its L2 lines
  uint32_t ph = 0;   // bit b: the parity of buffer b's next phase
  // A copy that has not landed within the wait limit: the warp stages
  // nothing more, sums the rest from global memory, and before it exits
  // waits (bounded again) for the buffers whose copies were still in flight.
  uint32_t pending = 0, pending_par = 0;  // bit b: buffer b, its parity
  if (lane == 0) {
    mbar_init(&s_bar[w][0], 1);
    mbar_init(&s_bar[w][1], 1);
    fence_mbar_init();
    pol = l2_policy_evict_first();
  }
  __syncwarp();
  const long long nchunks = (a.rows + 31) >> 5;
  const long long nw = (long long)gridDim.x * S::kWarps;
  long long q = (long long)blockIdx.x * S::kWarps + w;
  const VT* __restrict__ gvals = reinterpret_cast<const VT*>(a.values);

  auto load_rows = [&](long long qq) {
    TmRows r{0, 0, 1.f};
    const long long row = (qq << 5) + lane;
    if (qq < nchunks && row < a.rows) {
      r.lo = __ldg(a.offsets + row);
      r.hi = __ldg(a.offsets + row + 1);
      if (a.row_scale) r.scale = __ldg(a.row_scale + row);
    }
    return r;
  };
  // Chunk qq, ahead of its turn: staged into buffer `buf` (returns the
  // staged extent's start in indices, rounded down to 16 bytes) or left to
  // be summed from global memory (-1; also past the last chunk).
  auto stage = [&](long long qq, const TmRows& r, int buf) {
    int ai = -1;
    if (qq < nchunks && !pending) {
      const long long r0 = qq << 5;
      const int last = (int)((a.rows - r0 < 32 ? a.rows - r0 : 32) - 1);
      const bool mine = lane <= last;
      const int b0 = __shfl_sync(kFullMask, r.lo, 0);
      const int e0 = __shfl_sync(kFullMask, r.hi, last);
      const bool ok = !mine || (r.lo >= b0 && r.lo <= r.hi && r.hi <= e0);
      const int i0 = b0 & ~3;
      const int v0 = b0 & ~(S::kValPerUnit - 1);
      // copy units (16 bytes) of each array, checked against the buffers
      const long long ni = ((long long)e0 - i0 + 3) >> 2;
      const long long nv = ((long long)e0 - v0 + S::kValPerUnit - 1) / S::kValPerUnit;
      const bool fits = a.cols > 0 && b0 >= 0 && e0 <= a.nnz && b0 <= e0 &&
                        ni * 16 <= S::kIdxBytes && nv * 16 <= S::kValBytes;
      if (__all_sync(kFullMask, ok) && fits) {
        ai = i0;
        unsigned char* const dst = wbase + (size_t)buf * S::kBuf;
        // whole 16-byte units by bulk copies, the arrays' last partial
        // units (in the chunk that reaches their end) by plain loads
        const int* const gi = a.indices + i0;
        const int fi = (int)(ni < ((a.nnz - i0) >> 2) ? ni : ((a.nnz - i0) >> 2));
        const VT* const gv = gvals + v0;
        const long long vleft = (a.nnz - v0) / S::kValPerUnit;
        const int fv = (int)(nv < vleft ? nv : vleft);
        if (lane == 0) {
          uint64_t* const bar = &s_bar[w][buf];
          mbar_arrive_expect_tx(bar, 16u * (uint32_t)(fi + fv));
          if (fi) bulk_g2s(dst, gi, 16u * fi, bar, pol);
          if (fv) bulk_g2s(dst + S::kIdxBytes, gv, 16u * fv, bar, pol);
          for (long long el = i0 + 4LL * fi; el < e0; ++el)
            reinterpret_cast<int*>(dst)[el - i0] = __ldg(a.indices + el);
          for (long long el = v0 + (long long)S::kValPerUnit * fv; el < e0; ++el)
            reinterpret_cast<VT*>(dst + S::kIdxBytes)[el - v0] = gvals[el];
        }
      }
    }
    return ai;
  };

  TmRows cur = load_rows(q);
  int cst = stage(q, cur, 0);
  TmRows nxt = load_rows(q + nw);
  int buf = 0;
  for (; q < nchunks; q += nw) {
    const int nst = stage(q + nw, nxt, buf ^ 1);
    const TmRows nn = load_rows(q + 2 * nw);
    if (cst >= 0) {
      const uint32_t par = (ph >> buf) & 1u;
      if (!__all_sync(kFullMask, mbar_wait_bounded(&s_bar[w][buf], par, 2000000000ull))) {
        if (lane == 0) raise_flag(a.hdr, EL_FLAG_TIMEOUT, (unsigned)q);
        pending |= 1u << buf;
        pending_par |= par << buf;
        cst = -1;  // summed from global memory instead
      }
      ph ^= 1u << buf;
    }
    __syncwarp();
    const long long row = (q << 5) + lane;
    const bool has_row = row < a.rows;
    if (cst >= 0) {
      const unsigned char* const src = wbase + (size_t)buf * S::kBuf;
      const int av = cst & ~(S::kValPerUnit - 1);
      const int* __restrict__ si = reinterpret_cast<const int*>(src) + (cur.lo - cst);
      const VT* __restrict__ sv =
          reinterpret_cast<const VT*>(src + S::kIdxBytes) + (cur.lo - av);
      const int n = has_row ? cur.hi - cur.lo : 0;
      // Gathers use the column clamped to [0, cols); a row with a column out
      // of range is summed again by the unstaged walk, which skips those
      // nonzeros and raises the flag.
      const unsigned lastc = (unsigned)(a.cols - 1);
      unsigned cmax = 0;
      Acc<COMP> acc;
      int j0 = 0;
      // whole batches of W: no per-nonzero predicates
      for (; j0 + W <= n; j0 += W) {
        int c[W];
        float v[W], xv[W];
#pragma unroll
        for (int k = 0; k < W; ++k) {
          c[k] = si[j0 + k];
          v[k] = to_f32(sv[j0 + k]);
        }
#pragma unroll
        for (int k = 0; k < W; ++k) {
          cmax = max(cmax, (unsigned)c[k]);
          xv[k] = __ldg(a.x + min((unsigned)c[k], lastc));
        }
#pragma unroll
        for (int k = 0; k < W; ++k) acc.add(__fmul_rn(v[k], xv[k]));
      }
      // the rest, predicated per nonzero
      if (j0 < n) {
        int c[W];
        float v[W], xv[W];
#pragma unroll
        for (int k = 0; k < W; ++k) {
          const bool t = j0 + k < n;
          c[k] = t ? si[j0 + k] : 0;
          v[k] = t ? to_f32(sv[j0 + k]) : 0.f;
        }
#pragma unroll
        for (int k = 0; k < W; ++k) {
          cmax = max(cmax, (unsigned)c[k]);
          xv[k] = j0 + k < n ? __ldg(a.x + min((unsigned)c[k], lastc)) : 0.f;
        }
#pragma unroll
        for (int k = 0; k < W; ++k)
          if (j0 + k < n) acc.add(__fmul_rn(v[k], xv[k]));
      }
      if (has_row) {
        if (cmax > lastc)
          tm_direct_row<VT, COMP>(a, row);
        else
          a.y[row] = a.row_scale ? acc.value() * cur.scale : acc.value();
      }
    } else if (has_row) {
      tm_direct_row<VT, COMP>(a, row);
    }
    __syncwarp();  // the buffer is free before it is staged into again
    cur = nxt;
    nxt = nn;
    cst = nst;
    buf ^= 1;
  }
  for (int b = 0; b < 2; ++b)
    if ((pending >> b) & 1u)
      mbar_wait_bounded(&s_bar[w][b], (pending_par >> b) & 1u, 2000000000ull);
}

// ------------------------------------------------------------- group_mapped
// The reference's group_mapped schedule [include/loops/schedule/
// group_mapped.hxx:146-235, include/loops/algorithms/spmv/group_mapped.cuh:
// 26-60]: a group of GT threads owns GT consecutive rows (GT = 32 is the
// reference's warp_mapped, GT = block size its block_mapped); the group scans
// its rows' lengths and its threads stride over the group's nonzeros, each
// mapping its nonzero to a row by an upper bound in that scan.  Instead of
// one atomicAdd per nonzero, every chunk of GT nonzeros is reduced by a
// segmented scan and each row's chunk total is added once, in chunk order,
// to a shared-memory row accumulator.
template <typename VT, int GT, int TPB, bool COMP>
__global__ void __launch_bounds__(TPB)
    group_mapped_spmv_kernel(const BasicArgs a) {
  static_assert(GT == 32 || GT == TPB, "warp groups or one block group");
  constexpr int NG = TPB / GT;
  __shared__ int s_off[NG][GT + 1];
  __shared__ float s_acc[NG][GT];
  __shared__ float s_accc[NG][COMP ? GT : 1];
  __shared__ SegScratch<GT / 32> s_scan;
  const int grp = threadIdx.x / GT;
  const int t = threadIdx.x % GT;
  auto gsync = [&]() {
    if (GT == 32) __syncwarp(); else __syncthreads();
  };
  const long long ngroups = (a.rows + GT - 1) / GT;
  // block-uniform loop over groups
  for (long long g0 = (long long)blockIdx.x * NG; g0 < ngroups;
       g0 += (long long)gridDim.x * NG) {
    const long long g = g0 + grp;
    const long long r0 = g * GT;
    const int glen = g < ngroups ? (int)((a.rows - r0 < GT) ? a.rows - r0 : GT) : 0;
    for (int k = t; glen > 0 && k <= glen; k += GT) {
      long long v = __ldg(a.offsets + r0 + k);
      if (v < 0 || v > a.nnz) {
        raise_flag(a.hdr, EL_FLAG_OFFSETS, (unsigned)(r0 + k));
        v = v < 0 ? 0 : a.nnz;
      }
      s_off[grp][k] = (int)v;
    }
    s_acc[grp][t] = 0.f;
    if (COMP) s_accc[grp][t] = 0.f;
    gsync();
    const long long abeg = glen > 0 ? s_off[grp][0] : 0;
    long long aend = glen > 0 ? s_off[grp][glen] : 0;
    if (aend < abeg) aend = abeg;
    // group-uniform loop over chunks of GT nonzeros; each thread's index
    // and value for the next chunk load while this chunk's x gathers are
    // in flight
    const VT* __restrict__ vals = reinterpret_cast<const VT*>(a.values);
    bool bad = false;
    int cn = 0;
    float vn = 0.f;
    if (abeg + t < aend) {
      cn = __ldg(a.indices + abeg + t);
      vn = to_f32(vals[abeg + t]);
    }
    for (long long base = abeg; base < aend; base += GT) {
      const long long nz = base + t;
      const int c = cn;
      float v = vn;
      const bool ok = (unsigned)c < (unsigned long long)a.cols;
      const float xv = nz < aend && ok ? __ldg(a.x + c) : 0.f;
      if (nz + GT < aend) {
        cn = __ldg(a.indices + nz + GT);
        vn = to_f32(vals[nz + GT]);
      }
      SegVal<COMP> mine;
      int key = GT;  // sentinel for threads past the group's nonzeros
      mine.f = 1;
      bool tail = false;
      if (nz < aend) {
        int lo = 0, hi = glen + 1;  // upper_bound over s_off[0..glen]
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (nz < s_off[grp][mid]) hi = mid; else lo = mid + 1;
        }
        key = lo - 1;
        if (key < 0) key = 0;
        if (key > glen - 1) key = glen - 1;
        mine.f = (t == 0) || (nz == s_off[grp][key]);
        bad |= !ok;
        if (!ok) v = 0.f;
        mine.v.add(__fmul_rn(v, xv));
        tail = (t == GT - 1) || (nz + 1 == aend) || (nz + 1 >= s_off[grp][key + 1]);
      }
      SegVal<COMP> inc;
      if (GT == 32) {
        inc = warp_seg_scan<COMP>(mine);
      } else {
        SegVal<COMP> zero, tot;
        zero.f = 0;
        const SegVal<COMP> ex =
            block_seg_scan_excl<GT / 32, COMP>(mine, zero, &s_scan, 1, &tot);
        inc = seg_combine(ex, mine);
      }
      if (tail) {  // one tail per row per chunk: no two threads collide
        Acc<COMP> acc;
        acc.set(s_acc[grp][key], COMP ? s_accc[grp][key] : 0.f);
        acc.add(inc.v);
        s_acc[grp][key] = acc.s;
        if (COMP) s_accc[grp][key] = acc.comp();
      }
      gsync();
    }
    if (bad) raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)r0);
    gsync();
    if (t < glen) {
      Acc<COMP> acc;
      acc.set(s_acc[grp][t], COMP ? s_accc[grp][t] : 0.f);
      a.y[r0 + t] = scaled(a, r0 + t, acc.value());
    }
    gsync();
  }
}

// ------------------------------------------------------------ work_oriented
// The reference's work_oriented schedule [include/loops/schedule/
// work_oriented.hxx:141-195, include/loops/algorithms/spmv/work_oriented.cuh:
// 34-78]: num_threads threads each take an even share
// ceil((rows+nnz)/num_threads) of the merge path, found by two searches on
// the global row offsets, and walk it straight from global memory, complete
// rows first, then the partial last row.  The reference stores complete rows
// and atomically adds the partial one, which races with another block's store
// of the same row; here partial rows are stitched by a block-wide segmented
// scan and, across blocks, by the carry look-back of the merge-path kernel.
struct WoArgs {
  BasicArgs b;
  long long wpt;  // merge items per thread
  int num_blocks;
  unsigned long long wait_ns;
  WsView ws;
};

template <int NW>
struct WoCtl {
  int blk;
  unsigned epoch;
  int pend;
  float pend_s, pend_c;
  SegScratch<NW> scan;
};

template <typename VT, int TPB, bool COMP>
__global__ void __launch_bounds__(TPB)
    work_oriented_spmv_kernel(const WoArgs w) {
  const BasicArgs& a = w.b;
  __shared__ WoCtl<TPB / 32> ctl;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    ctl.blk = (int)atomicAdd(&w.ws.hdr->ticket, 1u);
    ctl.epoch = read_epoch(w.ws.hdr);
    ctl.pend = 0;
  }
  __syncthreads();
  const int blk = ctl.blk;
  const unsigned epoch = ctl.epoch;
  const unsigned tag = epoch_tag(epoch);
  const bool active = blk < w.num_blocks;
  const long long total = a.rows + a.nnz;
  const long long tid = (long long)blk * TPB + threadIdx.x;
  long long upper = active ? w.wpt * tid : total;
  if (upper > total) upper = total;
  long long lower = upper + w.wpt;
  if (lower > total) lower = total;
  auto row_end = [&](long long k) { return __ldg(a.offsets + 1 + k); };
  long long sx = seq_merge_search(row_end, a.rows, 0, a.nnz, upper);
  long long sy = upper - sx;
  if (sx > a.rows) sx = a.rows;
  long long ex = seq_merge_search(row_end, a.rows, 0, a.nnz, lower);
  long long ey = lower - ex;
  if (ex > a.rows) ex = a.rows;

  // The thread's nonzeros [sy, ey) are one contiguous run.  With short
  // rows they stream in software-pipelined batches of kW whatever the row
  // boundaries, and the ends of rows [sx, ex) come kE at a time into a
  // shift register, so short rows cost no round trip each.  Rows from ex on
  // do not end here (ex is the open row, finished by the carry).
  constexpr int kW = 8, kE = 8;
  const VT* __restrict__ vals = reinterpret_cast<const VT*>(a.values);
  const unsigned long long cols = (unsigned long long)a.cols;
  Acc<COMP> run, first_v;
  long long first_row = -1;
  bool bad = false, bad_off = false;
  long long row = sx;
  int ends[kE];  // ends[j] = end of row `row + j` (INT_MAX from row ex on)
  int left = 0;  // valid entries of ends
  int prev_end = (int)sy;
  auto refill = [&]() {
#pragma unroll
    for (int j = 0; j < kE; ++j) {
      const long long r = row + j;
      int e = r < ex ? __ldg(a.offsets + r + 1) : 0x7fffffff;
      if (r < ex && (e > ey || e < prev_end)) {  // malformed offsets: keep them monotone
        bad_off = true;
        e = e > ey ? (int)ey : prev_end;
      }
      if (r < ex) prev_end = e;
      ends[j] = e;
    }
    left = kE;
  };
  auto close_row = [&]() {
    if (first_row < 0) {
      first_row = row;
      first_v = run;
    } else {
      a.y[row] = scaled(a, row, run.value());
    }
    run = Acc<COMP>();
    ++row;
#pragma unroll
    for (int j = 0; j + 1 < kE; ++j) ends[j] = ends[j + 1];
    if (--left == 0) refill();
  };
  // Long rows (every lane of the warp averaging >= 12 nonzeros per row)
  // walk row by row, each row's nonzeros pipelined, the next row's end
  // fetched early; otherwise the nonzeros stream across rows as below.
  const bool rowwise = __all_sync(0xffffffffu, (ey - sy) >= 12 * (ex - sx));
  if (rowwise) {
    long long nz = sy;
    long long e_next = sx < ex ? __ldg(a.offsets + sx + 1) : 0;
    for (; row < ex; ++row) {
      long long e = e_next;
      if (row + 1 < ex) e_next = __ldg(a.offsets + row + 2);
      if (e > ey || e < nz) {
        bad_off = true;
        e = e > ey ? ey : nz;
      }
      accumulate<VT, 1, COMP>(a, nz, e, run, bad);
      nz = e;
      if (first_row < 0) {
        first_row = row;
        first_v = run;
      } else {
        a.y[row] = scaled(a, row, run.value());
      }
      run = Acc<COMP>();
    }
    if (nz < ey) accumulate<VT, 1, COMP>(a, nz, ey, run, bad);
  } else {
    refill();
    while (row < ex && ends[0] <= sy) close_row();  // rows that end before any nonzero
  }
  if (!rowwise && sy < ey) {
    int c[kW];
    float v[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) {
      const bool t = sy + k < ey;
      c[k] = t ? __ldg(a.indices + sy + k) : 0;
      v[k] = t ? to_f32(vals[sy + k]) : 0.f;
    }
    for (long long base = sy;; base += kW) {
      float p[kW];
#pragma unroll
      for (int k = 0; k < kW; ++k) {
        const bool t = base + k < ey;
        const bool ok = (unsigned)c[k] < cols;
        bad |= t && !ok;
        p[k] = t && ok ? __fmul_rn(v[k], __ldg(a.x + c[k])) : 0.f;
      }
      const long long nb = base + kW;
#pragma unroll
      for (int k = 0; k < kW; ++k) {
        const bool t = nb + k < ey;
        c[k] = t ? __ldg(a.indices + nb + k) : 0;
        v[k] = t ? to_f32(vals[nb + k]) : 0.f;
      }
      // rows ending in this batch: none, one (its end position by a
      // predicated select, one close per batch), or several
      const bool c1 = row < ex && ends[0] <= nb;
      const bool c2 = c1 && row + 1 < ex && ends[1] <= nb;
      if (!c2) {
        const int q = c1 ? (int)(ends[0] - base) - 1 : kW;  // the row ends after nonzero base + q
        Acc<COMP> closed;
#pragma unroll
        for (int k = 0; k < kW; ++k) {
          if (base + k < ey) run.add(p[k]);
          if (k == q) {
            closed = run;
            run = Acc<COMP>();
          }
        }
        if (c1) {
          const Acc<COMP> rest = run;
          run = closed;
          close_row();
          run = rest;
        }
      } else {
#pragma unroll
        for (int k = 0; k < kW; ++k) {
          if (base + k < ey) {
            run.add(p[k]);
            // rows that end right after this nonzero (and empty rows after them)
            while (row < ex && ends[0] <= base + k + 1) close_row();
          }
        }
      }
      if (nb >= ey) break;
    }
  }
  if (bad_off) raise_flag(a.hdr, EL_FLAG_OFFSETS, (unsigned)sx);
  if (bad) raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)sx);

  SegVal<COMP> mine, zero, tot;
  mine.f = first_row >= 0;
  mine.v = run;
  zero.f = 0;
  const SegVal<COMP> exs =
      block_seg_scan_excl<TPB / 32, COMP>(mine, zero, &ctl.scan, 1, &tot);
  // block range start = thread 0's start; does it begin inside a row?
  __shared__ long long s_bs[2];
  if (threadIdx.x == 0) {
    s_bs[0] = sx;
    s_bs[1] = sy;
  }
  __syncthreads();
  const long long rs = s_bs[0], ns = s_bs[1];
  const int off_rs = rs < a.rows ? __ldg(a.offsets + rs) : (int)a.nnz;
  const bool need_lb = active && ns > off_rs;
  if (first_row >= 0) {
    Acc<COMP> v = exs.v;
    v.add(first_v);
    if (need_lb && !exs.f && first_row == rs) {
      ctl.pend = 1;
      ctl.pend_s = v.s;
      ctl.pend_c = v.comp();
    } else {
      a.y[first_row] = scaled(a, first_row, v.value());
    }
  }
  // the block's last thread publishes the partial of its open row
  if (active && threadIdx.x == TPB - 1) {
    const long long re = ex, ne = ey;
    if (re < a.rows) {
      const long long off_re = __ldg(a.offsets + re);
      const long long lo = off_re > ns ? off_re : ns;
      if (ne > lo && blk < w.ws.nslots) {
        CarrySlot* sl = w.ws.slots + blk;
        sl->sum = tot.v.s;
        sl->comp = tot.v.comp();
        st_release_u32(&sl->flag, tag);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < 32 && ctl.pend) {
    const long long range_items = w.wpt * TPB;
    const long long gfirst = (rs + off_rs) / range_items;
    Acc<COMP> acc;
    bool ok = true;
    for (long long k = gfirst + lane; k < blk && k < w.ws.nslots; k += 32) {
      CarrySlot* sl = w.ws.slots + k;
      if (ld_acquire_u32(&sl->flag) != tag) {
        const uint64_t t0 = global_timer_ns();
        while (ld_acquire_u32(&sl->flag) != tag) {
          if (global_timer_ns() - t0 > w.wait_ns) {
            ok = false;
            break;
          }
          __nanosleep(100);
        }
      }
      if (!ok) break;
      Acc<COMP> v;
      v.set(__ldcg(&sl->sum), __ldcg(&sl->comp));
      acc.add(v);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      Acc<COMP> o;
      o.set(__shfl_xor_sync(kFullMask, acc.s, d),
            __shfl_xor_sync(kFullMask, acc.comp(), d));
      if ((lane & d) == 0) {
        acc.add(o);
      } else {
        o.add(acc);
        acc = o;
      }
    }
    ok = __all_sync(kFullMask, ok);
    if (lane == 0) {
      if (!ok) raise_flag(a.hdr, EL_FLAG_TIMEOUT, 5);
      Acc<COMP> p;
      p.set(ctl.pend_s, ctl.pend_c);
      acc.add(p);
      a.y[rs] = scaled(a, rs, acc.value());
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&w.ws.hdr->done, 1u);
    if (prev == gridDim.x - 1) finish_launch(w.ws.hdr, epoch);
  }
}

}  // namespace el
