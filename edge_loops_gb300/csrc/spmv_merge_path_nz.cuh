// spmv_merge_path_nz.cuh -- merge-path SpMV for sm_103a, nonzero-tiled warp
// variant (the default).
//
// The work split follows the reference's merge_path_flat schedule at the
// level of warp ranges [include/loops/schedule/merge_path_flat.hxx:108-138,
// util/search.hxx:34-60]: the merge of row ends and nonzeros is cut at
// global diagonals g * range_items, every warp taking one range (id from an
// atomic ticket, so a range only ever waits on ranges already running), so
// every warp gets the same number of rows + nonzeros.  Inside its range a
// warp walks TILES OF 32 KP NONZEROS (aligned to multiples of the tile),
// lane l owning the KP consecutive nonzeros KP l .. KP l + KP - 1 of the
// tile; KP = 8 (tiles of 256) by default, 16 (tiles of 512) for 16-bit
// values on long rows (nz_per_lane):
//
//   * a lane loads its KP column indices and KP values with 128-bit vector
//     loads straight into registers (the next tile's loads are issued while
//     the current tile reduces), gathers x and forms KP products;
//   * the rows that end inside the tile come from a window of row offsets
//     (one ballot per 32 rows) as a sorted list of end positions in shared
//     memory; a lane adds its products in order and closes a row whenever
//     an end position is reached (empty rows: several ends at one position);
//   * rows crossing lanes are stitched by a warp segmented scan, rows
//     crossing tiles by a register carry, rows crossing ranges by carries
//     that the range where the row ends collects (bounded spins, fixed
//     order: deterministic).  No CTA barrier anywhere.  y is overwritten.
#pragma once

#include "el_internal.h"

namespace el {
namespace mpn {

constexpr int kPer = 8;               // nonzeros per lane of the default tile (8 or 16)
constexpr int kTileNz = 32 * kPer;    // nonzeros per default tile; range lengths are
                                      // multiples of it whatever the tile
constexpr int kMaxEnds = 256;         // row ends per tile (tiles are cut short
                                      // after this many, e.g. empty rows)
// The tile of KP nonzeros per lane (KP = 8 or 16, chosen per call).
template <int KP>
struct Geom {
  static constexpr int log = KP == 16 ? 4 : 3;
  static constexpr int tile = 32 * KP;
  static constexpr int stage = tile > kMaxEnds ? tile : kMaxEnds;  // staging slots per warp
};
constexpr int kWarps = 8;
constexpr int kTPB = 32 * kWarps;

struct Args {
  long long rows, cols, nnz;
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  long long range_items;  // merge items per warp range
  long long num_ranges;
  int vec_ok;             // 128-bit loads allowed at tile starts (tile_phase)
  int ph;                 // tile phase (tile_phase)
  int rw;                 // merge items per row end (the ranges' split)
  int test_hooks;
  unsigned long long wait_ns;
  WsView ws;
  long long* trace;       // testing only: per range (d0, d1, rs, ns, re, ne), or nullptr
  long long trace_cap;    // ranges the trace holds
};

template <bool COMP, int KP = kPer>
struct __align__(16) WarpSmem {
  int re[kMaxEnds];                       // end position (tile-local nonzero index) of each row end
  float yv[Geom<KP>::stage];              // the tile's row sums (or, whole tiles, by end position)
  float yc[COMP ? Geom<KP>::stage : 4];
  unsigned char kp[32][KP];               // row end closed after lane l's product i (tile-local)
  unsigned mw[32];                        // whole tiles: bit i of word l = a row ends after
                                          // nonzero KP l + i
  int pend;
  float pend_s, pend_c;
};

// KP consecutive FP32 values (16-byte aligned: 128-bit loads).
template <int KP>
__device__ __forceinline__ void load8(const float* p, float (&v)[KP]) {
#pragma unroll
  for (int k = 0; k < KP / 4; ++k) {
    const float4 a = __ldcs(reinterpret_cast<const float4*>(p) + k);
    v[4 * k] = a.x; v[4 * k + 1] = a.y; v[4 * k + 2] = a.z; v[4 * k + 3] = a.w;
  }
}
template <int KP>
__device__ __forceinline__ void load8i(const int* p, int (&c)[KP]) {
#pragma unroll
  for (int k = 0; k < KP / 4; ++k) {
    const int4 a = __ldcs(reinterpret_cast<const int4*>(p) + k);
    c[4 * k] = a.x; c[4 * k + 1] = a.y; c[4 * k + 2] = a.z; c[4 * k + 3] = a.w;
  }
}

template <typename VT>
__device__ __forceinline__ float ld_val(const VT* p) {
  return to_f32(*p);
}

// A lane's 8 values of the tile in flight.  16-bit values stay packed as
// loaded (4 words) and are widened only when the products are formed, so no
// instruction waits on the load before then.
template <typename VT, int KP = kPer>
struct TileVals {
  float v[KP];
  __device__ __forceinline__ void load_vec(const float* p) { load8(p, v); }
  __device__ __forceinline__ void load_at(int i, const float* p) { v[i] = ld_val(p); }
  __device__ __forceinline__ void zero_at(int i) { v[i] = 0.f; }
  __device__ __forceinline__ float get(int i) const { return v[i]; }
};
template <typename H, int KP>
struct TileVals16 {
  uint32_t w[KP / 2];
  __device__ __forceinline__ void load_vec(const H* p) {
#pragma unroll
    for (int k = 0; k < KP / 8; ++k) {
      const uint4 u = __ldcs(reinterpret_cast<const uint4*>(p) + k);
      w[4 * k] = u.x; w[4 * k + 1] = u.y; w[4 * k + 2] = u.z; w[4 * k + 3] = u.w;
    }
  }
  __device__ __forceinline__ void put(int i, unsigned short h) {
    w[i >> 1] = (i & 1) ? ((w[i >> 1] & 0xffffu) | ((uint32_t)h << 16))
                        : ((w[i >> 1] & 0xffff0000u) | h);
  }
  __device__ __forceinline__ void load_at(int i, const H* p) {
    put(i, __ldcs(reinterpret_cast<const unsigned short*>(p)));
  }
  __device__ __forceinline__ void zero_at(int i) { put(i, 0); }
  __device__ __forceinline__ unsigned short half_at(int i) const {
    return (unsigned short)((i & 1) ? (w[i >> 1] >> 16) : (w[i >> 1] & 0xffffu));
  }
};
template <int KP>
struct TileVals<__nv_bfloat16, KP> : TileVals16<__nv_bfloat16, KP> {
  __device__ __forceinline__ float get(int i) const {
    return __uint_as_float((uint32_t)this->half_at(i) << 16);
  }
};
template <int KP>
struct TileVals<__half, KP> : TileVals16<__half, KP> {
  __device__ __forceinline__ float get(int i) const {
    return __half2float(__ushort_as_half(this->half_at(i)));
  }
};

// One matrix as the tile walk sees it.
struct Src {
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  int rows;
  unsigned cols;
  int nnz;
  int vec_ok;  // 128-bit loads allowed at tile starts
  int ph;      // tiles start where (nonzero index + ph) is a multiple of the tile size
};

// 128-bit loads of indices and values need both arrays at the same phase
// modulo 8 elements (indices 4-byte, values element-aligned); tiles then
// start on 32-byte boundaries of both.  Otherwise every load is scalar.
inline void tile_phase(const void* indices, const void* values, int vbytes, int* vec_ok,
                       int* ph, int tile = kTileNz) {
  const uintptr_t ia = (uintptr_t)indices, va = (uintptr_t)values;
  const bool ok = ia % 4 == 0 && va % (uintptr_t)vbytes == 0 &&
                  ((ia / 4) - (va / (uintptr_t)vbytes)) % 8 == 0;
  *vec_ok = ok ? 1 : 0;
  *ph = ok ? (int)((ia / 4) % (uintptr_t)tile) : 0;
}

// The warp walks the merge range from (rs, ns) to (re, ne): rows [rs, re)
// end inside it and are written to y (row rs only when it begins in the
// range, i.e. !need_lb; otherwise its partial is left in S.pend*), and the
// partial sum of the row still open at the end (row re's nonzeros [.., ne))
// is returned.  Sets bad / bad_col on malformed input; ra_out = the first
// row not closed.
template <typename VT, bool COMP, int KP = kPer>
__device__ __forceinline__ Acc<COMP> walk_rows(const Src& m, WarpSmem<COMP, KP>& S, const int lane,
                                               const int rs, const int re, const int ns,
                                               const int ne, const bool need_lb, bool& bad,
                                               bool& bad_col, int& ra_out) {
  constexpr int kPer = KP;  // this walk's tile: KP nonzeros per lane
  constexpr int kPerLog = Geom<KP>::log;
  constexpr int kTileNz = Geom<KP>::tile;
  const VT* vals = reinterpret_cast<const VT*>(m.values);
  const float* __restrict__ scale = m.row_scale;
  const int rows = m.rows;
  const unsigned cols = m.cols;

  // tile [lo, hi): nonzeros up to the next multiple of kTileNz (or ne)
  auto tile_hi = [&](int l) -> int {
    if (l >= ne) return l;
    const unsigned t = (((unsigned)l + m.ph) & ~(unsigned)(kTileNz - 1)) + kTileNz - m.ph;
    return t < (unsigned)ne ? (int)t : ne;
  };
  int c[kPer];
  TileVals<VT, KP> v;
  auto load_tile = [&](int l, int h) {
    const int j0 = l + kPer * lane;
    if (m.vec_ok && h - l == kTileNz && ((l + m.ph) & 7) == 0) {
      load8i(m.indices + j0, c);
      v.load_vec(vals + j0);
    } else {
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int j = j0 + i;
        if (j < h) {
          c[i] = __ldcs(m.indices + j);
          v.load_at(i, vals + j);
        } else {
          c[i] = -1;
          v.zero_at(i);
        }
      }
    }
  };
  auto load_ends = [&](int r) {  // offsets[r + 1 + lane]: end of row r + lane
    const int k = r + 1 + lane;
    return k <= rows ? __ldcs(m.offsets + k) : 0x7fffffff;
  };

  // x at the tile's columns, gathered one tile ahead (a column outside
  // [0, cols) reads nothing and raises the flag once per range)
  float xg[kPer];
  auto gather = [&]() {
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int col = c[i];
      xg[i] = 0.f;
      if ((unsigned)col < cols)
        xg[i] = __ldg(m.x + col);
      else if (col != -1)
        bad_col = true;
    }
  };

  S.mw[lane] = 0u;
  int ra = rs, lo = ns;  // first row not yet closed; first nonzero of the tile
  int hi = tile_hi(lo);
  load_tile(lo, hi);
  int o = load_ends(ra);
  // scales of rows ra + lane, fetched with the row-end window they belong to
  auto load_scales = [&](int r) {
    return scale && r + lane < rows ? __ldg(scale + r + lane) : 1.f;
  };
  float scn = load_scales(ra);
  int o2 = 0;          // ends of the next 32 rows, when the last tile predicts them
  bool has_o2 = false;
  gather();
  Acc<COMP> carry;

  while (lo < ne || ra < re) {
    // rows [ra, re) ending at or before hi, at most kMaxEnds of them: their
    // end positions in the tile (S.re; the first 32 also in el0)
    int X = 0, el0 = 0;
    bool rising = true;  // end positions strictly increasing (no empty rows)
    {
      int e = o;
      int prev = -1;
      for (int base = 0;;) {
        const bool in = (unsigned)(ra + base + lane) < (unsigned)re && e <= hi;
        const unsigned b = __ballot_sync(kFullMask, in);
        const int cnt = b == kFullMask ? 32 : __ffs(~b) - 1;
        const int el = (e <= hi ? max(e, lo) : hi) - lo;
        int pe = __shfl_up_sync(kFullMask, el, 1);
        if (lane == 0) pe = prev;
        if (lane < cnt) {
          if (base > 0) S.re[base + lane] = el;  // the first 32 stay in el0
          rising = rising && el > pe;
        }
        if (base == 0) el0 = el;
        X = base + cnt;
        if (cnt < 32 || X >= kMaxEnds) break;
        prev = __shfl_sync(kFullMask, el, 31);
        base += 32;
        const int k = ra + base + 1 + lane;
        e = base == 32 && has_o2 ? o2 : k <= rows ? __ldg(m.offsets + k) : 0x7fffffff;
      }
    }
    const bool fast = __all_sync(kFullMask, rising) && X < kMaxEnds && hi - lo == kTileNz;
    // row scales of the tile's first 32 rows (fetched with their row-end
    // window, a tile ahead), used by the store at the end of the tile
    const float sc0 = scn;
    if (!fast && lane < X) S.re[lane] = el0;
    __syncwarp();
    if (X >= kMaxEnds) hi = lo + S.re[kMaxEnds - 1];  // cut the tile at its 256th row end
    const int Y = hi - lo;
    if (X == 0 && Y == 0) {  // no progress possible: malformed offsets
      bad = true;
      break;
    }

    // products of this lane's nonzeros kPer lane + i
    float p[kPer];
    if (fast) {
#pragma unroll
      for (int i = 0; i < kPer; ++i) p[i] = __fmul_rn(v.get(i), xg[i]);
    } else {
#pragma unroll
      for (int i = 0; i < kPer; ++i) p[i] = kPer * lane + i < Y ? __fmul_rn(v.get(i), xg[i]) : 0.f;
    }
    // the window registers are free: start loading the next tile
    const int lo2 = hi, hi2 = tile_hi(hi), ra2 = ra + X;
    if (lo2 < ne) load_tile(lo2, hi2);
    if (ra2 < re) {
      o = load_ends(ra2);
      scn = load_scales(ra2);
    }
    // a tile with many row ends is likely followed by another: fetch the
    // second window too, so that its ballot does not wait on a dependent load
    has_o2 = X >= 24 && ra2 + 32 < re;
    if (has_o2) o2 = load_ends(ra2 + 32);

    if (fast) {
      // Whole tile, strictly increasing row ends.  A lane's close bits come
      // from a word per lane that the end positions are OR-ed into (bit i
      // of S.mw[l] = a row ends after nonzero 8 l + i); the lane's running
      // sums are staged by position
      // (its products since its previous close, up to nonzero q),
      // its tail is stitched by a segmented scan whose segment starts come
      // from one ballot, and row r's sum is read back at its end position.
      for (int kk = lane; kk < X; kk += 32) {
        const int P = kk < 32 ? el0 : S.re[kk];
        if (P > 0) atomicOr(&S.mw[(P - 1) >> kPerLog], 1u << ((P - 1) & (kPer - 1)));
      }
      __syncwarp();
      const unsigned mask = S.mw[lane];
      S.mw[lane] = 0u;  // only this lane reads it; the next tile writes it after a barrier
      Acc<COMP> run;
      float ss[kPer], sc[kPer];
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        run.add(p[i]);
        ss[i] = run.s;
        sc[i] = run.comp();
        if ((mask >> i) & 1u) run = Acc<COMP>();
      }
      // position q lives at S.yv[(q % kPer) * 32 + q / kPer]: conflict-free stores
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        S.yv[32 * i + lane] = ss[i];
        if (COMP) S.yc[32 * i + lane] = sc[i];
      }
      // a row closed at position 0 (before the tile's first nonzero) takes
      // the carry; otherwise the carry runs into the first lanes
      const bool z = X > 0 && __shfl_sync(kFullMask, el0, 0) == 0;
      const Acc<COMP> cin = z ? Acc<COMP>() : carry;
      const unsigned heads = __ballot_sync(kFullMask, mask != 0u);
      const unsigned upto = heads & (lane == 31 ? 0xffffffffu : (2u << lane) - 1u);
      const int dist = upto ? lane - (31 - __clz(upto)) : lane;  // lanes since my segment began
      Acc<COMP> inc = run;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        Acc<COMP> t = shfl_up_acc(inc, d);
        if (d <= dist) {
          t.add(inc);  // earlier lanes first
          inc = t;
        }
      }
      if (!upto) {
        Acc<COMP> t = cin;
        t.add(inc);
        inc = t;
      }
      Acc<COMP> ex = shfl_up_acc(inc, 1);
      if (lane == 0) ex = cin;
      const Acc<COMP> cout = shfl_idx_acc(inc, 31);
      if (mask) {  // the lane's first close: earlier parts of the row first
        const int f = 32 * (__ffs(mask) - 1) + lane;
        Acc<COMP> mine;
        mine.set(S.yv[f], COMP ? S.yc[f] : 0.f);
        ex.add(mine);
        S.yv[f] = ex.s;
        if (COMP) S.yc[f] = ex.comp();
      }
      __syncwarp();
      for (int kk = lane; kk < X; kk += 32) {  // coalesced store of the tile's rows
        const int P = kk < 32 ? el0 : S.re[kk];
        Acc<COMP> val = carry;
        const int q = 32 * ((P - 1) & (kPer - 1)) + ((P - 1) >> kPerLog);
        if (P > 0) val.set(S.yv[q], COMP ? S.yc[q] : 0.f);
        const int r = ra + kk;
        if (need_lb && r == rs) {
          // the range's first row end closes row rs, begun in an earlier
          // range: finished by the look-back
          S.pend = 1;
          S.pend_s = val.s;
          S.pend_c = val.comp();
          continue;
        }
        float vv = val.value();
        if (scale) vv *= kk < 32 ? sc0 : __ldg(scale + r);
        m.y[r] = vv;
      }
      carry = cout;
    } else {
      // this lane's row ends: end positions in (kPer lane, kPer lane + kPer] (lane 0:
      // also position 0, rows closed before any nonzero of the tile)
      int k = 0;
      if (lane > 0) {
        int lo_ = 0, hi_ = X;
        while (lo_ < hi_) {
          const int mid = (lo_ + hi_) >> 1;
          if (S.re[mid] <= kPer * lane) lo_ = mid + 1; else hi_ = mid;
        }
        k = lo_;
      }
      int kend = __shfl_down_sync(kFullMask, k, 1);
      if (lane == 31) kend = X;

      // rows of the tile start at 0 (an empty row stays 0); the lane's row
      // ends become "close after product i" bits (the first end at each
      // position closes the running sum, further ends there are empty rows)
      for (int kk = lane; kk < X; kk += 32) {
        S.yv[kk] = 0.f;
        if (COMP) S.yc[kk] = 0.f;
      }
      unsigned mask = 0;
      for (int kk = k; kk < kend; ++kk) {
        const int q = S.re[kk] - kPer * lane;
        if (q >= 1 && q <= kPer) {
          if (kk == k || S.re[kk - 1] != S.re[kk]) {
            mask |= 1u << (q - 1);
            S.kp[lane][q - 1] = (unsigned char)kk;
          }
        } else if (q != 0 || lane != 0) {
          bad = true;  // an end outside the lane's nonzeros: malformed offsets
        }
      }
      __syncwarp();
      Acc<COMP> run;
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        run.add(p[i]);
        if ((mask >> i) & 1u) {
          const int kk = S.kp[lane][i];
          S.yv[kk] = run.s;
          if (COMP) S.yc[kk] = run.comp();
          run = Acc<COMP>();
        }
      }
      const bool has_end = kend > k;  // the lane closes row ra + k first

      // stitch rows across lanes; lane 0 continues the previous tile's row
      SegVal<COMP> mine, cin;
      mine.f = has_end;
      mine.v = run;
      cin.f = 0;
      cin.v = carry;
      const SegVal<COMP> inc = warp_seg_scan<COMP>(mine);
      SegVal<COMP> ex;
      ex.f = __shfl_up_sync(kFullMask, inc.f, 1);
      ex.v = shfl_up_acc(inc.v, 1);
      ex = lane == 0 ? cin : seg_combine(cin, ex);
      if (has_end) {
        Acc<COMP> val = ex.v;  // earlier parts of the row first
        Acc<COMP> mine_part;
        mine_part.set(S.yv[k], COMP ? S.yc[k] : 0.f);
        val.add(mine_part);
        if (need_lb && ra + k == rs) {
          // the range's first row end closes row rs, begun in an earlier
          // range: finished by the look-back below
          S.pend = 1;
          S.pend_s = val.s;
          S.pend_c = val.comp();
        }
        S.yv[k] = val.s;
        if (COMP) S.yc[k] = val.comp();
      }
      __syncwarp();
      for (int kk = lane; kk < X; kk += 32) {  // coalesced store of the tile's rows
        const int r = ra + kk;
        if (need_lb && r == rs) continue;
        float vv = COMP ? __fadd_rn(S.yv[kk], S.yc[kk]) : S.yv[kk];
        if (scale) vv *= kk < 32 ? sc0 : __ldg(scale + r);
        m.y[r] = vv;
      }
      carry = shfl_idx_acc(seg_combine(cin, inc).v, 31);
    }

    ra = ra2;
    lo = lo2;
    hi = hi2;
    if (lo < ne) gather();  // the next tile's window has arrived by now
    __syncwarp();  // S.re and S.yv are rewritten by the next tile
  }
  ra_out = ra;
  return carry;
}

// The walk of this file as a policy of run_range.
template <int KP>
struct NzWalkK {
  template <typename VT, bool COMP, typename SmemT>
  static __device__ __forceinline__ Acc<COMP> walk(const Src& m, SmemT& S, int lane, int rs,
                                                   int re, int ns, int ne, bool need_lb,
                                                   bool& bad, bool& bad_col, int& ra) {
    return walk_rows<VT, COMP, KP>(m, S, lane, rs, re, ns, ne, need_lb, bad, bad_col, ra);
  }
};
using NzWalk = NzWalkK<kPer>;

// One warp's merge range, shared by the merge-path kernels: takes a range
// id from the ticket, finds its split points, walks it with `Walk`
// (rows ending inside are written), publishes the partial of the row left
// open at its end, and finishes the row it began with (begun in earlier
// ranges) by the look-back.  `SmemT` is the walk's per-warp shared memory
// (with the pend fields).  `warps_per_cta` warps share a CTA.
template <typename VT, bool COMP, typename Walk, typename SmemT>
__device__ __forceinline__ void run_range(const Args& a, SmemT& S, const int warps_per_cta) {
  const int lane = threadIdx.x & 31;
  WsHeader* hdr = a.ws.hdr;
  const float* __restrict__ scale = a.row_scale;

  // one ticket per CTA (its warps take ranges ticket * warps_per_cta + w):
  // a range only waits on ranges of CTAs that took their ticket earlier and
  // are therefore running.  Every CTA reads the epoch before its ticket, so
  // the CTA that takes the launch's last ticket knows that all of them hold
  // theirs and hands the workspace back for the next launch right away
  // (ticket to 0, epoch + 1) instead of a completion count at the end.
  __shared__ unsigned s_ticket[2];
  if (threadIdx.x == 0) {
    const unsigned ep = read_epoch(hdr);
    __threadfence();
    const unsigned t = atomicAdd(&hdr->ticket, 1u);
    if (t == gridDim.x - 1) {
      __threadfence();
      atomicExch(&hdr->ticket, 0u);
      atomicExch(&hdr->epoch, ep + 1u);
    }
    s_ticket[0] = t;
    s_ticket[1] = ep;
  }
  __syncthreads();
  const long long g = (long long)s_ticket[0] * warps_per_cta + (threadIdx.x >> 5);
  const unsigned epoch = s_ticket[1];
  const unsigned tag = epoch_tag(epoch);
  const long long w = a.rw;
  const long long total = w * a.rows + a.nnz;

  if (g < a.num_ranges) {
    // split points at diagonals g * range_items of the merge of row ends
    // (w items each) and nonzeros
    const long long dd0 = g * a.range_items;
    const long long d0 = dd0 < total ? dd0 : total;
    const long long d1 = dd0 + a.range_items < total ? dd0 + a.range_items : total;
    SplitPoint sa, sb;
    warp_merge_search2_w(a.offsets + 1, a.rows, a.nnz, d0, d1, w, sa, sb);
    auto nz_of = [&](long long d, const SplitPoint& sp) {  // the nonzero coordinate
      const long long n = d - w * sp.x;
      return (int)(sp.x < a.rows ? min(n, (long long)sp.end) : n);
    };
    const int rs = (int)sa.x;
    const int ns = nz_of(d0, sa);
    const int re = (int)sb.x;
    const int ne = nz_of(d1, sb);
    const int off_rs = sa.start;
    const bool need_lb = ns > off_rs;
    if (a.trace && g < a.trace_cap && lane < 6) {
      // the range's diagonals and split points exactly as the walk uses them
      const long long t6[6] = {d0, d1, rs, ns, re, ne};
      long long tv = t6[0];
#pragma unroll
      for (int k = 1; k < 6; ++k)
        if (lane == k) tv = t6[k];
      a.trace[6 * g + lane] = tv;
    }
    if (lane == 0) {
      S.pend = 0;
      if (g == 0 && off_rs != 0) raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, 0);
    }

    const Src m{a.offsets, a.indices,        a.values,      a.row_scale, a.x,  a.y,
                (int)a.rows, (unsigned)a.cols, (int)a.nnz, a.vec_ok,    a.ph};
    bool bad = false, bad_col = false;
    int ra = rs;
    const Acc<COMP> carry =
        Walk::template walk<VT, COMP>(m, S, lane, rs, re, ns, ne, need_lb, bad, bad_col, ra);
    if (__any_sync(kFullMask, bad_col) && lane == 0)
      raise_flag(hdr, EL_FLAG_INDEX_RANGE, (unsigned)ra);
    if (__any_sync(kFullMask, bad) && lane == 0) raise_flag(hdr, EL_FLAG_OFFSETS, (unsigned)ra);

    // range end (re, ne): publish the partial of the row still open, if this
    // range holds any of its nonzeros; exactly one later range reads it
    const int off_re = sb.start;
    if (lane == 0) {
      if ((long long)re == a.rows && (long long)off_re != a.nnz)
        raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, (unsigned)re);
      if (ne > max(off_re, ns) && g < a.ws.nslots && !(a.test_hooks & 1)) {
        CarrySlot* sl = a.ws.slots + g;
        sl->sum = carry.s;
        sl->comp = carry.comp();
        st_release_u32(&sl->flag, tag);
      }
    }
    __syncwarp();
    if (need_lb && S.pend) {
      // row rs began in range gfirst: sum the partials of ranges [gfirst, g)
      // in a fixed order
      const long long gfirst = (w * rs + off_rs) / a.range_items;
      Acc<COMP> acc;
      bool ok = true;
      for (long long kk = gfirst + lane; kk < g && kk < a.ws.nslots; kk += 32) {
        CarrySlot* sl = a.ws.slots + kk;
        if (ld_acquire_u32(&sl->flag) != tag) {
          const uint64_t t0 = global_timer_ns();
          while (ld_acquire_u32(&sl->flag) != tag) {
            if (global_timer_ns() - t0 > a.wait_ns) {
              ok = false;
              break;
            }
            __nanosleep(100);
          }
        }
        if (!ok) break;
        Acc<COMP> pv;
        pv.set(__ldcg(&sl->sum), __ldcg(&sl->comp));
        acc.add(pv);
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        Acc<COMP> ov = shfl_xor_acc(acc, d);
        if ((lane & d) == 0) {
          acc.add(ov);
        } else {
          ov.add(acc);
          acc = ov;
        }
      }
      ok = __all_sync(kFullMask, ok);
      if (lane == 0) {
        if (!ok) raise_flag(hdr, EL_FLAG_TIMEOUT, 4);
        Acc<COMP> pend;
        pend.set(S.pend_s, S.pend_c);
        acc.add(pend);
        float vv = acc.value();
        if (scale) vv *= __ldg(scale + rs);
        a.y[rs] = vv;
      }
    }
  }

}

template <typename VT, bool COMP, int KP = kPer>
__global__ void __launch_bounds__(kTPB, KP == 16 ? 2 : 3)
    merge_path_nz_kernel(const Args a) {
  __shared__ WarpSmem<COMP, KP> smem_all[kWarps];
  run_range<VT, COMP, NzWalkK<KP>>(a, smem_all[threadIdx.x >> 5], kWarps);
}

// Merge items per row end for the warp ranges: a row end costs the walk
// about as much as two nonzeros (its ballot, bit, staging and store), so
// ranges of short rows get fewer items.  Falls back to 1 where the weighted
// merge length would reach kMergeLimit.
constexpr int kDefaultRowWeight = 2;
inline int row_weight(const SpmvCall& c) {
  int w = c.o.row_weight > 0 ? c.o.row_weight : kDefaultRowWeight;
  if (w > 16) w = 16;
  if ((long long)w * c.A.rows + c.A.nnz >= kMergeLimit) w = 1;
  return w;
}

template <typename VT, bool COMP, int KP = kPer>
int resident_warps(int device) {
  const int per_sm =
      resident_ctas_per_sm((const void*)merge_path_nz_kernel<VT, COMP, KP>, kTPB, 0);
  return (per_sm > 0 ? per_sm : 1) * kWarps * device_info(device).sm_count;
}

// Nonzeros per lane of the tile walk: opts.nz_per_lane (8 or 16), else 16
// for 16-bit values on matrices with long rows (at least kLongRows nonzeros
// per row on average and at least 2^20 nonzeros), 8 otherwise.  A 512-nonzero
// tile halves the per-nonzero cost of the row-end ballot, scan and store,
// which binds 16-bit values on banded matrices, but its registers allow
// only two CTAs per SM, which costs more than it saves where the x gathers
// or short rows bind.
constexpr long long kLongRows = 24;
inline int nz_per_lane(const SpmvCall& c, int vbytes) {
  if (c.o.nz_per_lane == 8 || c.o.nz_per_lane == 16) return c.o.nz_per_lane;
  const bool long_rows = c.A.nnz >= kLongRows * c.A.rows && c.A.nnz >= (1LL << 20);
  return vbytes == 2 && long_rows ? 16 : 8;
}

template <typename VT, bool COMP, int KP>
el_status launch_kp(const SpmvCall& c);

template <typename VT, bool COMP>
el_status launch(const SpmvCall& c) {
  if (c.o.nz_per_lane != 0 && c.o.nz_per_lane != 8 && c.o.nz_per_lane != 16)
    return fail(EL_ERR_INVALID_ARGUMENT, "nz_per_lane must be 0, 8 or 16");
  return nz_per_lane(c, (int)sizeof(VT)) == 16 ? launch_kp<VT, COMP, 16>(c)
                                               : launch_kp<VT, COMP, 8>(c);
}

template <typename VT, bool COMP, int KP>
el_status launch_kp(const SpmvCall& c) {
  const int rw = row_weight(c);
  const long long total = (long long)rw * c.A.rows + c.A.nnz;
  // ranges of whole 256-item units, one per resident warp
  const long long units = (total + kTileNz - 1) / kTileNz;
  long long W = resident_warps<VT, COMP, KP>(c.device);
  if (c.o.max_ctas > 0 && (long long)c.o.max_ctas * kWarps < W) W = (long long)c.o.max_ctas * kWarps;
  if (W > units) W = units;
  if (W < 1) W = 1;
  const long long upr = (units + W - 1) / W;
  Args a;
  a.rows = c.A.rows;
  a.cols = c.A.cols;
  a.nnz = c.A.nnz;
  a.offsets = c.A.offsets;
  a.indices = c.A.indices;
  a.values = c.A.values;
  a.row_scale = c.A.row_scale;
  a.x = c.x;
  a.y = c.y;
  a.range_items = upr * kTileNz;
  a.num_ranges = (units + upr - 1) / upr;
  tile_phase(c.A.indices, c.A.values, (int)sizeof(VT), &a.vec_ok, &a.ph, Geom<KP>::tile);
  a.rw = rw;
  a.test_hooks = c.o.test_hooks;
  a.wait_ns = c.wait_ns;
  a.ws = c.ws;
  a.trace = c.trace;
  a.trace_cap = c.trace_cap;
  if (a.num_ranges > c.ws.nslots)
    return fail(EL_ERR_INVALID_ARGUMENT, "merge_path: workspace too small");
  const long long grid = (a.num_ranges + kWarps - 1) / kWarps;
  merge_path_nz_kernel<VT, COMP, KP><<<(unsigned)grid, kTPB, 0, c.stream>>>(a);
  return cuda_status(cudaGetLastError(), "merge_path launch");
}

template <typename VT, bool COMP>
long long slots_needed(const SpmvCall& c) {
  const long long a = resident_warps<VT, COMP, 8>(c.device);
  const long long b = resident_warps<VT, COMP, 16>(c.device);
  return a > b ? a : b;
}

}  // namespace mpn
}  // namespace el
