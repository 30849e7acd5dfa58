// spmv_merge_path_warp.cuh -- merge-path SpMV for sm_103a, warp-streaming
// variant (the default).
//
// Same split points as the reference's merge_path_flat schedule
// [include/loops/schedule/merge_path_flat.hxx:321-385,
//  include/loops/algorithms/spmv/merge_path_flat.cuh:38-83]: a tile of
// TILE = 32 * IPT merge items, lane t starting at the split point of local
// diagonal t * IPT.  Every warp is independent: it takes a contiguous RANGE
// of tiles (range id from an atomic ticket, so a range only ever waits on
// ranges that are already running), finds its start with one warp-
// cooperative 33-ary search, and walks the range tile by tile:
//
//   * the next tile's row offsets, column indices and values are loaded with
//     coalesced streaming loads (evict-first) into registers while the
//     current tile computes, so HBM latency overlaps work; with ~32 warps
//     per SM, every SM keeps tens of KB in flight;
//   * the tile end is one ballot over 32 row ends held one per lane
//     (p_k = k + offsets[r0+1+k] - n0 < TILE), and the lanes' split points
//     are scattered from the row ends into warp-private shared memory;
//   * products x[col] * value are formed once per nonzero, the walk and the
//     stitching of rows across lanes (warp segmented scan) and across tiles
//     (a register carry) need no CTA barrier;
//   * a row that crosses warp ranges is finished by the range where it
//     ends, from the carries earlier ranges publish (bounded spins, fixed
//     order: deterministic).  y is overwritten.
#pragma once

#include "el_internal.h"

namespace el {
namespace mpw {

constexpr int kWarps = 8;  // warps per CTA
constexpr int kTPB = 32 * kWarps;

struct Args {
  long long rows, cols, nnz;
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  long long range_items;  // merge items per warp range (multiple of the tile)
  long long num_ranges;
  unsigned long long wait_ns;
  int test_hooks;
  WsView ws;
};

template <int kTile>
struct WarpSmem {
  float prod[kTile];     // products of the tile's nonzeros
  int re[kTile + 1];     // tile-local row ends: offsets[r0+1+k] - n0
  int sx[33];            // first row of every lane
  int pend;
  float pend_s, pend_c;
};

template <typename VT>
__device__ __forceinline__ VT ld_stream(const VT* p);
template <>
__device__ __forceinline__ float ld_stream<float>(const float* p) {
  return __ldcs(p);
}
template <>
__device__ __forceinline__ __nv_bfloat16 ld_stream<__nv_bfloat16>(const __nv_bfloat16* p) {
  const unsigned short u = __ldcs(reinterpret_cast<const unsigned short*>(p));
  return __ushort_as_bfloat16(u);
}
template <>
__device__ __forceinline__ __half ld_stream<__half>(const __half* p) {
  const unsigned short u = __ldcs(reinterpret_cast<const unsigned short*>(p));
  return __ushort_as_half(u);
}

// IPT merge items per lane (tile = 32 * IPT); MINB resident CTAs per SM
// the register allocation must allow.
template <typename VT, int kIPT, bool COMP, int MINB>
__global__ void __launch_bounds__(kTPB, MINB)
    merge_path_warp_kernel(const Args a) {
  constexpr int kTile = 32 * kIPT;
  __shared__ WarpSmem<kTile> smem_all[kWarps];
  const int lane = threadIdx.x & 31;
  WarpSmem<kTile>& S = smem_all[threadIdx.x >> 5];
  WsHeader* hdr = a.ws.hdr;
  const VT* vals = reinterpret_cast<const VT*>(a.values);
  const float* __restrict__ scale = a.row_scale;
  const int rows = (int)a.rows, nnz = (int)a.nnz;

  unsigned tk = 0, ep = 0;
  if (lane == 0) {
    tk = atomicAdd(&hdr->ticket, 1u);
    ep = read_epoch(hdr);
  }
  const long long g = __shfl_sync(kFullMask, tk, 0);
  const unsigned epoch = __shfl_sync(kFullMask, ep, 0);
  const unsigned tag = epoch_tag(epoch);
  const long long total = a.rows + a.nnz;

  if (g < a.num_ranges) {
    const long long dd0 = g * a.range_items;
    const int d0 = (int)(dd0 < total ? dd0 : total);
    const int d1 = (int)(dd0 + a.range_items < total ? dd0 + a.range_items : total);
    const int rs = (int)warp_merge_search(a.offsets + 1, a.rows, a.nnz, d0);
    const int ns = d0 - rs;
    const int off_rs = __ldg(a.offsets + rs);
    const bool need_lb = ns > off_rs;
    if (lane == 0) S.pend = 0;
    if (g == 0 && off_rs != 0 && lane == 0) raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, 0);

    int r0 = rs, n0 = ns;
    Acc<COMP> carry;
    bool bad = false;

    // register window of the current tile: row end r0+1+lane, and the
    // nonzeros n0 + lane + 32 i
    int o_reg, c_reg[kIPT];
    VT v_reg[kIPT];
    auto load_window = [&](int r, int n, int& o, int (&cc)[kIPT], VT (&vv)[kIPT]) {
      const int k = r + 1 + lane;
      o = k <= rows ? __ldcs(a.offsets + k) : 0x7fffffff;
      if (n + kTile <= nnz) {  // whole window inside the arrays
        const int* ip = a.indices + n + lane;
        const VT* vp = vals + n + lane;
#pragma unroll
        for (int i = 0; i < kIPT; ++i) {
          cc[i] = __ldcs(ip + 32 * i);
          vv[i] = ld_stream<VT>(vp + 32 * i);
        }
      } else {
#pragma unroll
        for (int i = 0; i < kIPT; ++i) {
          const int e = n + lane + 32 * i;
          if (e < nnz) {
            cc[i] = __ldcs(a.indices + e);
            vv[i] = ld_stream<VT>(vals + e);
          } else {
            cc[i] = -1;
            vv[i] = VT(0.f);
          }
        }
      }
    };
    load_window(r0, n0, o_reg, c_reg, v_reg);

    while (r0 + n0 < d1) {
      const int D = min(kTile, d1 - (r0 + n0));
      const int a_need = min(D, rows - r0);
      const int b_need = min(D, nnz - n0);
      const int x_min = max(D - b_need, 0);
      // tile end: X = first k in [x_min, a_need) whose row end sits at merge
      // position >= D (for a valid CSR the positions only grow with k)
      int X;
      {
        const int k = lane;
        const bool pr = k < x_min || (k < a_need && k + (o_reg - n0) < D);
        if (k < a_need && k < kTile) S.re[k] = o_reg - n0;
        const unsigned b = __ballot_sync(kFullMask, pr);
        X = b == kFullMask ? 32 : __ffs(~b) - 1;
        // more than 32 row ends in this tile: continue in windows of 32
        for (int base = 32; X == base && base < a_need; base += 32) {
          const int kk = base + lane;
          int o = 0x7fffffff;
          if (kk < a_need) o = __ldg(a.offsets + r0 + 1 + kk);
          if (kk < a_need && kk < kTile) S.re[kk] = o - n0;
          const bool p2 = kk < x_min || (kk < a_need && kk + (o - n0) < D);
          const unsigned b2 = __ballot_sync(kFullMask, p2);
          X = base + (b2 == kFullMask ? 32 : __ffs(~b2) - 1);
        }
        X = min(max(X, x_min), a_need);
      }
      const int Y = D - X;


      // products of the tile's nonzeros (nonzero j of the tile is register
      // i = j / 32 of lane j % 32)
#pragma unroll
      for (int i = 0; i < kIPT; ++i) {
        const int j = lane + 32 * i;
        if (j < Y) {
          const int col = c_reg[i];
          float p = 0.f;
          if ((unsigned)col < (unsigned long long)a.cols)
            p = __fmul_rn(to_f32(v_reg[i]), __ldg(a.x + col));
          else
            raise_flag(hdr, EL_FLAG_INDEX_RANGE, (unsigned)(n0 + j));
          S.prod[j] = p;
        }
      }
      // the window registers are consumed: load the next tile's window into
      // them now, so the loads overlap this tile's split, walk and scan
      if (r0 + n0 + D < d1) load_window(r0 + X, n0 + Y, o_reg, c_reg, v_reg);
      __syncwarp();  // the row ends in S.re come from every lane
      // split points: lane t starts at row sx[t] = #{k : p_k < t * kIPT}
      for (int k = lane; k <= X; k += 32) {
        int hi = 31, lo = 0;
        if (k < X) hi = min(max(k + S.re[k], 0) / kIPT, 31);
        if (k > 0) lo = min(max(k - 1 + S.re[k - 1], 0) / kIPT, 31) + 1;
        for (int t = lo; t <= hi; ++t) S.sx[t] = k;
      }
      if (lane == 0) S.sx[32] = X;
      __syncwarp();

      // walk this lane's kIPT merge items
      Acc<COMP> run, first_v;
      int first_x = -1;
      {
        int x = min(S.sx[lane], lane * kIPT);
        const int xe = min(S.sx[lane + 1], X);
        int y = lane * kIPT - x;
        const int steps = D - lane * kIPT;
        // tile-local nonzero position where the lane's current row ends
        // (past the end: the lane has no row end left)
        int nre = x < xe ? min(S.re[x], Y) : 0x7fffffff;
#pragma unroll
        for (int i = 0; i < kIPT; ++i) {
          if (i < steps) {
            if (y >= nre) {
              if (first_x < 0) {
                first_x = x;
                first_v = run;
              } else {
                const int r = r0 + x;
                float v = run.value();
                if (scale) v *= __ldg(scale + r);
                a.y[r] = v;
              }
              run = Acc<COMP>();
              ++x;
              nre = x < xe ? min(S.re[x], Y) : 0x7fffffff;
            } else if (y < Y) {
              run.add(S.prod[y]);
              ++y;
            } else {
              bad = true;
            }
          }
        }
      }

      // stitch rows across lanes; lane 0 continues the previous tile's row
      SegVal<COMP> mine;
      mine.f = first_x >= 0;
      mine.v = run;
      const SegVal<COMP> inc = warp_seg_scan<COMP>(mine);
      SegVal<COMP> ex;
      ex.f = __shfl_up_sync(kFullMask, inc.f, 1);
      ex.v = shfl_up_acc(inc.v, 1);
      SegVal<COMP> cin;
      cin.f = 0;
      cin.v = carry;
      ex = lane == 0 ? cin : seg_combine(cin, ex);
      if (first_x >= 0) {
        Acc<COMP> v = ex.v;  // earlier parts of the row first
        v.add(first_v);
        if (need_lb && r0 + first_x == rs) {
          // the range's first row end closes row rs, begun in an earlier
          // range: finished by the look-back below
          S.pend = 1;
          S.pend_s = v.s;
          S.pend_c = v.comp();
        } else {
          const int r = r0 + first_x;
          float vv = v.value();
          if (scale) vv *= __ldg(scale + r);
          a.y[r] = vv;
        }
      }
      const SegVal<COMP> all = seg_combine(cin, inc);  // carry (+) lanes 0..lane
      carry = shfl_idx_acc(all.v, 31);

      r0 += X;
      n0 += Y;
      __syncwarp();  // shared scratch is reused by the next tile
    }
    if (__any_sync(kFullMask, bad) && lane == 0) raise_flag(hdr, EL_FLAG_OFFSETS, (unsigned)r0);

    // range end (r0, n0): publish the partial of the row still open, if this
    // range holds any of its nonzeros; exactly one later range reads it
    const int off_re = __ldg(a.offsets + r0);
    if (lane == 0) {
      if (r0 == rows && off_re != nnz) raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, (unsigned)r0);
      if (n0 > max(off_re, ns) && g < a.ws.nslots && !(a.test_hooks & 1)) {
        CarrySlot* sl = a.ws.slots + g;
        sl->sum = carry.s;
        sl->comp = carry.comp();
        st_release_u32(&sl->flag, tag);
      }
    }
    __syncwarp();
    if (need_lb && S.pend) {
      // the row rs began in range gfirst: sum the partials of ranges
      // [gfirst, g) in a fixed order
      const long long gfirst = ((long long)rs + off_rs) / a.range_items;
      Acc<COMP> acc;
      bool ok = true;
      for (long long k = gfirst + lane; k < g && k < a.ws.nslots; k += 32) {
        CarrySlot* sl = a.ws.slots + k;
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
        Acc<COMP> v;
        v.set(__ldcg(&sl->sum), __ldcg(&sl->comp));
        acc.add(v);
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        Acc<COMP> o = shfl_xor_acc(acc, d);
        if ((lane & d) == 0) {
          acc.add(o);
        } else {
          o.add(acc);
          acc = o;
        }
      }
      ok = __all_sync(kFullMask, ok);
      if (lane == 0) {
        if (!ok) raise_flag(hdr, EL_FLAG_TIMEOUT, 4);
        Acc<COMP> pend;
        pend.set(S.pend_s, S.pend_c);
        acc.add(pend);
        float v = acc.value();
        if (scale) v *= __ldg(scale + rs);
        a.y[rs] = v;
      }
    }
  }

  // the last warp to finish hands the workspace back for the next launch
  if (lane == 0) {
    __threadfence();
    const unsigned total_warps = gridDim.x * kWarps;
    const unsigned prev = atomicAdd(&hdr->done, 1u);
    if (prev == total_warps - 1) finish_launch(hdr, epoch);
  }
}

template <typename VT, int kIPT, bool COMP, int MINB>
int resident_warps(int device) {
  const int per_sm = resident_ctas_per_sm(
      (const void*)merge_path_warp_kernel<VT, kIPT, COMP, MINB>, kTPB, 0);
  return (per_sm > 0 ? per_sm : 1) * kWarps * device_info(device).sm_count;
}

template <typename VT, int kIPT, bool COMP, int MINB>
el_status launch(const SpmvCall& c) {
  constexpr int kTile = 32 * kIPT;
  const long long total = c.A.rows + c.A.nnz;
  const long long tiles = (total + kTile - 1) / kTile;
  long long W = resident_warps<VT, kIPT, COMP, MINB>(c.device);
  if (c.o.max_ctas > 0 && (long long)c.o.max_ctas * kWarps < W) W = (long long)c.o.max_ctas * kWarps;
  if (W > tiles) W = tiles;
  if (W < 1) W = 1;
  const long long tpr = (tiles + W - 1) / W;  // tiles per range
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
  a.range_items = tpr * kTile;
  a.num_ranges = (tiles + tpr - 1) / tpr;
  a.wait_ns = c.wait_ns;
  a.test_hooks = c.o.test_hooks;
  a.ws = c.ws;
  if (a.num_ranges > c.ws.nslots)
    return fail(EL_ERR_INVALID_ARGUMENT, "merge_path: workspace too small");
  const long long grid = (a.num_ranges + kWarps - 1) / kWarps;
  merge_path_warp_kernel<VT, kIPT, COMP, MINB><<<(unsigned)grid, kTPB, 0, c.stream>>>(a);
  return cuda_status(cudaGetLastError(), "merge_path launch");
}

template <typename VT, int kIPT, bool COMP, int MINB>
long long slots_needed(const SpmvCall& c) {
  return resident_warps<VT, kIPT, COMP, MINB>(c.device);
}

}  // namespace mpw
}  // namespace el
