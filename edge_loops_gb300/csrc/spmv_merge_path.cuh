// spmv_merge_path.cuh -- merge-path SpMV for sm_103a: persistent,
// warp-specialised, streaming.
//
// Behaviour follows the reference's merge_path_flat schedule
// [include/loops/schedule/merge_path_flat.hxx:244-436,
//  include/loops/algorithms/spmv/merge_path_flat.cuh:38-139]: the merge of
// the row-end offsets with the nonzero indices is cut into tiles of
// ITEMS = 256 * IPT merge items at global diagonals k * ITEMS, and thread t
// of a tile starts at the split point of local diagonal t * IPT (the split
// the reference finds with util/search.hxx:34-60).  What differs is how the
// tiles are fed, split and stitched:
//
//   * one CTA per resident slot takes a contiguous RANGE of tiles (its id
//     comes from an atomic ticket, so every range it may wait on is already
//     running); one warp-cooperative 33-ary search per range end replaces
//     the reference's two binary searches per tile;
//   * two producer warps stream the range's row offsets and its
//     (column, value) pairs into shared-memory rings with 1-D bulk copies
//     (cp.async.bulk, mbarrier completion, L2 evict-first), several tiles
//     ahead of the eight consumer warps;
//   * per tile, each consumer warp finds the tile end with a 33-ary search
//     in shared memory, and the threads' split points are SCATTERED from the
//     row ends (row end k at merge position p_k closes the rows of every
//     thread whose diagonal lies beyond p_k) instead of searched: the same
//     split points, without a binary search per thread;
//   * consumers gather x and form every product once, walk their IPT items
//     in shared memory and stitch rows that cross threads with a block-wide
//     segmented scan and rows that cross tiles through a register carry,
//     instead of one atomicAdd per nonzero (merge_path_flat.cuh:77);
//   * a row that crosses CTA ranges is finished by the range where it ends,
//     which sums the carries the earlier ranges publish (bounded spins, in a
//     fixed order: the result is deterministic).  y is overwritten.
#pragma once

#include "el_internal.h"

namespace el {
namespace mp {

template <int IPT_>
struct Cfg {
  static constexpr int IPT = IPT_;
  static constexpr int TPB_C = 256;          // consumer threads
  static constexpr int NW_C = TPB_C / 32;    // consumer warps
  static constexpr int TPB = TPB_C + 64;     // + offsets / nonzero producers
  static constexpr int ITEMS = TPB_C * IPT;  // merge items per tile
  static constexpr int LOG_C = 9;
  static constexpr int C = 1 << LOG_C;  // elements per ring chunk
  // A tile needs at most ITEMS+1 offsets and ITEMS nonzeros; starting
  // anywhere in a chunk they span at most ITEMS/C + 2 chunks.  The rest of
  // each ring is prefetch depth.
  static constexpr int K_O = (ITEMS + 4 + C - 1) / C + 2;
  static constexpr int K_N = ITEMS / C + 6;
  static constexpr int RING_O = K_O * C;
  static constexpr int RING_N = K_N * C;
  static constexpr int WARP_PO = NW_C;      // offsets producer warp
  static constexpr int WARP_PN = NW_C + 1;  // nonzero producer warp
};

struct Args {
  long long rows, cols, nnz;
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  long long range_items;  // merge items per CTA range (multiple of ITEMS)
  int num_ranges;
  int tma_o;  // offsets base 16-byte aligned: bulk copies allowed
  int tma_n;  // indices and values bases 16-byte aligned
  unsigned long long wait_ns;
  int test_hooks;
  WsView ws;
};

template <typename VT, int IPT>
struct Smem {
  using C_ = Cfg<IPT>;
  uint64_t full_o[C_::K_O];
  uint64_t empty_o[C_::K_O];
  uint64_t full_n[C_::K_N];
  uint64_t empty_n[C_::K_N];
  alignas(16) int ring_o[C_::RING_O];
  alignas(16) int ring_c[C_::RING_N];
  alignas(16) VT ring_v[C_::RING_N];
  alignas(16) float prod[2][C_::ITEMS];  // per tile parity
  int sx[2][C_::TPB_C + 1];              // first row of every thread
};

template <int NW>
struct Ctl {
  int rs, ns, re, ne;  // range start / end coordinate (row, nonzero)
  int g;               // range id
  unsigned epoch;
  int pend;
  float pend_s, pend_c;
  SegScratch<NW> scan;
};

__device__ __forceinline__ int wrap(int q, int ring) { return q >= ring ? q - ring : q; }

template <typename VT, int IPT, bool COMP>
__global__ void __launch_bounds__(Cfg<IPT>::TPB)
    merge_path_spmv_kernel(const Args a) {
  using C_ = Cfg<IPT>;
  constexpr int C = C_::C;
  constexpr int K_O = C_::K_O;
  constexpr int K_N = C_::K_N;
  constexpr int TPB_C = C_::TPB_C;
  constexpr int ITEMS = C_::ITEMS;
  constexpr int RING_O = C_::RING_O;
  constexpr int RING_N = C_::RING_N;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<VT, IPT>& S = *reinterpret_cast<Smem<VT, IPT>*>(smem_raw);
  __shared__ Ctl<C_::NW_C> ctl;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  WsHeader* hdr = a.ws.hdr;

  if (tid == 0) {
    ctl.g = (int)atomicAdd(&hdr->ticket, 1u);
    ctl.epoch = read_epoch(hdr);
    ctl.pend = 0;
    for (int i = 0; i < K_O; ++i) {
      mbar_init(&S.full_o[i], 1);
      mbar_init(&S.empty_o[i], C_::NW_C);
    }
    for (int i = 0; i < K_N; ++i) {
      mbar_init(&S.full_n[i], 1);
      mbar_init(&S.empty_n[i], C_::NW_C);
    }
    fence_mbar_init();
  }
  __syncthreads();
  const int g = ctl.g;
  const unsigned epoch = ctl.epoch;
  const unsigned tag = epoch_tag(epoch);
  const long long total = a.rows + a.nnz;
  const bool active = g < a.num_ranges;  // false only if the state was stale
  if (warp < 2) {
    long long diag = active ? (long long)(g + warp) * a.range_items : total;
    if (diag > total) diag = total;
    const long long xx = warp_merge_search(a.offsets + 1, a.rows, a.nnz, diag);
    if (lane == 0) {
      if (warp == 0) {
        ctl.rs = (int)xx;
        ctl.ns = (int)(diag - xx);
      } else {
        ctl.re = (int)xx;
        ctl.ne = (int)(diag - xx);
      }
    }
  }
  __syncthreads();
  if (!active && tid == 0) raise_flag(hdr, EL_FLAG_TIMEOUT, (unsigned)g);
  const int rs = ctl.rs, ns = ctl.ns, re = ctl.re, ne = ctl.ne;
  const int o_base = rs & ~3;  // 16-byte aligned element index
  const int n_base = ns & ~7;  // 16-byte aligned for 2- and 4-byte values

  if (warp == C_::WARP_PO) {
    // ------------------------------------------- producer: row offsets
    const int o_end = active ? re + 1 : o_base;  // elements [o_base, re]
    const int nch = (o_end - o_base + C - 1) / C;
    const uint64_t pol = l2_policy_evict_first();
    int c = 0;
    bool ok = true;
    for (; c < nch; ++c) {
      const int slot = c % K_O;
      if (c >= K_O) {
        bool w = true;
        if (lane == 0)
          w = mbar_wait_bounded(&S.empty_o[slot], (uint32_t)(((c / K_O) - 1) & 1), a.wait_ns);
        if (!__shfl_sync(kFullMask, (int)w, 0)) {
          ok = false;
          break;
        }
      }
      const int e0 = o_base + c * C;
      const int e1 = min(e0 + C, o_end);
      int* dst = S.ring_o + slot * C;
      int eb = e0;  // [e0, eb) by bulk copy, [eb, e1) by plain loads
      if (a.tma_o) {
        const int up = (e1 + 3) & ~3;
        eb = ((long long)up <= a.rows + 1) ? up : (e1 & ~3);
      }
      for (int e = eb + lane; e < e1; e += 32) dst[e - e0] = __ldg(a.offsets + e);
      __syncwarp();
      if (lane == 0) {
        if (eb > e0) {
          const uint32_t bytes = (uint32_t)(eb - e0) * 4u;
          mbar_arrive_expect_tx(&S.full_o[slot], bytes);
          bulk_g2s(dst, a.offsets + e0, bytes, &S.full_o[slot], pol);
        } else {
          mbar_arrive(&S.full_o[slot]);
        }
      }
    }
    if (lane == 0) {
      if (!ok) raise_flag(hdr, EL_FLAG_TIMEOUT, 1);
      // no bulk copy may still be landing in shared memory when we leave
      for (int s = 0; s < K_O; ++s)
        if (s < c) {
          const int last = s + ((c - 1 - s) / K_O) * K_O;
          mbar_wait_bounded(&S.full_o[s], (uint32_t)((last / K_O) & 1), a.wait_ns);
        }
    }
  } else if (warp == C_::WARP_PN) {
    // --------------------------------- producer: (column, value) pairs
    const int nch = (active && ne > ns) ? (ne - n_base + C - 1) / C : 0;
    const uint64_t pol = l2_policy_evict_first();
    const VT* vals = reinterpret_cast<const VT*>(a.values);
    int c = 0;
    bool ok = true;
    for (; c < nch; ++c) {
      const int slot = c % K_N;
      if (c >= K_N) {
        bool w = true;
        if (lane == 0)
          w = mbar_wait_bounded(&S.empty_n[slot], (uint32_t)(((c / K_N) - 1) & 1), a.wait_ns);
        if (!__shfl_sync(kFullMask, (int)w, 0)) {
          ok = false;
          break;
        }
      }
      const int e0 = n_base + c * C;
      const int e1 = min(e0 + C, ne);
      int* dc = S.ring_c + slot * C;
      VT* dv = S.ring_v + slot * C;
      int eb = e0;
      if (a.tma_n) {
        const int up = (e1 + 7) & ~7;
        eb = ((long long)up <= a.nnz) ? up : (e1 & ~7);
      }
      for (int e = eb + lane; e < e1; e += 32) {
        dc[e - e0] = __ldg(a.indices + e);
        dv[e - e0] = vals[e];
      }
      __syncwarp();
      if (lane == 0) {
        if (eb > e0) {
          const uint32_t bc = (uint32_t)(eb - e0) * 4u;
          const uint32_t bv = (uint32_t)(eb - e0) * (uint32_t)sizeof(VT);
          mbar_arrive_expect_tx(&S.full_n[slot], bc + bv);
          bulk_g2s(dc, a.indices + e0, bc, &S.full_n[slot], pol);
          bulk_g2s(dv, vals + e0, bv, &S.full_n[slot], pol);
        } else {
          mbar_arrive(&S.full_n[slot]);
        }
      }
    }
    if (lane == 0) {
      if (!ok) raise_flag(hdr, EL_FLAG_TIMEOUT, 2);
      for (int s = 0; s < K_N; ++s)
        if (s < c) {
          const int last = s + ((c - 1 - s) / K_N) * K_N;
          mbar_wait_bounded(&S.full_n[s], (uint32_t)((last / K_N) & 1), a.wait_ns);
        }
    }
  } else {
    // ------------------------------------------------------- consumers
    const float* __restrict__ scale = a.row_scale;
    int o_ready = 0, n_ready = 0, o_rel = 0, n_rel = 0;  // chunk counters
    int r0 = rs, n0 = ns;
    int po = rs - o_base;  // ring position of offsets[r0]
    int pn = ns - n_base;  // ring position of nonzero n0
    const int d_end = active ? re + ne : rs + ns;
    Acc<COMP> carry;  // partial of row r0 carried in from the previous tile
    bool need_lb = false;  // the range starts inside a row begun earlier
    int off_rs = 0;
    bool bad = false;
    bool first_tile = true;
    int buf = 0;

    while (r0 + n0 < d_end) {
      const int D = min(ITEMS, d_end - (r0 + n0));
      const int a_need = min(D, re - r0);  // row ends that may fall in the tile
      const int b_need = min(D, ne - n0);
      // every consumer thread waits for the offsets [r0, r0 + a_need]
      bool late = false;
      {
        const int co = (r0 + a_need - o_base) >> C_::LOG_C;
        for (; o_ready <= co; ++o_ready)
          if (!mbar_wait_bounded(&S.full_o[o_ready % K_O], (uint32_t)((o_ready / K_O) & 1),
                                 a.wait_ns))
            late = true;
      }
      // offsets[r0 + 1 + k] from the ring
      auto row_end = [&](int k) { return S.ring_o[wrap(po + 1 + k, RING_O)]; };
      if (first_tile) {
        off_rs = S.ring_o[po];
        need_lb = ns > off_rs;
      }
      // tile end: X row ends among the next D items.  Row end k sits at merge
      // position p_k = k + row_end(k) - n0; X = first k with p_k >= D.
      const int x_min = max(D - b_need, 0);
      const int X =
          warp_lower_bound(x_min, a_need, [&](int k) { return k + row_end(k) - n0 < D; });
      const int Y = D - X;
      {
        const int cn = Y > 0 ? (n0 + Y - 1 - n_base) >> C_::LOG_C : -1;
        for (; n_ready <= cn; ++n_ready)
          if (!mbar_wait_bounded(&S.full_n[n_ready % K_N], (uint32_t)((n_ready / K_N) & 1),
                                 a.wait_ns))
            late = true;
      }
      // products of the tile's nonzeros: one gather of x each
      float* prod = S.prod[buf];
      for (int j = tid; j < Y; j += TPB_C) {
        const int q = wrap(pn + j, RING_N);
        const int col = S.ring_c[q];
        float p = 0.f;
        if ((unsigned)col < (unsigned long long)a.cols)
          p = __fmul_rn(to_f32(S.ring_v[q]), __ldg(a.x + col));
        else
          raise_flag(hdr, EL_FLAG_INDEX_RANGE, (unsigned)(n0 + j));
        prod[j] = p;
      }
      // split points: thread t starts at row sx[t] = #{k : p_k < t * IPT}
      int* sx = S.sx[buf];
      for (int k = tid; k <= X; k += TPB_C) {
        int hi = TPB_C - 1, lo = 0;
        if (k < X) hi = min(max(k + row_end(k) - n0, 0) / IPT, TPB_C - 1);
        if (k > 0) lo = min(max(k - 1 + row_end(k - 1) - n0, 0) / IPT, TPB_C - 1) + 1;
        for (int t = lo; t <= hi; ++t) sx[t] = k;
      }
      if (tid == 0) sx[TPB_C] = X;
      if (named_bar_or(2, TPB_C, late)) {  // uniform: every thread sees it
        if (tid == 0) raise_flag(hdr, EL_FLAG_TIMEOUT, 3);
        break;
      }

      // walk this thread's IPT merge items
      Acc<COMP> run;
      int first_x = -1;
      Acc<COMP> first_v;
      {
        // x <= tid * IPT and xe <= X hold for every valid CSR; the clamps
        // keep a malformed one inside the tile's arrays
        int x = min(sx[tid], tid * IPT);
        const int xe = min(sx[tid + 1], X);
        int y = tid * IPT - x;
        const int steps = D - tid * IPT;
#pragma unroll
        for (int i = 0; i < IPT; ++i) {
          if (i < steps) {
            const bool rowend = x < xe && (y >= Y || n0 + y >= row_end(x));
            if (rowend) {
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
            } else if (y < Y) {
              run.add(prod[y]);
              ++y;
            } else {
              bad = true;
            }
          }
        }
      }

      // stitch rows across threads (and the carry from the previous tile)
      SegVal<COMP> mine, cin, tot;
      mine.f = first_x >= 0;
      mine.v = run;
      cin.f = 0;
      cin.v = carry;
      const SegVal<COMP> ex =
          block_seg_scan_excl<C_::NW_C, COMP>(mine, cin, &ctl.scan, 1, &tot);
      if (first_x >= 0) {
        Acc<COMP> v = ex.v;  // earlier parts of the row first
        v.add(first_v);
        if (need_lb && r0 + first_x == rs) {
          // the range's first row end closes row rs, begun in an earlier
          // range: finished by the look-back below
          ctl.pend = 1;
          ctl.pend_s = v.s;
          ctl.pend_c = v.comp();
        } else {
          const int r = r0 + first_x;
          float vv = v.value();
          if (scale) vv *= __ldg(scale + r);
          a.y[r] = vv;
        }
      }
      carry = tot.v;

      // hand fully consumed chunks back to the producers (one arrival per
      // warp: a chunk is refilled once all consumer warps are done with it)
      const int r1 = r0 + X, n1 = n0 + Y;
      const int orel = (r1 - o_base) >> C_::LOG_C;
      const int nrel = (n1 - n_base) >> C_::LOG_C;
      __syncwarp();
      if (lane == 0) {
        for (int c = o_rel; c < orel; ++c) mbar_arrive(&S.empty_o[c % K_O]);
        for (int c = n_rel; c < nrel; ++c) mbar_arrive(&S.empty_n[c % K_N]);
      }
      o_rel = max(o_rel, orel);
      n_rel = max(n_rel, nrel);
      po = wrap(po + X, RING_O);
      pn = wrap(pn + Y, RING_N);
      r0 = r1;
      n0 = n1;
      buf ^= 1;
      first_tile = false;
    }
    if (bad) raise_flag(hdr, EL_FLAG_OFFSETS, (unsigned)r0);
    // every consumer has left the tile loop (and written ctl.pend) before
    // the end-of-range work reads it
    named_bar_sync(1, TPB_C);

    if (active && r0 + n0 >= d_end) {
      if (tid == 0) {
        const int off_re = S.ring_o[po];  // offsets[re]
        if (g == 0 && off_rs != 0) raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, 0);
        if ((long long)re == a.rows && (long long)off_re != a.nnz)
          raise_flag(hdr, EL_FLAG_NNZ_MISMATCH, (unsigned)re);
        // publish the partial of the row still open at the range end, if
        // this range holds any of its nonzeros; exactly one later range
        // (the one where the row ends) reads it
        const int lo = max(off_re, ns);
        if (ne > lo && g < a.ws.nslots && !(a.test_hooks & 1)) {
          CarrySlot* sl = a.ws.slots + g;
          sl->sum = carry.s;
          sl->comp = carry.comp();
          st_release_u32(&sl->flag, tag);
        }
      }
      if (warp == 0 && need_lb && ctl.pend) {
        // the row rs began in range gfirst: sum the partials of ranges
        // [gfirst, g) in a fixed order (each published with this launch's
        // tag; exactly this range reads them)
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
          if (!ok) raise_flag(hdr, EL_FLAG_TIMEOUT, 4);
          Acc<COMP> pend;
          pend.set(ctl.pend_s, ctl.pend_c);
          acc.add(pend);
          float v = acc.value();
          if (scale) v *= __ldg(scale + rs);
          a.y[rs] = v;
        }
      }
    }
  }

  // the last CTA to finish hands the workspace back for the next launch
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&hdr->done, 1u);
    if (prev == gridDim.x - 1) finish_launch(hdr, epoch);
  }
}

// Per device: raise the kernel's dynamic shared memory limit once and
// return how many CTAs of it fit on one SM.
template <typename VT, int IPT, bool COMP>
int prepare(int device, el_status* st) {
  using C_ = Cfg<IPT>;
  auto kern = merge_path_spmv_kernel<VT, IPT, COMP>;
  const size_t smem = sizeof(Smem<VT, IPT>);
  static int attr_done[64] = {0};
  *st = EL_OK;
  if (device >= 0 && device < 64 && !attr_done[device]) {
    cudaError_t e = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      *st = cuda_status(e, "merge_path smem attribute");
      return 0;
    }
    attr_done[device] = 1;
  }
  return resident_ctas_per_sm((const void*)kern, C_::TPB, smem);
}

// Host launcher for one value type / tile size / accumulation mode.
template <typename VT, int IPT, bool COMP>
el_status launch(const SpmvCall& c) {
  using C_ = Cfg<IPT>;
  auto kern = merge_path_spmv_kernel<VT, IPT, COMP>;
  const size_t smem = sizeof(Smem<VT, IPT>);
  el_status st;
  const int per_sm = prepare<VT, IPT, COMP>(c.device, &st);
  if (st != EL_OK) return st;
  if (per_sm < 1) return fail(EL_ERR_CUDA, "merge_path: kernel does not fit on an SM");
  const long long total = c.A.rows + c.A.nnz;
  const long long tiles = (total + C_::ITEMS - 1) / C_::ITEMS;
  long long G = (long long)per_sm * device_info(c.device).sm_count;
  if (c.o.max_ctas > 0 && c.o.max_ctas < G) G = c.o.max_ctas;
  if (G > tiles) G = tiles;
  if (G < 1) G = 1;
  const long long tpc = (tiles + G - 1) / G;
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
  a.range_items = tpc * C_::ITEMS;
  a.num_ranges = (int)((tiles + tpc - 1) / tpc);
  a.tma_o = ((uintptr_t)c.A.offsets % 16) == 0;
  a.tma_n = ((uintptr_t)c.A.indices % 16) == 0 && ((uintptr_t)c.A.values % 16) == 0;
  a.wait_ns = c.wait_ns;
  a.test_hooks = c.o.test_hooks;
  a.ws = c.ws;
  if (a.num_ranges > c.ws.nslots)
    return fail(EL_ERR_INVALID_ARGUMENT, "merge_path: workspace too small");
  kern<<<a.num_ranges, C_::TPB, smem, c.stream>>>(a);
  return cuda_status(cudaGetLastError(), "merge_path launch");
}

// Upper bound of the carry slots `launch` may use (one per resident CTA).
template <typename VT, int IPT, bool COMP>
long long slots_needed(const SpmvCall& c) {
  el_status st;
  const int per_sm = prepare<VT, IPT, COMP>(c.device, &st);
  return (long long)(per_sm > 0 ? per_sm : 1) * device_info(c.device).sm_count;
}

}  // namespace mp
}  // namespace el
