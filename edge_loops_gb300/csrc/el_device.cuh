// el_device.cuh -- device-side building blocks shared by every kernel:
// inline-PTX wrappers (mbarrier, 1-D bulk copies, acquire/release),
// the merge-path searches, FP32 accumulators and the block-wide segmented
// scan used to stitch partial row sums together.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/edge_loops.h"

namespace el {

constexpr unsigned kFullMask = 0xffffffffu;

// ---------------------------------------------------------------- workspace
// Device state of the persistent schedules.  A launch reads `epoch` when it
// starts and tags every carry it publishes with epoch_tag(epoch); readers
// accept only that tag, so carries left by any earlier launch are never
// mistaken for fresh ones.  The last CTA (or warp) of a launch resets the
// ticket and done counters and advances the epoch, all on the device, so a
// launch can be replayed from a CUDA graph without host-side bookkeeping.
struct WsHeader {
  unsigned int ticket;    // next range/tile id handed out
  unsigned int done;      // CTAs finished (the last one resets both)
  unsigned int errors;    // EL_FLAG_* bits, sticky until cleared
  unsigned int err_info;  // first offending index (diagnostics)
  unsigned int epoch;     // launches completed on this workspace
  unsigned int pad[11];
};
static_assert(sizeof(WsHeader) == 64, "header is one 64-byte line");

struct CarrySlot {  // one partial row sum handed to a later CTA
  float sum;
  float comp;
  unsigned int flag;  // == epoch_tag(epoch of the publishing launch)
  unsigned int pad;
};

// Never 0 (the value of a slot nobody ever published).
__device__ __forceinline__ unsigned epoch_tag(unsigned epoch) {
  return epoch + 1u == 0u ? 1u : epoch + 1u;
}

__device__ __forceinline__ unsigned read_epoch(const WsHeader* h) {
  return *reinterpret_cast<const volatile unsigned*>(&h->epoch);
}

// Called by the last CTA/warp of a launch: hand the counters back and
// advance the epoch for the next launch on this workspace.
__device__ __forceinline__ void finish_launch(WsHeader* h, unsigned epoch) {
  atomicExch(&h->ticket, 0u);
  atomicExch(&h->done, 0u);
  atomicExch(&h->epoch, epoch + 1u);
  __threadfence();
}

struct WsView {
  WsHeader* hdr;
  CarrySlot* slots;
  long long nslots;
};

__device__ __forceinline__ void raise_flag(WsHeader* h, unsigned flag,
                                           unsigned info = 0) {
  if ((atomicOr(&h->errors, flag) & flag) == 0) atomicExch(&h->err_info, info);
}

// ------------------------------------------------------------------- values
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

// FP32 accumulators.  Acc<false> is a plain sum; Acc<true> is Neumaier's
// compensated sum (per-element) with Knuth's two-sum when two partials meet.
template <bool COMP>
struct Acc;

template <>
struct Acc<false> {
  float s;
  __device__ __forceinline__ Acc() : s(0.f) {}
  __device__ __forceinline__ void add(float v) { s = __fadd_rn(s, v); }
  __device__ __forceinline__ void add(const Acc& o) { s = __fadd_rn(s, o.s); }
  __device__ __forceinline__ float value() const { return s; }
  __device__ __forceinline__ float comp() const { return 0.f; }
  __device__ __forceinline__ void set(float a, float) { s = a; }
};

template <>
struct Acc<true> {
  float s, c;
  __device__ __forceinline__ Acc() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(float v) {
    float t = __fadd_rn(s, v);
    if (fabsf(s) >= fabsf(v))
      c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, t), v));
    else
      c = __fadd_rn(c, __fadd_rn(__fsub_rn(v, t), s));
    s = t;
  }
  __device__ __forceinline__ void add(const Acc& o) {
    float t = __fadd_rn(s, o.s);  // two-sum (Knuth)
    float bb = __fsub_rn(t, s);
    float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(o.s, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(o.c, err));
  }
  __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
  __device__ __forceinline__ float comp() const { return c; }
  __device__ __forceinline__ void set(float a, float b) { s = a; c = b; }
};

// -------------------------------------------------------------------- PTX
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of `bar` with the given parity to complete, for at
// most limit_ns nanoseconds.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar,
                                                  uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

// L2 policy for data read exactly once (the matrix streams): evict first,
// so the gathered vector x keeps its place in L2.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;"
               : "=l"(p));
  return p;
}

// 1-D bulk copy global -> shared, completing on an mbarrier (transaction
// bytes).  dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar,
                                         uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes."
      "L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Named barrier over the first `nthreads` threads of the CTA (the consumer
// warps of a warp-specialised kernel; the producer warps never join it).
__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// The same barrier, also returning the OR of `v` over the participants.
__device__ __forceinline__ bool named_bar_or(int id, int nthreads, bool v) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.s32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.s32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((int)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}

// First k in [lo, hi) where pred(k) is false, pred being true on a prefix
// (else hi): 33-ary search by the whole warp, each round testing 32 evenly
// spaced candidates, so a range of 2048 takes three rounds.  All 32 lanes
// call it and get the same answer; the answer stays in [lo, hi] whatever
// pred returns.
template <typename Pred>
__device__ __forceinline__ int warp_lower_bound(int lo, int hi, const Pred& pred) {
  const int lane = threadIdx.x & 31;
  while (hi - lo > 32) {
    const int span = hi - lo;
    const int p = lo + ((lane + 1) * span) / 33;
    const int c = __popc(__ballot_sync(kFullMask, pred(p)));
    const int plo = __shfl_sync(kFullMask, p, c > 0 ? c - 1 : 0);
    const int phi = __shfl_sync(kFullMask, p, c < 32 ? c : 31);
    if (c > 0) lo = plo + 1;
    if (c < 32) hi = phi;
  }
  const int p = lo + lane;
  const bool t = (p < hi) && pred(p);
  return lo + __popc(__ballot_sync(kFullMask, t));
}

// ------------------------------------------------------------ merge path
// Merge of the row-end offsets (list a) with the nonzero indices (list b,
// a counting sequence) cut at a diagonal: the reference's
// search::_binary_search [include/loops/util/search.hxx:34-60] gives
// x = lower_bound over [max(diag-b_len,0), min(diag,a_len)) of
// "a[i] <= b[diag-i-1]", coordinate {min(x,a_len), diag-x}.  The first
// index where that predicate fails is unique, so any search order returns
// the same split point.

// Sequential lower bound with thrust::lower_bound's exact semantics (an
// empty or inverted range returns its first element).  a(k) reads list a;
// list b is b0, b0+1, ...  Returns x before the min(x, a_len) clamp.
template <typename AFn>
__device__ __forceinline__ long long seq_merge_search(const AFn& a,
                                                      long long a_len,
                                                      long long b0,
                                                      long long b_len,
                                                      long long diag) {
  long long first = diag - b_len;
  if (first < 0) first = 0;
  long long x_max = diag < a_len ? diag : a_len;
  long long len = x_max - first;
  while (len > 0) {
    long long half = len >> 1;
    long long mid = first + half;
    if (a(mid) <= (int)(b0 + (diag - mid - 1))) {
      first = mid + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

// Warp-cooperative 33-ary search of the same split point directly in
// global memory: each round the 32 lanes test 32 evenly spaced candidates,
// so 2^20 rows need 4 dependent rounds instead of 20.  row_end = offsets+1.
// Valid for diag <= rows + nnz.  All 32 lanes must call it; all return x.
__device__ __forceinline__ long long warp_merge_search(
    const int* __restrict__ row_end, long long rows, long long nnz,
    long long diag) {
  const int lane = threadIdx.x & 31;
  long long lo = diag - nnz;
  if (lo < 0) lo = 0;
  long long hi = diag < rows ? diag : rows;
  while (hi - lo > 32) {
    const long long span = hi - lo;
    const long long p = lo + ((long long)(lane + 1) * span) / 33;
    const bool t = __ldg(row_end + p) <= (int)(diag - p - 1);
    const int c = __popc(__ballot_sync(kFullMask, t));
    const long long plo = __shfl_sync(kFullMask, p, c > 0 ? c - 1 : 0);
    const long long phi = __shfl_sync(kFullMask, p, c < 32 ? c : 31);
    if (c > 0) lo = plo + 1;
    if (c < 32) hi = phi;
  }
  const long long p = lo + lane;
  const bool t = (p < hi) && (__ldg(row_end + p) <= (int)(diag - p - 1));
  return lo + __popc(__ballot_sync(kFullMask, t));
}

// The split with every row end counted as `w` merge items (w >= 1): rows i
// with offsets[i+1] + w (i + 1) <= diag are closed before diagonal diag, and
// the diagonal's nonzero coordinate is min(diag - w x, offsets[x+1]) for that
// count x (w = 1 is warp_merge_search).  Two such split points at once (diagonals da and db, rows w items
// each), with both searches' probes in flight together.  Also returns
// offsets[x] and offsets[x+1] of each split row x (row_end = offsets + 1;
// offsets[rows + 1] reads as nnz), taken from the final probes where they
// hold them.
struct SplitPoint {
  long long x;  // rows closed before the diagonal
  int start;    // offsets[x]
  int end;      // offsets[x + 1] (nnz for x == rows)
};
__device__ __forceinline__ void warp_merge_search2_w(const int* __restrict__ row_end,
                                                     long long rows, long long nnz,
                                                     long long da, long long db, long long w,
                                                     SplitPoint& A, SplitPoint& B) {
  const int lane = threadIdx.x & 31;
  long long lo[2], hi[2];
  const long long d[2] = {da, db};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    lo[k] = d[k] > nnz ? (d[k] - nnz) / w : 0;
    hi[k] = d[k] / w;
    if (lo[k] > rows) lo[k] = rows;
    if (hi[k] > rows) hi[k] = rows;
  }
  while (hi[0] - lo[0] > 32 || hi[1] - lo[1] > 32) {  // warp-uniform
    long long p[2];
    int v[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      p[k] = lo[k] + ((long long)(lane + 1) * (hi[k] - lo[k])) / 33;
      v[k] = hi[k] - lo[k] > 32 ? __ldg(row_end + p[k]) : 0;  // both loads before either use
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (hi[k] - lo[k] <= 32) continue;
      const bool t = (long long)v[k] <= d[k] - w * (p[k] + 1);
      const int c = __popc(__ballot_sync(kFullMask, t));
      const long long plo = __shfl_sync(kFullMask, p[k], c > 0 ? c - 1 : 0);
      const long long phi = __shfl_sync(kFullMask, p[k], c < 32 ? c : 31);
      if (c > 0) lo[k] = plo + 1;
      if (c < 32) hi[k] = phi;
    }
  }
  long long p[2];
  int v[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    p[k] = lo[k] + lane;
    v[k] = p[k] < hi[k] ? __ldg(row_end + p[k]) : 0;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    SplitPoint& S = k == 0 ? A : B;
    const bool t = p[k] < hi[k] && (long long)v[k] <= d[k] - w * (p[k] + 1);
    const int c = __popc(__ballot_sync(kFullMask, t));
    S.x = lo[k] + c;
    // offsets[x + 1] = row_end[x] was probed by lane c (if x < hi), offsets[x]
    // = row_end[x - 1] by lane c - 1 (if c > 0)
    const int ve = __shfl_sync(kFullMask, v[k], c < 32 ? c : 31);
    const int vs = __shfl_sync(kFullMask, v[k], c > 0 ? c - 1 : 0);
    S.end = (S.x < hi[k] && c < 32) ? ve : S.x < rows ? __ldg(row_end + S.x) : (int)nnz;
    S.start = c > 0 ? vs : S.x > 0 ? __ldg(row_end + S.x - 1) : __ldg(row_end - 1);
  }
}

// ------------------------------------------------------ segmented scan
// Operator of a segmented sum over items in order: (f1,v1) (+) (f2,v2) =
// (f1|f2, f2 ? v2 : v1+v2), where f marks an item that starts a new
// segment (merge path: a thread that closed at least one row).
template <bool COMP>
struct SegVal {
  int f;
  Acc<COMP> v;
};

template <bool COMP>
__device__ __forceinline__ SegVal<COMP> seg_combine(const SegVal<COMP>& a,
                                                    const SegVal<COMP>& b) {
  SegVal<COMP> r;
  r.f = a.f | b.f;
  if (b.f) {
    r.v = b.v;
  } else {
    r.v = a.v;
    r.v.add(b.v);
  }
  return r;
}

// Warp shuffles of an accumulator (the compensation term only when there
// is one).
__device__ __forceinline__ Acc<false> shfl_up_acc(const Acc<false>& a, int d) {
  Acc<false> r;
  r.s = __shfl_up_sync(kFullMask, a.s, d);
  return r;
}
__device__ __forceinline__ Acc<true> shfl_up_acc(const Acc<true>& a, int d) {
  Acc<true> r;
  r.set(__shfl_up_sync(kFullMask, a.s, d), __shfl_up_sync(kFullMask, a.c, d));
  return r;
}
__device__ __forceinline__ Acc<false> shfl_idx_acc(const Acc<false>& a, int src) {
  Acc<false> r;
  r.s = __shfl_sync(kFullMask, a.s, src);
  return r;
}
__device__ __forceinline__ Acc<true> shfl_idx_acc(const Acc<true>& a, int src) {
  Acc<true> r;
  r.set(__shfl_sync(kFullMask, a.s, src), __shfl_sync(kFullMask, a.c, src));
  return r;
}
__device__ __forceinline__ Acc<false> shfl_xor_acc(const Acc<false>& a, int m) {
  Acc<false> r;
  r.s = __shfl_xor_sync(kFullMask, a.s, m);
  return r;
}
__device__ __forceinline__ Acc<true> shfl_xor_acc(const Acc<true>& a, int m) {
  Acc<true> r;
  r.set(__shfl_xor_sync(kFullMask, a.s, m), __shfl_xor_sync(kFullMask, a.c, m));
  return r;
}

// Inclusive warp-level segmented scan.
template <bool COMP>
__device__ __forceinline__ SegVal<COMP> warp_seg_scan(SegVal<COMP> me) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    SegVal<COMP> o;
    o.f = __shfl_up_sync(kFullMask, me.f, d);
    o.v = shfl_up_acc(me.v, d);
    if (lane >= d) me = seg_combine(o, me);
  }
  return me;
}

// Scratch for the block-level scan (NW warps).
template <int NW>
struct SegScratch {
  int f[NW];
  float s[NW];
  float c[NW];
};

// Block-level segmented scan over the first NW*32 threads, all of which must
// call it (it uses named barrier `bar_id` over NW*32 threads).  `carry_in`
// is an item placed before thread 0.  Returns each thread's EXCLUSIVE scan
// value (carry_in (+) items before it) and, in *total, carry_in (+) all
// items (the same in every thread).
template <int NW, bool COMP>
__device__ __forceinline__ SegVal<COMP> block_seg_scan_excl(
    const SegVal<COMP>& mine, const SegVal<COMP>& carry_in,
    SegScratch<NW>* scratch, int bar_id, SegVal<COMP>* total) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  SegVal<COMP> inc = warp_seg_scan<COMP>(mine);
  if (lane == 31) {
    scratch->f[warp] = inc.f;
    scratch->s[warp] = inc.v.s;
    scratch->c[warp] = inc.v.comp();
  }
  if (NW > 1) named_bar_sync(bar_id, NW * 32); else __syncwarp();
  SegVal<COMP> pre = carry_in;  // carry_in (+) warps [0, warp)
  SegVal<COMP> tot = carry_in;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    SegVal<COMP> wv;
    wv.f = scratch->f[w];
    wv.v.set(scratch->s[w], scratch->c[w]);
    if (w < warp) pre = seg_combine(pre, wv);
    tot = seg_combine(tot, wv);
  }
  // exclusive within the warp: the inclusive value of lane-1
  SegVal<COMP> ex;
  ex.f = __shfl_up_sync(kFullMask, inc.f, 1);
  ex.v = shfl_up_acc(inc.v, 1);
  SegVal<COMP> out = (lane == 0) ? pre : seg_combine(pre, ex);
  *total = tot;
  return out;
}

}  // namespace el
