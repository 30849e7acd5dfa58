// spmv_impl.cuh -- per-value-type launchers of the four SpMV schedules.
// Included once per value type (spmv_f32.cu, spmv_bf16.cu, spmv_f16.cu) so
// the heavy template instantiations compile in parallel.
#pragma once

#include "spmv_merge_path.cuh"
#include "spmv_merge_path_nz.cuh"
#include "spmv_merge_path_warp.cuh"
#include "spmv_schedules.cuh"

namespace el {

template <typename VT>
struct SpmvImpl {
  static el_status merge_path(const SpmvCall& c) {
    const int ipt = c.o.items_per_thread;
    const bool comp = c.o.compensated != 0;
    if (c.o.variant == 0)
      return comp ? mpn::launch<VT, true>(c) : mpn::launch<VT, false>(c);
    if (c.o.variant == 2) {
      if (ipt >= 12)
        return comp ? mpw::launch<VT, 16, true, 2>(c) : mpw::launch<VT, 16, false, 3>(c);
      return comp ? mpw::launch<VT, 8, true, 4>(c) : mpw::launch<VT, 8, false, 5>(c);
    }
    if (c.o.variant != 1)
      return fail(EL_ERR_INVALID_ARGUMENT, "merge_path variant must be 0, 1 or 2");
    if (ipt > 0 && ipt <= 4)
      return comp ? mp::launch<VT, 4, true>(c) : mp::launch<VT, 4, false>(c);
    return comp ? mp::launch<VT, 8, true>(c) : mp::launch<VT, 8, false>(c);
  }
  static long long merge_path_slots(const SpmvCall& c) {
    const int ipt = c.o.items_per_thread;
    const bool comp = c.o.compensated != 0;
    if (c.o.variant == 0)
      return comp ? mpn::slots_needed<VT, true>(c) : mpn::slots_needed<VT, false>(c);
    if (c.o.variant == 2) {
      if (ipt >= 12)
        return comp ? mpw::slots_needed<VT, 16, true, 2>(c)
                    : mpw::slots_needed<VT, 16, false, 3>(c);
      return comp ? mpw::slots_needed<VT, 8, true, 4>(c) : mpw::slots_needed<VT, 8, false, 5>(c);
    }
    if (ipt > 0 && ipt <= 4)
      return comp ? mp::slots_needed<VT, 4, true>(c) : mp::slots_needed<VT, 4, false>(c);
    return comp ? mp::slots_needed<VT, 8, true>(c) : mp::slots_needed<VT, 8, false>(c);
  }

  static BasicArgs basic(const SpmvCall& c) {
    BasicArgs a;
    a.rows = c.A.rows;
    a.cols = c.A.cols;
    a.nnz = c.A.nnz;
    a.offsets = c.A.offsets;
    a.indices = c.A.indices;
    a.values = c.A.values;
    a.row_scale = c.A.row_scale;
    a.x = c.x;
    a.y = c.y;
    a.hdr = c.ws.hdr;
    return a;
  }

  static constexpr long long kTmCtasPerSm = 64;
  template <int TPR, bool COMP>
  static el_status tm(const SpmvCall& c) {
    // one lane group per row, up to a cap (opts.max_ctas, else
    // kTmCtasPerSm CTAs per SM): past it the lane groups stride over rows
    const int tpb = 256;
    long long grid = (c.A.rows * TPR + tpb - 1) / tpb;
    const long long cap = c.o.max_ctas > 0
                              ? (long long)c.o.max_ctas
                              : (long long)device_info(c.device).sm_count * kTmCtasPerSm;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    thread_mapped_spmv_kernel<VT, TPR, COMP><<<(unsigned)grid, tpb, 0, c.stream>>>(basic(c));
    return cuda_status(cudaGetLastError(), "thread_mapped launch");
  }
  // One lane per row, rows staged through shared memory (indices and values
  // 16-byte aligned): a grid of every resident CTA at most, each warp
  // striding over chunks of 32 rows.
  template <bool COMP>
  static el_status tm_staged(const SpmvCall& c) {
    using S = TmStage<VT>;
    auto kern = thread_mapped_staged_kernel<VT, COMP>;
    static int attr_done[64] = {0};
    if (c.device >= 0 && c.device < 64 && !attr_done[c.device]) {
      cudaError_t e =
          cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
      if (e != cudaSuccess) return cuda_status(e, "thread_mapped smem attribute");
      attr_done[c.device] = 1;
    }
    const int per_sm = resident_ctas_per_sm((const void*)kern, 32 * S::kWarps, S::kSmem);
    if (per_sm < 1) return fail(EL_ERR_CUDA, "thread_mapped: staged kernel does not fit on an SM");
    const long long chunks = (c.A.rows + 31) / 32;
    long long grid = (chunks + S::kWarps - 1) / S::kWarps;
    const long long cap = c.o.max_ctas > 0 ? (long long)c.o.max_ctas
                                           : (long long)device_info(c.device).sm_count * per_sm;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, 32 * S::kWarps, S::kSmem, c.stream>>>(basic(c));
    return cuda_status(cudaGetLastError(), "thread_mapped launch");
  }
  template <bool COMP>
  static el_status tm_tpr(const SpmvCall& c) {
    if (c.o.variant != 0 && c.o.variant != 1)
      return fail(EL_ERR_INVALID_ARGUMENT, "thread_mapped variant must be 0 or 1");
    // variant 1: one lane per row, rows staged through shared memory
    const bool aligned = ((uintptr_t)c.A.indices % 16 == 0) && ((uintptr_t)c.A.values % 16 == 0);
    if (c.o.variant == 1 && c.o.threads_per_row <= 1 && aligned) return tm_staged<COMP>(c);
    switch (c.o.threads_per_row) {
      case 0:
      case 1: return tm<1, COMP>(c);
      case 2: return tm<2, COMP>(c);
      case 4: return tm<4, COMP>(c);
      case 8: return tm<8, COMP>(c);
      case 16: return tm<16, COMP>(c);
      case 32: return tm<32, COMP>(c);
    }
    return fail(EL_ERR_INVALID_ARGUMENT, "threads_per_row must be 1,2,4,8,16 or 32");
  }
  static el_status thread_mapped(const SpmvCall& c) {
    return c.o.compensated ? tm_tpr<true>(c) : tm_tpr<false>(c);
  }

  template <int GT, int TPB, bool COMP>
  static el_status gm(const SpmvCall& c) {
    constexpr int NG = TPB / GT;
    const long long groups = (c.A.rows + GT - 1) / GT;
    long long grid = (groups + NG - 1) / NG;
    const long long cap = (long long)device_info(c.device).sm_count * 32;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    group_mapped_spmv_kernel<VT, GT, TPB, COMP><<<(unsigned)grid, TPB, 0, c.stream>>>(basic(c));
    return cuda_status(cudaGetLastError(), "group_mapped launch");
  }
  template <bool COMP>
  static el_status gm_cfg(const SpmvCall& c) {
    const int tpb = c.o.threads_per_block > 0 ? c.o.threads_per_block : 128;
    const int rows = c.o.group_rows > 0 ? c.o.group_rows : tpb;
    if (rows == 32) return gm<32, 256, COMP>(c);
    if (rows == 128 && tpb == 128) return gm<128, 128, COMP>(c);
    if (rows == 256 && tpb == 256) return gm<256, 256, COMP>(c);
    return fail(EL_ERR_INVALID_ARGUMENT,
                "group_mapped: group_rows 32 (warp groups) or == threads_per_block "
                "in {128, 256}");
  }
  static el_status group_mapped(const SpmvCall& c) {
    return c.o.compensated ? gm_cfg<true>(c) : gm_cfg<false>(c);
  }

  static constexpr int kWoTpb = 128;
  static constexpr long long kWoShare = 256;    // merge items per thread aimed at
  static constexpr long long kWoMinShare = 32;  // merge items per thread, at least
  static constexpr int kWoBlocksPerSm = 16;     // at most this many blocks per SM
  static long long wo_num_threads(const SpmvCall& c) {
    if (c.o.num_threads > 0) return c.o.num_threads;
    // The reference launches 2 x SM count blocks of 128, so each thread walks
    // thousands of items one latency chain at a time.  Here: every resident
    // block, and more (one thread per kWoShare items, up to kWoBlocksPerSm
    // blocks per SM) on large merges -- blocks take their ids from a ticket,
    // so a look-back only waits on blocks already running -- but no thread
    // with fewer than kWoMinShare items, since each share pays two global
    // merge-path searches.
    const long long blk_items = kWoShare * kWoTpb, min_items = kWoMinShare * kWoTpb;
    const long long total = c.A.rows + c.A.nnz;
    const long long sms = device_info(c.device).sm_count;
    const void* k = c.o.compensated ? (const void*)work_oriented_spmv_kernel<VT, kWoTpb, true>
                                    : (const void*)work_oriented_spmv_kernel<VT, kWoTpb, false>;
    const int per_sm = resident_ctas_per_sm(k, kWoTpb, 0);
    long long nb = (long long)(per_sm > 2 ? per_sm : 2) * sms;
    const long long share = (total + blk_items - 1) / blk_items;
    if (share > nb) nb = share;
    if (nb > kWoBlocksPerSm * sms) nb = kWoBlocksPerSm * sms;
    const long long most = (total + min_items - 1) / min_items;
    if (nb > most) nb = most;
    if (nb < 1) nb = 1;
    return nb * kWoTpb;
  }
  static long long work_oriented_slots(const SpmvCall& c) {
    return (wo_num_threads(c) + kWoTpb - 1) / kWoTpb;
  }
  template <bool COMP>
  static el_status wo(const SpmvCall& c) {
    const long long nt = wo_num_threads(c);
    if (nt % kWoTpb != 0)
      return fail(EL_ERR_INVALID_ARGUMENT, "work_oriented: num_threads must be a multiple of %d",
                  kWoTpb);
    WoArgs w;
    w.b = basic(c);
    const long long total = c.A.rows + c.A.nnz;
    w.wpt = (total + nt - 1) / nt;
    if (w.wpt < 1) w.wpt = 1;
    w.num_blocks = (int)(nt / kWoTpb);
    w.wait_ns = c.wait_ns;
    w.ws = c.ws;
    if (w.num_blocks > c.ws.nslots)
      return fail(EL_ERR_INVALID_ARGUMENT, "work_oriented: workspace too small");
    work_oriented_spmv_kernel<VT, kWoTpb, COMP><<<w.num_blocks, kWoTpb, 0, c.stream>>>(w);
    return cuda_status(cudaGetLastError(), "work_oriented launch");
  }
  static el_status work_oriented(const SpmvCall& c) {
    return c.o.compensated ? wo<true>(c) : wo<false>(c);
  }
};

template <typename VT> el_status spmv_merge_path(const SpmvCall& c) {
  return SpmvImpl<VT>::merge_path(c);
}
template <typename VT> long long spmv_merge_path_slots(const SpmvCall& c) {
  return SpmvImpl<VT>::merge_path_slots(c);
}
template <typename VT> el_status spmv_thread_mapped(const SpmvCall& c) {
  return SpmvImpl<VT>::thread_mapped(c);
}
template <typename VT> el_status spmv_group_mapped(const SpmvCall& c) {
  return SpmvImpl<VT>::group_mapped(c);
}
template <typename VT> el_status spmv_work_oriented(const SpmvCall& c) {
  return SpmvImpl<VT>::work_oriented(c);
}
template <typename VT> long long spmv_work_oriented_slots(const SpmvCall& c) {
  return SpmvImpl<VT>::work_oriented_slots(c);
}

#define EL_INSTANTIATE_SPMV(VT)                                          \
  template el_status spmv_merge_path<VT>(const SpmvCall&);               \
  template long long spmv_merge_path_slots<VT>(const SpmvCall&);         \
  template el_status spmv_thread_mapped<VT>(const SpmvCall&);            \
  template el_status spmv_group_mapped<VT>(const SpmvCall&);             \
  template el_status spmv_work_oriented<VT>(const SpmvCall&);            \
  template long long spmv_work_oriented_slots<VT>(const SpmvCall&);

}  // namespace el
