// spmv_dispatch.cu -- value-type dispatch of the SpMV launchers.
#include "el_internal.h"

namespace el {

#define EL_BY_DTYPE(fn)                                  \
  switch (c.A.value_dtype) {                             \
    case EL_F32: return fn<float>(c);                    \
    case EL_BF16: return fn<__nv_bfloat16>(c);           \
    default: return fn<__half>(c);                       \
  }

el_status launch_merge_path(const SpmvCall& c) { EL_BY_DTYPE(spmv_merge_path) }
long long merge_path_slots_needed(const SpmvCall& c) { EL_BY_DTYPE(spmv_merge_path_slots) }
el_status launch_thread_mapped(const SpmvCall& c) { EL_BY_DTYPE(spmv_thread_mapped) }
el_status launch_group_mapped(const SpmvCall& c) { EL_BY_DTYPE(spmv_group_mapped) }
el_status launch_work_oriented(const SpmvCall& c) { EL_BY_DTYPE(spmv_work_oriented) }
long long work_oriented_slots_needed(const SpmvCall& c) {
  EL_BY_DTYPE(spmv_work_oriented_slots)
}

}  // namespace el
