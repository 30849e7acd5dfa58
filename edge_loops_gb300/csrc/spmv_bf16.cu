// spmv_bf16.cu -- SpMV schedules instantiated for __nv_bfloat16 values.
#include "spmv_impl.cuh"

namespace el {
EL_INSTANTIATE_SPMV(__nv_bfloat16)
}  // namespace el
