// spmv_f16.cu -- SpMV schedules instantiated for __half values.
#include "spmv_impl.cuh"

namespace el {
EL_INSTANTIATE_SPMV(__half)
}  // namespace el
