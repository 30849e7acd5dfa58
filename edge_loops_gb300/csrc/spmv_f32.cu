// spmv_f32.cu -- SpMV schedules instantiated for float values.
#include "spmv_impl.cuh"

namespace el {
EL_INSTANTIATE_SPMV(float)
}  // namespace el
