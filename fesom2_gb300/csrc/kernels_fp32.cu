// kernels_fp32.cu -- FP32 ("batched") instantiation of the tracer kernels:
// FP32 storage and arithmetic, compensated node sums, FP64 Thomas solve and
// FP64 content sums (see tracer_kernels.cuh).
#include "tracer_kernels.cuh"

namespace fesom {
template struct Launch<float>;
}
