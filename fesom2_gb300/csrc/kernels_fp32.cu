// kernels_fp32.cu -- the one FP32 instantiation of the generic tracer kernels the FP32
// form uses: the FP64 global content sums of FP32 tracer values (k_content_partial /
// k_content_final).  Every other FP32 stage has its own kernels (kernels_fp32_batched.cu).
#include "tracer_kernels.cuh"

namespace fesom {
template void Launch<float>::content(const DTopo &, const DGeom<float> &, const DTracers<float> &, double *, int,
                                     double *, cudaStream_t);
}
