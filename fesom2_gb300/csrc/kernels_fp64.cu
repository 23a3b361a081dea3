// kernels_fp64.cu -- FP64 ("plain") instantiation of the tracer kernels.
// Built with --fmad=false: no multiply-add contraction, so every operation
// rounds exactly as the reference's FP64 Fortran loops do.
#include "tracer_kernels.cuh"

namespace fesom {
template struct Launch<double>;
}
