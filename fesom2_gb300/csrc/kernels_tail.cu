// kernels_tail.cu -- the tail of the tracer loop of solve_tracers_ale, FP64 (built with
// --fmad=false so every product and sum rounds as in the reference):
//   radioactive decay of IDs 14 / 39 (src/oce_ale_tracer.F90:355-356), relax_to_clim
//   (src/oce_tracer_mod.F90:236-298) or the Soufflet channel's relax_zonal_temp of tracer 1
//   (src/toy_channel_soufflet.F90:91-121), the salinity clamp to [3, 45] and the age-tracer
//   floor (src/oce_ale_tracer.F90:497-525).
#include <cuda_runtime.h>

#include "fesom_internal.h"

namespace fesom {

// one tracer: v *= decay (whole field) ; relaxation ; clamp, element by element in that order
__global__ void k_tracer_tail(DTopo tp, const double *__restrict__ coord_y, double *__restrict__ v, TailArgs a) {
    const int L1 = tp.L1;
    const size_t N = (size_t)L1 * tp.N2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(i / L1), nz = (int)(i - (size_t)n * L1) + 1;
        double x = v[i];
        if (a.decay) x = x * a.decay_f;
        const int nzmin = tp.n_ulev[n], nlev = tp.n_nlev[n];
        if (a.relax == 1 && nz >= nzmin && nz <= nlev - 1) {
            x = x + a.r2c[n] * a.dt * (a.clim[i] - x);
        } else if (a.relax == 2 && nz <= nlev - 1) {
            const double yy = coord_y[n] - a.lat0;
            double w = 0.0;
            int nn, nn1;
            if (yy < a.dy / 2.0) {
                nn = 1;
                nn1 = 1;
            } else {
                nn = (int)floor(yy / a.dy - 0.5) + 1;
                if (nn > a.nbins) nn = a.nbins;  // outside the table (the reference reads past it)
                nn1 = nn + 1;
                if (nn1 > a.nbins) nn1 = nn;
                w = yy / a.dy + 0.5 - nn;
            }
            const double Tzon = (1.0 - w) * a.ztem[(nz - 1) + (size_t)(nn - 1) * L1] + w * a.ztem[(nz - 1) + (size_t)(nn1 - 1) * L1];
            for (int r = 0; r < a.repeat; r++) x = x + a.dt * a.tau_inv * (a.clim[i] - Tzon);
        }
        if (a.clamp && nz >= nzmin && nz <= nlev - 1) {
            if (a.clamp == 1) {
                if (x > 45.0) x = 45.0;
                if (x < 3.0) x = 3.0;
            } else if (x < 0.0) {
                x = 0.0;
            }
        }
        v[i] = x;
    }
}

void launch_tracer_tail(const DTopo &tp, const double *coord_y, double *v, const TailArgs &a, cudaStream_t s) {
    const size_t N = (size_t)tp.L1 * tp.N2;
    const int blocks = (int)((N + 255) / 256 < 152 * 32 ? (N + 255) / 256 : 152 * 32);
    k_tracer_tail<<<blocks, 256, 0, s>>>(tp, coord_y, v, a);
}

}  // namespace fesom
