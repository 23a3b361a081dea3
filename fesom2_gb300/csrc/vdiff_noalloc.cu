// vdiff_noalloc.cu -- implicit vertical diffusion that allocates nothing.
//
// Some callers of this library cannot call cudaMalloc: FESOM2's OpenACC build
// keeps every device array inside `!$ACC DATA` regions owned by the OpenACC
// runtime and hands them to native code as device addresses (`!$ACC HOST_DATA
// USE_DEVICE`), and codes that run under a fixed device-memory budget may not
// grow their footprint per call.  They already hold the inputs and outputs on
// the device; what the regular entry point (fesom_gpu_vdiff_impl) adds is a
// context with its own allocations, including the scratch of the column solve.
// This variant of that solve (k_vdiff, FP64) takes the caller's device arrays
// and keeps its scratch in a fixed file-scope device array instead, so a call
// allocates nothing.
//
// The scratch holds, per column, Z_n and the Thomas factors cp/tp, level-major;
// every entry a call reads is written by the same call first, so nothing has to
// start at zero.  All calls share the array: calls that overlap on the GPU
// (different streams, or different host threads) race on it.
//
// Built with --fmad=false like the FP64 kernels, so the results equal those of
// fesom_gpu_vdiff_impl bit for bit.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/fesom_gpu.h"

namespace {

// 3 arrays of (nl+1) levels per column: nod2D * (nl+1) * 3 <= this bound.
constexpr size_t kScratchDoubles = FESOM_GPU_NOALLOC_SCRATCH_DOUBLES;
static __device__ __align__(256) double g_vdiff_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices] = {nullptr};

void set_err(char *errbuf, int32_t errlen, const char *msg) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, msg, (size_t)errlen - 1);
        errbuf[errlen - 1] = 0;
    }
}

// diff_ver_part_impl_ale (src/oce_ale_tracer.F90:1071-1430) for one column per
// thread; same statements and evaluation order as k_vdiff<double>.
__global__ void __launch_bounds__(128)
k_vdiff_noalloc(int N2_, int nl, const int *__restrict__ nlev, const int *__restrict__ ulev,
                const double *__restrict__ zbar_n_bot, const double *__restrict__ hnode_new,
                const double *__restrict__ area, const double *__restrict__ areasvol, const double *__restrict__ Kv,
                const double *__restrict__ bc_surf, double dt, double *__restrict__ values, double *scratch) {
    typedef double A;
    const int L1 = nl - 1;
    const size_t N2 = (size_t)N2_;
    A *Zs = scratch, *cps = scratch + (size_t)(L1 + 1) * N2, *tps = cps + (size_t)(L1 + 1) * N2;
#define ZN(k) Zs[(size_t)(k) * N2 + n]
#define CP(k) cps[(size_t)(k) * N2 + n]
#define TP(k) tps[(size_t)(k) * N2 + n]
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N2_; n += gridDim.x * blockDim.x) {
        const int nzmax = nlev[n], nzmin = ulev[n];
        const A *hn = hnode_new + (size_t)n * L1 - 1;
        const A *ar = area + (size_t)n * nl - 1;
        const A *av = areasvol + (size_t)n * nl - 1;
        const A *kv = Kv + (size_t)n * nl - 1;
        A *Tc = values + (size_t)n * L1 - 1;
        A zb = zbar_n_bot[n];
        ZN(nzmax - 1) = zb + hn[nzmax - 1] / 2.0;
        for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
            zb = zb + hn[nz];
            ZN(nz - 1) = zb + hn[nz - 1] / 2.0;
        }
        const A bc = bc_surf ? bc_surf[n] : 0.0;
        int nz = nzmin;
        A zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1));
        const A zinv = 1.0 * dt;
        A c = -(kv[nz + 1] * zinv2 * zinv * ar[nz + 1] / av[nz]);
        A b = -c + hn[nz];
        A Tm = Tc[nz], T0 = Tm, Tp1 = Tc[nz + 1];
        A dz = hn[nz];
        A rhs = -((b - dz) * T0) - c * Tp1;
        rhs = rhs + bc;
        A cp = c / b, tpv = rhs / b;
        CP(nz) = cp;
        TP(nz) = tpv;
        A zinv1 = zinv2;
        for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
            zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1));
            const A a = -(kv[nz] * zinv1 * zinv * (ar[nz] / av[nz]));
            c = -(kv[nz + 1] * zinv2 * zinv * ar[nz + 1] / av[nz]);
            b = -a - c + hn[nz];
            zinv1 = zinv2;
            Tm = T0;
            T0 = Tp1;
            Tp1 = Tc[nz + 1];
            dz = hn[nz];
            rhs = -(a * Tm) - (b - dz) * T0 - c * Tp1;
            const A m = b - cp * a;
            cp = c / m;
            tpv = (rhs - tpv * a) / m;
            CP(nz) = cp;
            TP(nz) = tpv;
        }
        nz = nzmax - 1;
        {
            const A a = -(kv[nz] * zinv1 * zinv * (ar[nz] / av[nz]));
            b = -a + hn[nz];
            Tm = T0;
            T0 = Tp1;
            dz = hn[nz];
            rhs = -(a * Tm) - (b - dz) * T0;
            const A m = b - cp * a;
            tpv = (rhs - tpv * a) / m;
        }
        A trv = tpv;
        Tc[nzmax - 1] = Tc[nzmax - 1] + trv;
        for (nz = nzmax - 2; nz >= nzmin; nz--) {
            trv = TP(nz) - CP(nz) * trv;
            Tc[nz] = Tc[nz] + trv;
        }
    }
#undef ZN
#undef CP
#undef TP
}

}  // namespace

extern "C" int fesom_gpu_vdiff_impl_noalloc(int32_t nod2D, int32_t nl, const int32_t *nlevels_nod2D,
                                            const int32_t *ulevels_nod2D, const double *zbar_n_bot,
                                            const double *hnode_new, const double *area, const double *areasvol,
                                            const double *Kv, const double *bc_surf, double dt, double *values,
                                            void *stream, char *errbuf, int32_t errlen) {
    if (nod2D <= 0 || nl < 3 || !nlevels_nod2D || !ulevels_nod2D || !zbar_n_bot || !hnode_new || !area ||
        !areasvol || !Kv || !values) {
        set_err(errbuf, errlen, "fesom_gpu_vdiff_impl_noalloc: null array or non-positive size");
        return FESOM_ERR_ARG;
    }
    const size_t need = 3 * (size_t)nl * (size_t)nod2D;
    if (need > kScratchDoubles) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "fesom_gpu_vdiff_impl_noalloc: mesh too large for the fixed scratch: 3*nl*nod2D = %zu doubles "
                      "> %zu (use fesom_gpu_vdiff_impl)",
                      need, kScratchDoubles);
        set_err(errbuf, errlen, msg);
        return FESOM_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_err(errbuf, errlen, "fesom_gpu_vdiff_impl_noalloc: no current CUDA device");
        return FESOM_ERR_CUDA;
    }
    double *scratch;
    {
        // one-time set-up per device, with that device current: the host-side name of
        // the array is not a device address, so fetch the address the kernel must use
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_vdiff_scratch);
            if (e != cudaSuccess || !p) {
                set_err(errbuf, errlen, cudaGetErrorString(e));
                return FESOM_ERR_CUDA;
            }
            g_scratch_addr[dev] = (double *)p;
        }
        scratch = g_scratch_addr[dev];
    }
    const int threads = 128;
    int blocks = (nod2D + threads - 1) / threads;
    k_vdiff_noalloc<<<blocks, threads, 0, (cudaStream_t)stream>>>(nod2D, nl, nlevels_nod2D, ulevels_nod2D, zbar_n_bot,
                                                                   hnode_new, area, areasvol, Kv, bc_surf, dt, values,
                                                                   scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err(errbuf, errlen, cudaGetErrorString(e));
        return FESOM_ERR_CUDA;
    }
    return FESOM_OK;
}
