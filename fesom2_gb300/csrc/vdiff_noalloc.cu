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
// start at zero.  A status word beside it records columns whose level bounds the
// kernel refused (it is cleared at the start of every call).  All calls share both:
// calls that overlap on the GPU (different streams, or different host threads) race
// on them.  A call waits, with a time limit, for its kernel and reads the status word
// back, so it returns only when the values are final.
//
// The column solve is the one k_vdiff<double> runs (vdiff_column.cuh), built with
// --fmad=false in both places, so the results equal those of fesom_gpu_vdiff_impl bit
// for bit.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>

#include "../../include/fesom_gpu.h"
#include "vdiff_column.cuh"

namespace {

using fesom::ColScratch;
using fesom::vdiff_col_solve;
using fesom::vdiff_col_z;

// 3 arrays of nl levels per column (Z_n, cp, tp at levels 0 .. nl-1): nod2D * nl * 3 <= this bound.
constexpr size_t kScratchDoubles = FESOM_GPU_NOALLOC_SCRATCH_DOUBLES;
static __device__ __align__(256) double g_vdiff_scratch[kScratchDoubles];
// FESOM_STATUS_* bits of the last call (cleared at the start of each call)
static __device__ unsigned g_status;

constexpr int kMaxDevices = 64;
constexpr int kWaitLimitMs = 60000;
std::mutex g_mu;
// per device, looked up once with the device current: the device addresses of the two arrays
// above, and an event the call waits on
struct DevState {
    double *scratch = nullptr;
    unsigned *status = nullptr;
    cudaEvent_t done = nullptr;
};
DevState g_dev[kMaxDevices];

void set_err(char *errbuf, int32_t errlen, const char *msg) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, msg, (size_t)errlen - 1);
        errbuf[errlen - 1] = 0;
    }
}

// diff_ver_part_impl_ale (src/oce_ale_tracer.F90:1071-1430) for one column per thread, the
// column solve k_vdiff<double> uses.  The level arrays come from the caller and are not
// validated on the host: a column outside 1 <= ulevels_nod2D, nlevels_nod2D <= nl with at least
// two wet layers is skipped (its values untouched, nothing read or written outside the arrays)
// and raises FESOM_STATUS_INDEX in g_status.
__global__ void __launch_bounds__(128)
k_vdiff_noalloc(int N2_, int nl, const int *__restrict__ nlev, const int *__restrict__ ulev,
                const double *__restrict__ zbar_n_bot, const double *__restrict__ hnode_new,
                const double *__restrict__ area, const double *__restrict__ areasvol, const double *__restrict__ Kv,
                const double *__restrict__ bc_surf, double dt, double *__restrict__ values, double *scratch,
                unsigned *status) {
    const int L1 = nl - 1;
    const size_t N2 = (size_t)N2_;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N2_; n += gridDim.x * blockDim.x) {
        const int nzmax = nlev[n], nzmin = ulev[n];
        if (nzmin < 1 || nzmax > nl || nzmax - nzmin < 2) {
            atomicOr(status, FESOM_STATUS_INDEX);
            continue;
        }
        const ColScratch cs{scratch + n, scratch + (size_t)(L1 + 1) * N2 + n, scratch + 2 * (size_t)(L1 + 1) * N2 + n,
                            N2};
        const double *hn = hnode_new + (size_t)n * L1 - 1;
        vdiff_col_z<double>(cs, nzmin, nzmax, zbar_n_bot[n], hn);
        vdiff_col_solve<double>(cs, nzmin, nzmax, hn, area + (size_t)n * nl - 1, areasvol + (size_t)n * nl - 1,
                                Kv + (size_t)n * nl - 1, false, nullptr, bc_surf ? bc_surf[n] : 0.0, dt,
                                values + (size_t)n * L1 - 1);
    }
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
    DevState st;
    {
        // one-time set-up per device, with that device current: the host-side names of the
        // arrays are not device addresses, so fetch the addresses the kernel must use
        std::lock_guard<std::mutex> lk(g_mu);
        DevState &d = g_dev[dev];
        if (!d.scratch) {
            void *p = nullptr, *q = nullptr;
            e = cudaGetSymbolAddress(&p, g_vdiff_scratch);
            if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_status);
            if (e == cudaSuccess && !d.done) e = cudaEventCreateWithFlags(&d.done, cudaEventDisableTiming);
            if (e != cudaSuccess || !p || !q) {
                set_err(errbuf, errlen, cudaGetErrorString(e));
                return FESOM_ERR_CUDA;
            }
            d.status = (unsigned *)q;
            d.scratch = (double *)p;
        }
        st = d;
    }
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemsetAsync(st.status, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) {
        set_err(errbuf, errlen, cudaGetErrorString(e));
        return FESOM_ERR_CUDA;
    }
    const int threads = 128;
    int blocks = (nod2D + threads - 1) / threads;
    k_vdiff_noalloc<<<blocks, threads, 0, s>>>(nod2D, nl, nlevels_nod2D, ulevels_nod2D, zbar_n_bot, hnode_new, area,
                                               areasvol, Kv, bc_surf, dt, values, st.scratch, st.status);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(st.done, s);
    if (e != cudaSuccess) {
        set_err(errbuf, errlen, cudaGetErrorString(e));
        return FESOM_ERR_CUDA;
    }
    // wait, with a time limit, for the kernel, then read its status word
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        e = cudaEventQuery(st.done);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) {
            set_err(errbuf, errlen, cudaGetErrorString(e));
            return FESOM_ERR_CUDA;
        }
        const auto ms =
            std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
        if (ms > kWaitLimitMs) {
            set_err(errbuf, errlen, "fesom_gpu_vdiff_impl_noalloc: the solve did not finish within the time limit");
            return FESOM_ERR_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(ms < 10 ? 20 : 500));
    }
    unsigned bits = 0;
    e = cudaMemcpy(&bits, st.status, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_err(errbuf, errlen, cudaGetErrorString(e));
        return FESOM_ERR_CUDA;
    }
    if (bits & FESOM_STATUS_INDEX) {
        set_err(errbuf, errlen,
                "fesom_gpu_vdiff_impl_noalloc: a column outside 1 <= ulevels_nod2D, nlevels_nod2D <= nl with at least "
                "two wet layers was skipped");
        return FESOM_ERR_MESH;
    }
    return FESOM_OK;
}
