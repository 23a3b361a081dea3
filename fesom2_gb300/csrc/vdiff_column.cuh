// vdiff_column.cuh -- the column solve of diff_ver_part_impl_ale (FP64), shared by the
// context kernel k_vdiff (tracer_kernels.cuh) and the allocation-free entry point
// (vdiff_noalloc.cu).  Both translation units build with --fmad=false, so the two give
// the same bits.
//
// One thread per column.  Scratch entry k of a column (Z_n, the Thomas factors cp and tp)
// sits at p[k * st]: level-major over the columns of a launch, so the threads of a warp
// touch consecutive addresses at every level.
#pragma once
#include <cuda_runtime.h>

namespace fesom {

struct ColScratch {
    double *z, *cp, *tp;  // already offset to the thread's column
    size_t st;            // distance between consecutive levels of one column
};

// Z_n of the column from the bottom up (src/oce_ale_tracer.F90:1088-1096); hn is 1-based
template <typename R>
__device__ __forceinline__ void vdiff_col_z(const ColScratch &s, int nzmin, int nzmax, double zbot, const R *hn) {
    typedef double A;
    A zb = zbot;
    s.z[(size_t)(nzmax - 1) * s.st] = zb + (A)hn[nzmax - 1] / 2.0;
    for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
        zb = zb + (A)hn[nz];
        s.z[(size_t)(nz - 1) * s.st] = zb + (A)hn[nz - 1] / 2.0;
    }
}

// The tridiagonal system of one tracer's column (coefficients built on the fly,
// src/oce_ale_tracer.F90:1099-1229, bc_surface at the top :1377-1383), forward elimination
// (:1406-1414) and back substitution (:1417-1430), T += the solution.  wimpl: the implicit
// part of a split vertical velocity joins the solve (:961, 1134-1216).  Arrays are 1-based
// column pointers; the column holds nzmin .. nzmax-1 with at least two layers.
template <typename R>
__device__ __forceinline__ void vdiff_col_solve(const ColScratch &s, int nzmin, int nzmax, const R *hn, const R *ar,
                                                const R *av, const R *kv, bool wimpl, const R *wi, double bc,
                                                double dt, R *Tc) {
    typedef double A;
#define ZN(k) s.z[(size_t)(k) * s.st]
#define CP(k) s.cp[(size_t)(k) * s.st]
#define TP(k) s.tp[(size_t)(k) * s.st]
    int nz = nzmin;
    A zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1));
    const A zinv = 1.0 * dt;
    A c = -((A)kv[nz + 1] * zinv2 * zinv * (A)ar[nz + 1] / (A)av[nz]);
    A b = -c + (A)hn[nz];
    if (wimpl) {  // :1134-1147
        A v = zinv * ((A)ar[nz] / (A)av[nz]);
        b = b + (A)wi[nz] * v;
        v = zinv * (A)ar[nz + 1] / (A)av[nz];
        b = b - fmin(0.0, (A)wi[nz + 1]) * v;
        c = c - fmax(0.0, (A)wi[nz + 1]) * v;
    }
    A Tm = (A)Tc[nz], T0 = Tm, Tp1 = (A)Tc[nz + 1];
    A dz = (A)hn[nz];
    A rhs = -((b - dz) * T0) - c * Tp1;
    rhs = rhs + bc;
    A cp = c / b, tpv = rhs / b;
    CP(nz) = cp;
    TP(nz) = tpv;
    A zinv1 = zinv2;
    for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
        zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1));
        A a = -((A)kv[nz] * zinv1 * zinv * ((A)ar[nz] / (A)av[nz]));
        c = -((A)kv[nz + 1] * zinv2 * zinv * (A)ar[nz + 1] / (A)av[nz]);
        b = -a - c + (A)hn[nz];
        zinv1 = zinv2;
        if (wimpl) {  // :1176-1189
            A v = zinv * ((A)ar[nz] / (A)av[nz]);
            a = a + fmin(0.0, (A)wi[nz]) * v;
            b = b + fmax(0.0, (A)wi[nz]) * v;
            v = zinv * (A)ar[nz + 1] / (A)av[nz];
            b = b - fmin(0.0, (A)wi[nz + 1]) * v;
            c = c - fmax(0.0, (A)wi[nz + 1]) * v;
        }
        Tm = T0;
        T0 = Tp1;
        Tp1 = (A)Tc[nz + 1];
        dz = (A)hn[nz];
        rhs = -(a * Tm) - (b - dz) * T0 - c * Tp1;
        const A m = b - cp * a;
        cp = c / m;
        tpv = (rhs - tpv * a) / m;
        CP(nz) = cp;
        TP(nz) = tpv;
    }
    nz = nzmax - 1;
    {
        A a = -((A)kv[nz] * zinv1 * zinv * ((A)ar[nz] / (A)av[nz]));
        b = -a + (A)hn[nz];
        if (wimpl) {  // :1207-1216
            const A v = zinv * ((A)ar[nz] / (A)av[nz]);
            a = a + fmin(0.0, (A)wi[nz]) * v;
            b = b + fmax(0.0, (A)wi[nz]) * v;
        }
        Tm = T0;
        T0 = Tp1;
        dz = (A)hn[nz];
        rhs = -(a * Tm) - (b - dz) * T0;
        const A m = b - cp * a;
        tpv = (rhs - tpv * a) / m;
    }
    A trv = tpv;
    Tc[nzmax - 1] = (R)((A)Tc[nzmax - 1] + trv);
    for (nz = nzmax - 2; nz >= nzmin; nz--) {
        trv = TP(nz) - CP(nz) * trv;
        Tc[nz] = (R)((A)Tc[nz] + trv);
    }
#undef ZN
#undef CP
#undef TP
}

}  // namespace fesom
