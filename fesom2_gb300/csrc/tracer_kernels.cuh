// tracer_kernels.cuh -- sm_103a kernels of the FESOM2 tracer-transport step, FP64 form.
//
// Instantiated with R = double (kernels_fp64.cu, built with --fmad=false): the
// reference's FP64 arithmetic in the reference's evaluation order, so the results
// match the serial Fortran loops bit for bit.  The FP32 form has its own kernels
// (kernels_fp32_batched.cu) and takes only the content sums from here
// (kernels_fp32.cu).
//
// Mapping: edge and node kernels run one warp per entity with the lanes over
// the levels of the column (the reference's arrays are level-contiguous, so
// every lane load is coalesced).  Node sums are gathers over the node's
// ascending edge list instead of the reference's edge scatters: the terms are
// added in the same order, without atomics, so sums are deterministic.  The
// tridiagonal solve runs one thread per column (GB300's FP64 pipe is narrow;
// a full warp of columns keeps every lane busy).
#pragma once
#include <cuda_runtime.h>

#include "fesom_internal.h"
#include "vdiff_column.cuh"

namespace fesom {

constexpr int kWarpsPerBlock = 4;
constexpr int kThreads = 32 * kWarpsPerBlock;

template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R rabs(R a) { return fabs(a); }
template <> __device__ __forceinline__ float rabs<float>(float a) { return fabsf(a); }

// The FP64 form keeps the reference's statements and evaluation order.  The FP32
// form keeps LO's increment (the low-order flux divergence times dt/areasvol)
// in the LO buffer instead of LO itself, so the final update is a compensated
// sum of flux terms rather than the difference LO*hnode_new - T*hnode of two
// nearly equal products (which loses most FP32 bits); LO is rebuilt where the
// FCT bounds need it.
template <typename R> struct Exact { static constexpr bool value = false; };
template <> struct Exact<double> { static constexpr bool value = true; };

__device__ __forceinline__ size_t ix1(int nz, int n, int L1) { return (size_t)n * L1 + (nz - 1); }
__device__ __forceinline__ size_t ixn(int nz, int n, int nl) { return (size_t)n * nl + (nz - 1); }

// ---------------------------------------------------------------------------
// Node-sum accumulator: plain for FP64 (the reference's order and rounding),
// Neumaier-compensated for FP32.
// ---------------------------------------------------------------------------
template <typename R>
struct Acc {
    R s;
    __device__ __forceinline__ Acc() : s(R(0)) {}
    __device__ __forceinline__ void add(R x) { s = s + x; }
    __device__ __forceinline__ void sub(R x) { s = s - x; }
    __device__ __forceinline__ R get() const { return s; }
};
template <>
struct Acc<float> {
    float s, c;
    __device__ __forceinline__ Acc() : s(0.f), c(0.f) {}
    __device__ __forceinline__ void add(float x) {
        float t = s + x;
        c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
        s = t;
    }
    __device__ __forceinline__ void sub(float x) { add(-x); }
    __device__ __forceinline__ float get() const { return s + c; }
};

// ===========================================================================
// init_tracers_AB: valuesAB and the valuesold shift (src/oce_tracer_mod.F90:46-123)
// ===========================================================================
template <typename R>
__global__ void k_ab(DTracers<R> tr, size_t n, int ab) {
    const R ca = R(0.5 + kABEpsilon), cb = R(1.5 + kABEpsilon);
    for (int t = 0; t < tr.ntr; t++) {
        R *T = tr.T + t * tr.sN, *TAB = tr.TAB + t * tr.sN;
        R *O = tr.Told + t * tr.sN * (ab - 1);
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            R v = T[i];
            if (ab == 2) {
                TAB[i] = -(ca * O[i]) + cb * v;
                O[i] = v;
            } else {
                R o1 = O[2 * i], o2 = O[2 * i + 1];
                R x = R(5.0) * o2 - R(16.0) * o1 + R(23.0) * v;
                TAB[i] = x / R(12.0);
                O[2 * i + 1] = o1;
                O[2 * i] = v;
            }
        }
    }
}

// ===========================================================================
// tracer_gradient_elements (src/oce_tracer_mod.F90:147-188): warp per element
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(kThreads) k_trxy(DTopo tp, DGeom<R> g, DTracers<R> tr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1;
    for (int el = blockIdx.x * kWarpsPerBlock + warp; el < tp.T2; el += gridDim.x * kWarpsPerBlock) {
        const int a = tp.t_n[3 * el], b = tp.t_n[3 * el + 1], c = tp.t_n[3 * el + 2];
        const R *gs = g.gs + 6 * (size_t)el;
        const R g0 = gs[0], g1 = gs[1], g2 = gs[2], g3 = gs[3], g4 = gs[4], g5 = gs[5];
        const int nzmin = tp.t_ulev[el], nzmax = tp.t_nlev[el];
        for (int t = 0; t < tr.ntr; t++) {
            const R *T = tr.T + t * tr.sN;
            R *out = tr.trxy + t * tr.sT;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                R ta = T[ix1(nz, a, L1)], tb = T[ix1(nz, b, L1)], tc = T[ix1(nz, c, L1)];
                R s = R(0);
                s = s + g0 * ta;
                s = s + g1 * tb;
                s = s + g2 * tc;
                R s2 = R(0);
                s2 = s2 + g3 * ta;
                s2 = s2 + g4 * tb;
                s2 = s2 + g5 * tc;
                out[2 * ix1(nz, el, L1)] = s;
                out[2 * ix1(nz, el, L1) + 1] = s2;
            }
        }
    }
}

// ===========================================================================
// tracer_gradient_z (src/oce_tracer_mod.F90:192-232): warp per node, lanes over levels;
// tr_z(nz) = (T(nz-1) - T(nz)) / (0.5 (hnode(nz-1) + hnode(nz))) inside the column, zero at
// the first and last interface; the interfaces outside [nzmin, nzmax] are left as they are
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(kThreads) k_trz(DTopo tp, DGeom<R> g, const R *__restrict__ T, R *__restrict__ trz) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        for (int nz = nzmin + 1 + lane; nz <= nzmax - 1; nz += 32) {
            const R dz = R(0.5) * (g.hnode[ix1(nz - 1, n, L1)] + g.hnode[ix1(nz, n, L1)]);
            trz[ixn(nz, n, nl)] = (T[ix1(nz - 1, n, L1)] - T[ix1(nz, n, L1)]) / dz;
        }
        if (lane == 0) {
            trz[ixn(nzmin, n, nl)] = R(0);
            trz[ixn(nzmax, n, nl)] = R(0);
        }
    }
}

// area-weighted mean of tr_xy over the node's elements wet at level nz
// (fill_up_dn_grad, src/oce_muscl_adv.F90:388-405)
template <typename R>
__device__ __forceinline__ void node_mean_grad(const DTopo &tp, const DGeom<R> &g, const R *trxy, int node, int nz,
                                               R &gx, R &gy) {
    const int L1 = tp.L1;
    R tvol = R(0), tx = R(0), ty = R(0);
    for (int k = tp.nie_ptr[node]; k < tp.nie_ptr[node + 1]; k++) {
        const int el = tp.nie_idx[k];
        if (tp.t_nlev[el] - 1 < nz || nz < tp.t_ulev[el]) continue;
        const R ea = g.elem_area[el];
        tvol = tvol + ea;
        tx = tx + trxy[2 * ix1(nz, el, L1)] * ea;
        ty = ty + trxy[2 * ix1(nz, el, L1) + 1] * ea;
    }
    gx = tx / tvol;
    gy = ty / tvol;
}

// ===========================================================================
// Edge fluxes: adv_tra_hor_upw1 (LO, values) and adv_tra_hor_muscl / _mfct /
// _upw1 (HO, valuesAB) with fill_up_dn_grad inlined
// (src/oce_adv_tra_hor.F90:64-834, src/oce_muscl_adv.F90:356-525).
// Writes FLO (FCT only) and ADh = HO - LO (FCT) or HO (no limiter).
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(kThreads)
k_edge_flux(DTopo tp, DGeom<R> g, DForcing<R> f, DTracers<R> tr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1;
    const R RE = R(kREarth);
    for (int e = blockIdx.x * kWarpsPerBlock + warp; e < tp.E2; e += gridDim.x * kWarpsPerBlock) {
        const int n1 = tp.e_n1[e], n2 = tp.e_n2[e];
        const int el1 = tp.e_t1[e], el2 = tp.e_t2[e];
        const int nl1 = tp.t_nlev[el1] - 1, nu1 = tp.t_ulev[el1];
        const R dX1 = g.ecd[4 * (size_t)e], dY1 = g.ecd[4 * (size_t)e + 1];
        R a = RE * g.elem_cos[el1];
        int nl2 = 0, nu2 = 0;
        R dX2 = R(0), dY2 = R(0);
        if (el2 >= 0) {
            dX2 = g.ecd[4 * (size_t)e + 2];
            dY2 = g.ecd[4 * (size_t)e + 3];
            nl2 = tp.t_nlev[el2] - 1;
            nu2 = tp.t_ulev[el2];
            a = R(0.5) * (a + RE * g.elem_cos[el2]);
        }
        const int fnl12 = nl1 < nl2 ? nl1 : nl2;
        const int fnu12 = nu1 > nu2 ? nu1 : nu2;
        const int lo = tp.e_lo[e], hi = tp.e_hi[e];
        const R ex = g.edxy[2 * (size_t)e], ey = g.edxy[2 * (size_t)e + 1];
        const int up = tp.e_up[e], dn = tp.e_dn[e];
        const bool inner = (up >= 0) && (dn >= 0);
        int gzmin = 0, gzmax = 0;
        if (inner) {
            gzmin = max(tp.n_ulevmax[n1], tp.n_ulevmax[n2]);
            gzmax = min(tp.n_nlevmin[n1], tp.n_nlevmin[n2]);
        }
        const int nbl1 = tp.n_nbl[n1], nbl2 = tp.n_nbl[n2];
        for (int nz = lo + lane; nz <= hi; nz += 32) {
            // segment rule of the reference's five loops (A..E)
            int seg = 0;
            if (nz >= nu1 && nz <= fnu12 - 1) seg = 1;
            else if (nu2 > 0 && nz >= nu2 && nz <= fnu12 - 1) seg = 2;
            else if (nz >= fnu12 && nz <= fnl12) seg = 3;
            else if (nz >= fnl12 + 1 && nz <= nl1) seg = 1;
            else if (nz >= fnl12 + 1 && nz <= nl2) seg = 2;
            R vf = R(0);
            if (seg & 1) {
                const R u = f.uv[2 * ix1(nz, el1, L1)], v = f.uv[2 * ix1(nz, el1, L1) + 1];
                vf = (-(v * dX1) + u * dY1) * g.helem[ix1(nz, el1, L1)];
            }
            if (seg & 2) {
                const R u = f.uv[2 * ix1(nz, el2, L1)], v = f.uv[2 * ix1(nz, el2, L1) + 1];
                const R v2 = (v * dX2 - u * dY2) * g.helem[ix1(nz, el2, L1)];
                vf = (seg == 3) ? vf + v2 : v2;
            }
            const R avf = rabs(vf);
            for (int t = 0; t < tr.ntr; t++) {
                const DCfg c = tr.cfg[t];
                const int fct = c.lim;
                const R *T = tr.T + t * tr.sN;
                const R *TA = tr.TAB + t * tr.sN;
                R flo = R(0);
                if (fct && seg)
                    flo = -(R(0.5) * (T[ix1(nz, n1, L1)] * (vf + avf) + T[ix1(nz, n2, L1)] * (vf - avf))) - R(0);
                const R fin = fct ? flo : R(0);
                R ad = fin;
                if (seg) {
                    const R t1 = TA[ix1(nz, n1, L1)], t2 = TA[ix1(nz, n2, L1)];
                    if (c.hor == 2) {
                        ad = -(R(0.5) * (t1 * (vf + avf) + t2 * (vf - avf))) - fin;
                    } else {
                        const R *txy = tr.trxy + t * tr.sT;
                        R g1, g2, g3, g4;
                        if (inner && nz >= gzmin && nz <= gzmax - 1) {
                            g1 = txy[2 * ix1(nz, up, L1)];
                            g3 = txy[2 * ix1(nz, up, L1) + 1];
                            g2 = txy[2 * ix1(nz, dn, L1)];
                            g4 = txy[2 * ix1(nz, dn, L1) + 1];
                        } else {
                            node_mean_grad(tp, g, txy, n1, nz, g1, g3);
                            node_mean_grad(tp, g, txy, n2, nz, g2, g4);
                        }
                        R Tm2, Tm1;
                        if (c.hor == 0) {
                            const R clo1 = (nbl1 - nz) >= 0 ? R(1) : R(0);
                            const R clo2 = (nbl2 - nz) >= 0 ? R(1) : R(0);
                            Tm2 = t2 - (R(2.0) * (t2 - t1) + ex * a * g2 + ey * RE * g4) / R(6.0) * clo2;
                            Tm1 = t1 + (R(2.0) * (t2 - t1) + ex * a * g1 + ey * RE * g3) / R(6.0) * clo1;
                        } else {
                            Tm2 = t2 - (R(2.0) * (t2 - t1) + ex * a * g2 + ey * RE * g4) / R(6.0);
                            Tm1 = t1 + (R(2.0) * (t2 - t1) + ex * a * g1 + ey * RE * g3) / R(6.0);
                        }
                        const R no = R(c.ph);
                        const R cHO = (vf + avf) * Tm1 + (vf - avf) * Tm2;
                        ad = -(R(0.5) * (R(1.0) - no) * cHO) - vf * no * R(0.5) * (Tm1 + Tm2) - fin;
                    }
                }
                if (fct) tr.FLO[t * tr.sE + ix1(nz, e, L1)] = flo;
                tr.ADh[t * tr.sE + ix1(nz, e, L1)] = ad;
            }
        }
    }
}

// ===========================================================================
// Node columns, stage 1: LO solution (edge gather of the upwind fluxes,
// adv_tra_ver_upw1 with w_e, src/oce_adv_tra_driver.F90:122-250) and the
// vertical high-order flux minus the LO flux (adv_tra_ver_qr4c / _upw1 with w,
// src/oce_adv_tra_ver.F90:244-434).  Without a limiter only the HO vertical
// flux (with w_e) is formed.
// ===========================================================================
template <typename R>
__device__ __forceinline__ R ver_upw1_flux(const R *T, const R *W, const R *area, int nz, int n, int nzmin, int nzmax,
                                           int L1, int nl, R fin) {
    // statement order of the reference: surface, bottom, interior
    R v = fin;
    if (nz == nzmin) v = -(W[ixn(nz, n, nl)] * T[ix1(nz, n, L1)] * area[ixn(nz, n, nl)]) - v;
    if (nz == nzmax) v = R(0.0) - v;
    if (nz >= nzmin + 1 && nz <= nzmax - 1) {
        const R Wv = W[ixn(nz, n, nl)], aW = rabs(Wv);
        v = -(R(0.5) * (T[ix1(nz, n, L1)] * (Wv + aW) + T[ix1(nz - 1, n, L1)] * (Wv - aW)) * area[ixn(nz, n, nl)]) - v;
    }
    return v;
}

template <typename R>
__device__ __forceinline__ R ver_qr4c_flux(const R *T, const R *W, const R *area, const R *Z3, const R *zb3, int nz,
                                           int n, int nzmin, int nzmax, int L1, int nl, R no, R fin) {
    // statement order of the reference: nzmin, nzmin+1, nzmax-1, nzmax, interior
    R v = fin;
    if (nz == nzmin) v = -(T[ix1(nz, n, L1)] * W[ixn(nz, n, nl)] * area[ixn(nz, n, nl)]) - v;
    if (nz == nzmin + 1)
        v = -(R(0.5) * (T[ix1(nz - 1, n, L1)] + T[ix1(nz, n, L1)]) * W[ixn(nz, n, nl)] * area[ixn(nz, n, nl)]) - v;
    if (nz == nzmax - 1)
        v = -(R(0.5) * (T[ix1(nz - 1, n, L1)] + T[ix1(nz, n, L1)]) * W[ixn(nz, n, nl)] * area[ixn(nz, n, nl)]) - v;
    if (nz == nzmax) v = R(0.0) - v;
    if (nz >= nzmin + 2 && nz <= nzmax - 2) {
        const R tm2 = T[ix1(nz - 2, n, L1)], tm1 = T[ix1(nz - 1, n, L1)], t0 = T[ix1(nz, n, L1)],
                tp1 = T[ix1(nz + 1, n, L1)];
        const R zm2 = Z3[ix1(nz - 2, n, L1)], zm1 = Z3[ix1(nz - 1, n, L1)], z0 = Z3[ix1(nz, n, L1)],
                zp1 = Z3[ix1(nz + 1, n, L1)];
        const R qc = (tm1 - t0) / (zm1 - z0);
        const R qu = (t0 - tp1) / (z0 - zp1);
        const R qd = (tm2 - tm1) / (zm2 - zm1);
        const R zb = zb3[ixn(nz, n, nl)];
        const R Tm1 = t0 + (R(2.0) * qc + qu) * (zb - z0) / R(3.0);
        const R Tm2 = tm1 + (R(2.0) * qc + qd) * (zb - zm1) / R(3.0);
        const R Wv = W[ixn(nz, n, nl)], aW = rabs(Wv);
        const R Tmean = (Wv + aW) * Tm1 + (Wv - aW) * Tm2;
        v = (-(R(0.5) * (R(1.0) - no) * Tmean) - no * (R(0.5) * (Tm1 + Tm2)) * Wv) * area[ixn(nz, n, nl)] - v;
    }
    return v;
}

// adv_tra_ver_cdiff (src/oce_adv_tra_ver.F90:635-695): the bottom interface keeps its input
template <typename R>
__device__ __forceinline__ R ver_cdiff_flux(const R *T, const R *W, const R *area, int nz, int n, int nzmin, int nzmax,
                                            int L1, int nl, R fin) {
    if (nz == nzmin) return -(W[ixn(nz, n, nl)] * T[ix1(nz, n, L1)] * area[ixn(nz, n, nl)]) - fin;
    if (nz == nzmax) return fin;
    const R tv = R(0.5) * (T[ix1(nz - 1, n, L1)] + T[ix1(nz, n, L1)]);
    return -(tv * W[ixn(nz, n, nl)] * area[ixn(nz, n, nl)]) - fin;
}

template <typename R>
__device__ __forceinline__ R min3r(R a, R b, R c) { return rmin(rmin(a, b), c); }
// Fortran sign(1, b)
template <typename R>
__device__ __forceinline__ R sign1(R b) { return signbit(b) ? R(-1.0) : R(1.0); }

// interface value tv(k) of adv_tra_vert_ppm (src/oce_adv_tra_ver.F90:488-562) on a column:
// Tc, hc 1-based views of the layer values and the new thicknesses
template <typename R>
__device__ R ppm_tv(const R *Tc, const R *hc, int k, int nzmin, int nzmax) {
    if (k == nzmax) return Tc[nzmax - 1];
    if (k == nzmin) return Tc[nzmin];
    if (k == nzmax - 1) return R(0.5) * (Tc[nzmax - 2] + Tc[nzmax - 1]);
    if (k == nzmin + 1) return R(0.5) * (Tc[nzmin] + Tc[nzmin + 1]);
    const int nz = k - 1;
    const R dzjm1 = hc[nz - 1], dzj = hc[nz], dzjp1 = hc[nz + 1], dzjp2 = hc[nz + 2];
    const R tm1 = Tc[nz - 1], t0 = Tc[nz], tp1 = Tc[nz + 1], tp2 = Tc[nz + 2];
    R deltaj = dzj / (dzjm1 + dzj + dzjp1) *
               ((R(2.0) * dzjm1 + dzj) / (dzjp1 + dzj) * (tp1 - t0) + (dzj + R(2.0) * dzjp1) / (dzjm1 + dzj) * (t0 - tm1));
    R deltajp1 = dzjp1 / (dzj + dzjp1 + dzjp2) *
                 ((R(2.0) * dzj + dzjp1) / (dzjp2 + dzjp1) * (tp2 - tp1) +
                  (dzjp1 + R(2.0) * dzjp2) / (dzj + dzjp1) * (tp1 - t0));
    if ((tp1 - t0) * (t0 - tm1) > R(0.0))
        deltaj = min3r(rabs(deltaj), R(2.0) * rabs(tp1 - t0), R(2.0) * rabs(t0 - tm1)) * sign1(deltaj);
    else
        deltaj = R(0.0);
    if ((tp2 - tp1) * (tp1 - t0) > R(0.0))
        deltajp1 = min3r(rabs(deltajp1), R(2.0) * rabs(tp2 - tp1), R(2.0) * rabs(tp1 - t0)) * sign1(deltajp1);
    else
        deltajp1 = R(0.0);
    return t0 + dzj / (dzj + dzjp1) * (tp1 - t0) +
           R(1.0) / (dzjm1 + dzj + dzjp1 + dzjp2) *
               ((R(2.0) * dzjp1 * dzj) / (dzj + dzjp1) *
                    ((dzjm1 + dzj) / (R(2.0) * dzj + dzjp1) - (dzjp2 + dzjp1) / (R(2.0) * dzjp1 + dzj)) * (tp1 - t0) -
                dzj * (dzjm1 + dzj) / (R(2.0) * dzj + dzjp1) * deltajp1 +
                dzjp1 * (dzjp1 + dzjp2) / (dzj + R(2.0) * dzjp1) * deltaj);
}

// the PPM flux of interface nz (:564-620): the monotonised parabola of the upwind layer (nz
// when w(nz) > 0, nz-1 when w(nz) < 0) integrated over the part swept in dt (old thickness);
// the surface takes -tv w area, the bottom 0; minus the input flux
template <typename R>
__device__ R ver_ppm_flux(const R *T, const R *W, const R *area, const R *hn, const R *ho, R dt, int nz, int n,
                          int nzmin, int nzmax, int L1, int nl, R fin) {
    const R *Tc = T + (size_t)n * L1 - 1, *hc = hn + (size_t)n * L1 - 1, *oc = ho + (size_t)n * L1 - 1;
    const R *Wc = W + (size_t)n * nl - 1, *ac = area + (size_t)n * nl - 1;
    if (nz == nzmin) return -(ppm_tv(Tc, hc, nzmin, nzmin, nzmax) * Wc[nzmin] * ac[nzmin]) - fin;
    if (nz == nzmax) return R(0.0) - fin;
    const R w = Wc[nz];
    if (!(w > R(0.0)) && !(w < R(0.0))) return R(0.0) - fin;
    const bool top = w > R(0.0);
    const int j = top ? nz : nz - 1;  // the upwind layer
    R aL = ppm_tv(Tc, hc, j, nzmin, nzmax), aR = ppm_tv(Tc, hc, j + 1, nzmin, nzmax);
    const R t = Tc[j];
    if ((aR - t) * (t - aL) <= R(0.0)) {
        aL = t;
        aR = t;
    }
    if ((aR - aL) * (t - R(0.5) * (aL + aR)) > (aR - aL) * (aR - aL) / R(6.0)) aL = R(3.0) * t - R(2.0) * aR;
    if ((aR - aL) * (t - R(0.5) * (aR + aL)) < -((aR - aL) * (aR - aL) / R(6.0))) aR = R(3.0) * t - R(2.0) * aL;
    const R dzj = oc[j];
    const R aj = R(6.0) * (t - R(0.5) * (aL + aR));
    R v;
    if (top) {
        const R x = rmin(w * dt / dzj, R(1.0));
        v = -aL - R(0.5) * x * (aR - aL + (R(1.0) - R(2.0) / R(3.0) * x) * aj);
    } else {
        const R x = rmin(-(w * dt / dzj), R(1.0));
        v = -aR + R(0.5) * x * (aR - aL - (R(1.0) - R(2.0) / R(3.0) * x) * aj);
    }
    return v * ac[nz] * w - fin;
}

template <typename R>
__global__ void __launch_bounds__(kThreads)
k_node_lo(DTopo tp, DGeom<R> g, DForcing<R> f, DTracers<R> tr, R dt) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        const int k0 = tp.ne_ptr[n], k1 = tp.ne_ptr[n + 1];
        for (int t = 0; t < tr.ntr; t++) {
            const DCfg c = tr.cfg[t];
            const int fct = c.lim;
            const R *T = tr.T + t * tr.sN;
            const R *TA = tr.TAB + t * tr.sN;
            const R *FLO = tr.FLO + t * tr.sE;
            for (int nz = nzmin + lane; nz <= nzmax; nz += 32) {
                R fv0 = R(0);
                if (fct) {
                    fv0 = ver_upw1_flux(T, f.we, g.area, nz, n, nzmin, nzmax, L1, nl, R(0));
                    if (nz <= nzmax - 1) {
                        const R fv1 = ver_upw1_flux(T, f.we, g.area, nz + 1, n, nzmin, nzmax, L1, nl, R(0));
                        Acc<R> acc;
                        for (int k = k0; k < k1; k++) {
                            const int code = tp.ne_idx[k];
                            const int e = code >= 0 ? code : ~code;
                            if (nz < tp.e_lo[e] || nz > tp.e_hi[e]) continue;
                            const R x = FLO[ix1(nz, e, L1)];
                            if (code >= 0) acc.add(x);
                            else acc.sub(x);
                        }
                        const size_t i = ix1(nz, n, L1);
                        if (Exact<R>::value) {
                            tr.LO[t * tr.sN + i] = (T[i] * g.hnode[i] + (acc.get() + (fv0 - fv1)) * dt /
                                                    g.areasvol[ixn(nz, n, nl)]) / g.hnode_new[i];
                        } else {
                            acc.add(fv0);
                            acc.sub(fv1);
                            tr.LO[t * tr.sN + i] = acc.get() * dt / g.areasvol[ixn(nz, n, nl)];
                        }
                    }
                }
                const R *pw = fct ? f.w : f.we;
                // with the split vertical velocity the LO part of the antidiffusive flux is the
                // upwind flux of the full w (oce_adv_tra_driver.F90:323-334)
                const R fin = (fct && f.wsplit) ? ver_upw1_flux(T, f.w, g.area, nz, n, nzmin, nzmax, L1, nl, R(0)) : fv0;
                R v;
                if (c.ver == 0)
                    v = ver_qr4c_flux(TA, pw, g.area, g.Z3, g.zbar3, nz, n, nzmin, nzmax, L1, nl, R(c.pv), fin);
                else if (c.ver == 2)
                    v = ver_cdiff_flux(TA, pw, g.area, nz, n, nzmin, nzmax, L1, nl, fin);
                else if (c.ver == 3)
                    v = ver_ppm_flux(TA, pw, g.area, g.hnode_new, g.hnode, dt, nz, n, nzmin, nzmax, L1, nl, fin);
                else
                    v = ver_upw1_flux(TA, pw, g.area, nz, n, nzmin, nzmax, L1, nl, fin);
                tr.ADv[t * tr.sNI + ixn(nz, n, nl)] = v;
            }
        }
    }
}

// ===========================================================================
// FCT bounds a1-a3 and bound increments (src/oce_adv_tra_fct.F90:124-248).
// The element max/min (AUX) is recomputed per node from the element's three
// nodes (max/min are exact, so this equals the reference's two passes).
// ===========================================================================
// LO of node x at layer nz (the FP32 form stores the increment, see Exact)
template <typename R>
__device__ __forceinline__ R lo_value(const R *LO, const R *T, const DGeom<R> &g, int nz, int x, int L1) {
    const size_t i = ix1(nz, x, L1);
    if (Exact<R>::value) return LO[i];
    return (T[i] * g.hnode[i] + LO[i]) / g.hnode_new[i];
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_bounds(DTopo tp, DGeom<R> g, DTracers<R> tr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sm = reinterpret_cast<R *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1;
    R *tvmax = sm + (size_t)warp * 2 * (L1 + 2);
    R *tvmin = tvmax + (L1 + 2);
    const R big = R(kBigNumber);
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        const int k0 = tp.nie_ptr[n], k1 = tp.nie_ptr[n + 1];
        for (int t = 0; t < tr.ntr; t++) {
            if (!tr.cfg[t].lim) continue;
            const R *T = tr.T + t * tr.sN;
            const R *LO = tr.LO + t * tr.sN;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                R mx = R(0), mn = R(0);
                for (int k = k0; k < k1; k++) {
                    const int el = tp.nie_idx[k];
                    R amx, amn;
                    if (nz >= tp.t_ulev[el] && nz <= tp.t_nlev[el] - 1) {
                        const int a = tp.t_n[3 * el], b = tp.t_n[3 * el + 1], cc = tp.t_n[3 * el + 2];
                        const R la = lo_value(LO, T, g, nz, a, L1), ta = T[ix1(nz, a, L1)];
                        const R lb = lo_value(LO, T, g, nz, b, L1), tb = T[ix1(nz, b, L1)];
                        const R lc = lo_value(LO, T, g, nz, cc, L1), tc = T[ix1(nz, cc, L1)];
                        amx = rmax(rmax(rmax(la, ta), rmax(lb, tb)), rmax(lc, tc));
                        amn = rmin(rmin(rmin(la, ta), rmin(lb, tb)), rmin(lc, tc));
                    } else {
                        amx = -big;
                        amn = big;
                    }
                    if (k == k0) { mx = amx; mn = amn; }
                    else { mx = rmax(mx, amx); mn = rmin(mn, amn); }
                }
                tvmax[nz] = mx;
                tvmin[nz] = mn;
            }
            __syncwarp();
            R *bmx = tr.bmax + t * tr.sN, *bmn = tr.bmin + t * tr.sN;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const R lo = lo_value(LO, T, g, nz, n, L1);
                R vmx, vmn;
                if (nz == nzmin || nz == nzmax - 1) {
                    vmx = tvmax[nz] - lo;
                    vmn = tvmin[nz] - lo;
                } else {
                    vmx = rmax(rmax(tvmax[nz - 1], tvmax[nz]), tvmax[nz + 1]) - lo;
                    vmn = rmin(rmin(tvmin[nz - 1], tvmin[nz]), tvmin[nz + 1]) - lo;
                }
                bmx[ix1(nz, n, L1)] = vmx;
                bmn[ix1(nz, n, L1)] = vmn;
            }
            __syncwarp();
        }
    }
}

// ===========================================================================
// FCT b1 + b2: sums of positive / negative antidiffusive fluxes into each
// node-layer (vertical, then edges in ascending order) and the ratios R+ / R-
// (src/oce_adv_tra_fct.F90:265-405).  R+ / R- overwrite bmax / bmin.
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(kThreads) k_rpm(DTopo tp, DGeom<R> g, DTracers<R> tr, R dt) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    const R eps = R(kFluxEps);
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        const int k0 = tp.ne_ptr[n], k1 = tp.ne_ptr[n + 1];
        for (int t = 0; t < tr.ntr; t++) {
            if (!tr.cfg[t].lim) continue;
            const R *ADv = tr.ADv + t * tr.sNI;
            const R *ADh = tr.ADh + t * tr.sE;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const R v0 = ADv[ixn(nz, n, nl)], v1 = ADv[ixn(nz + 1, n, nl)];
                Acc<R> P, M;
                P.add(rmax(R(0), v0) + rmax(R(0), -v1));
                M.add(rmin(R(0), v0) + rmin(R(0), -v1));
                for (int k = k0; k < k1; k++) {
                    const int code = tp.ne_idx[k];
                    const int e = code >= 0 ? code : ~code;
                    if (nz < tp.e_lo[e] || nz > tp.e_hi[e]) continue;
                    const R x = ADh[ix1(nz, e, L1)];
                    if (code >= 0) { P.add(rmax(R(0), x)); M.add(rmin(R(0), x)); }
                    else { P.add(rmax(R(0), -x)); M.add(rmin(R(0), -x)); }
                }
                const size_t i = ix1(nz, n, L1);
                const R av = g.areasvol[ixn(nz, n, nl)], hn = g.hnode_new[i];
                R fl = P.get() * dt / av / hn + eps;
                const R rp = rmin(R(1.0), tr.bmax[t * tr.sN + i] / fl);
                fl = M.get() * dt / av / hn - eps;
                const R rm = rmin(R(1.0), tr.bmin[t * tr.sN + i] / fl);
                tr.bmax[t * tr.sN + i] = rp;
                tr.bmin[t * tr.sN + i] = rm;
            }
        }
    }
}

// ===========================================================================
// FCT b3 limiting + oce_tra_adv_flux2dtracer (src/oce_adv_tra_fct.F90:425-500,
// src/oce_adv_tra_driver.F90:494-646) + (mode 1) the del_ttf sum and the T*
// update of diff_tracers_ale (src/oce_ale_tracer.F90:319-321, 743-754).
// The limited edge flux is formed at each end node from R+/R- of both ends.
// ===========================================================================
template <typename R>
__device__ __forceinline__ R limited_adv(const R *ADv, const R *Rp, const R *Rm, int nz, int n, int nzmin, int nzmax,
                                         int L1, int nl) {
    const R x = ADv[ixn(nz, n, nl)];
    if (nz == nzmax) return x;
    R ae = R(1.0);
    if (nz == nzmin) {
        ae = x >= R(0) ? rmin(ae, Rp[ix1(nz, n, L1)]) : rmin(ae, Rm[ix1(nz, n, L1)]);
    } else if (x >= R(0)) {
        ae = rmin(ae, Rm[ix1(nz - 1, n, L1)]);
        ae = rmin(ae, Rp[ix1(nz, n, L1)]);
    } else {
        ae = rmin(ae, Rp[ix1(nz - 1, n, L1)]);
        ae = rmin(ae, Rm[ix1(nz, n, L1)]);
    }
    return ae * x;
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_update(DTopo tp, DGeom<R> g, DTracers<R> tr, R dt, int mode) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        const int k0 = tp.ne_ptr[n], k1 = tp.ne_ptr[n + 1];
        for (int t = 0; t < tr.ntr; t++) {
            const int fct = tr.cfg[t].lim;
            R *T = tr.T + t * tr.sN;
            const R *ADv = tr.ADv + t * tr.sNI;
            const R *ADh = tr.ADh + t * tr.sE;
            const R *Rp = tr.bmax + t * tr.sN, *Rm = tr.bmin + t * tr.sN;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const size_t i = ix1(nz, n, L1);
                const R av = g.areasvol[ixn(nz, n, nl)];
                R dv = R(0.0);
                R f0, f1;
                if (fct) {
                    if (Exact<R>::value) dv = dv - T[i] * g.hnode[i] + tr.LO[t * tr.sN + i] * g.hnode_new[i];
                    f0 = limited_adv(ADv, Rp, Rm, nz, n, nzmin, nzmax, L1, nl);
                    f1 = limited_adv(ADv, Rp, Rm, nz + 1, n, nzmin, nzmax, L1, nl);
                } else {
                    f0 = ADv[ixn(nz, n, nl)];
                    f1 = ADv[ixn(nz + 1, n, nl)];
                }
                Acc<R> dh;
                if (!Exact<R>::value) {
                    // FP32: one compensated sum of LO increment, vertical and horizontal terms
                    if (fct) dh.add(tr.LO[t * tr.sN + i]);
                    dh.add(f0 * dt / av);
                    dh.sub(f1 * dt / av);
                } else {
                    dv = dv + (f0 - f1) * dt / av;
                }
                for (int k = k0; k < k1; k++) {
                    const int code = tp.ne_idx[k];
                    const int e = code >= 0 ? code : ~code;
                    if (nz < tp.e_lo[e] || nz > tp.e_hi[e]) continue;
                    R x = ADh[ix1(nz, e, L1)];
                    if (fct) {
                        const int a = tp.e_n1[e], b = tp.e_n2[e];
                        R ae = R(1.0);
                        if (x >= R(0)) {
                            ae = rmin(ae, Rp[ix1(nz, a, L1)]);
                            ae = rmin(ae, Rm[ix1(nz, b, L1)]);
                        } else {
                            ae = rmin(ae, Rm[ix1(nz, a, L1)]);
                            ae = rmin(ae, Rp[ix1(nz, b, L1)]);
                        }
                        x = ae * x;
                    }
                    if (code >= 0) dh.add(x * dt / av);
                    else dh.sub(x * dt / av);
                }
                if (!Exact<R>::value) dh.add(T[i] * (g.hnode[i] - g.hnode_new[i]));
                const R dhv = dh.get();
                if (mode == 0) {
                    tr.dttf_h[t * tr.sN + i] = dhv;
                    tr.dttf_v[t * tr.sN + i] = dv;
                } else {
                    R del = dhv;
                    if (Exact<R>::value) {
                        del = R(0.0) + dhv + dv;
                        // diff_tracers_ale: horizontal, then explicit vertical diffusion
                        if (tr.HD) del = hdiff_add(tp, tr.HD + t * tr.sE, del, n, nz, L1, dt, av);
                        if (tr.VX && !tr.cfg[t].ivd) del = del + tr.VX[t * tr.sN + i];
                        // Redi: diff_ver_part_redi_expl (:623)
                        if (tr.RV) del = del + tr.RV[t * tr.sN + i];
                        del = del + T[i] * (g.hnode[i] - g.hnode_new[i]);
                    }
                    const R tn = T[i] + del / g.hnode_new[i];
                    T[i] = tn;
                    if (!isfinite(tn)) atomicOr(tr.status, 1u);
                }
            }
        }
    }
}

// ===========================================================================
// diff_ver_part_impl_ale (src/oce_ale_tracer.F90:1071-1430): one thread per
// column, arithmetic in A (double for both forms).  Scratch holds Z_n, cp and
// tp level-major ([level][node]) so that a warp's accesses are coalesced.
// ===========================================================================
// ---------------------------------------------------------------------------
// diff_part_hor_redi (oce_ale_tracer.F90:1526-1689): per edge-layer the flux c of the segment
// (A/D: element 1, B/E: element 2, C: both), Kh = (Ki(n1) + Ki(n2)) / 2, F = Kh grad T, with
// Redi F = Kh (grad T + S_xy Tz): Tz = mean over the layer of the vertical gradient at each
// edge node, S_xy Tz = (Tz(n1) S(n1) + Tz(n2) S(n2)) / 2 (:1583-1595)
// ---------------------------------------------------------------------------
// tracer_gradient_z (oce_tracer_mod.F90:192-232) of T at interface nz of node n: 0 at the
// column's top and bottom interfaces
template <typename R>
__device__ __forceinline__ R trz_node(const DTopo &tp, const DGeom<R> &g, const R *T, int n, int nz) {
    const int L1 = tp.L1;
    if (nz <= tp.n_ulev[n] || nz >= tp.n_nlev[n]) return R(0);
    const R dz = R(0.5) * (g.hnode[ix1(nz - 1, n, L1)] + g.hnode[ix1(nz, n, L1)]);
    return (T[ix1(nz - 1, n, L1)] - T[ix1(nz, n, L1)]) / dz;
}

template <typename R>
__device__ __forceinline__ void hdiff_flux(const DTopo &tp, const DGeom<R> &g, const DTracers<R> &tr, const R *T,
                                          int n1, int n2, int nz, R Kh, R Tx, R Ty, R &Fx, R &Fy) {
    if (!tr.slope) {
        Fx = Kh * Tx;
        Fy = Kh * Ty;
        return;
    }
    const int L1 = tp.L1;
    const R tz1 = R(0.5) * (trz_node(tp, g, T, n1, nz) + trz_node(tp, g, T, n1, nz + 1));
    const R tz2 = R(0.5) * (trz_node(tp, g, T, n2, nz) + trz_node(tp, g, T, n2, nz + 1));
    const R *s1 = tr.slope + 3 * ix1(nz, n1, L1), *s2 = tr.slope + 3 * ix1(nz, n2, L1);
    const R sx = (tz1 * s1[0] + tz2 * s2[0]) / R(2.0);
    const R sy = (tz1 * s1[1] + tz2 * s2[1]) / R(2.0);
    Fx = Kh * (Tx + sx);
    Fy = Kh * (Ty + sy);
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_hdiff(DTopo tp, DGeom<R> g, DTracers<R> tr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1;
    for (int e = blockIdx.x * kWarpsPerBlock + warp; e < tp.E2; e += gridDim.x * kWarpsPerBlock) {
        const int el1 = tp.e_t1[e], el2 = tp.e_t2[e], n1 = tp.e_n1[e], n2 = tp.e_n2[e];
        const int nl1 = tp.t_nlev[el1] - 1, ul1 = tp.t_ulev[el1];
        int nl2 = 0, ul2 = 0;
        const R dX1 = g.ecd[4 * (size_t)e], dY1 = g.ecd[4 * (size_t)e + 1];
        R dX2 = R(0), dY2 = R(0);
        if (el2 >= 0) {
            nl2 = tp.t_nlev[el2] - 1;
            ul2 = tp.t_ulev[el2];
            dX2 = g.ecd[4 * (size_t)e + 2];
            dY2 = g.ecd[4 * (size_t)e + 3];
        }
        const int nl12 = nl1 < nl2 ? nl1 : nl2, ul12 = ul1 > ul2 ? ul1 : ul2;
        for (int nz = tp.e_lo[e] + lane; nz <= tp.e_hi[e]; nz += 32) {
            int seg = 0;
            if (nz >= ul1 && nz <= ul12 - 1) seg = 1;                    // (A)
            else if (ul2 > 0 && nz >= ul2 && nz <= ul12 - 1) seg = 2;    // (B)
            else if (nz >= ul12 && nz <= nl12) seg = 3;                 // (C)
            else if (nz >= nl12 + 1 && nz <= nl1) seg = 1;              // (D)
            else if (nz >= nl12 + 1 && nz <= nl2) seg = 2;              // (E)
            for (int t = 0; t < tr.ntr; t++) {
                const R *Ki = tr.Ki;
                const R *xy = tr.trxy + t * tr.sT;
                const R *T = tr.T + t * tr.sN;
                const R Kh = (Ki[ix1(nz, n1, L1)] + Ki[ix1(nz, n2, L1)]) / R(2.0);
                R c = R(0), Fx, Fy;
                if (seg == 1) {
                    const R dz = g.helem[ix1(nz, el1, L1)];
                    hdiff_flux(tp, g, tr, T, n1, n2, nz, Kh, xy[2 * ix1(nz, el1, L1)], xy[2 * ix1(nz, el1, L1) + 1], Fx,
                               Fy);
                    c = (-dX1 * Fy + dY1 * Fx) * dz;
                } else if (seg == 2) {
                    const R dz = g.helem[ix1(nz, el2, L1)];
                    hdiff_flux(tp, g, tr, T, n1, n2, nz, Kh, xy[2 * ix1(nz, el2, L1)], xy[2 * ix1(nz, el2, L1) + 1], Fx,
                               Fy);
                    c = (dX2 * Fy - dY2 * Fx) * dz;
                } else if (seg == 3) {
                    const R dz = (g.helem[ix1(nz, el1, L1)] + g.helem[ix1(nz, el2, L1)]) / R(2.0);
                    const R Tx = R(0.5) * (xy[2 * ix1(nz, el1, L1)] + xy[2 * ix1(nz, el2, L1)]);
                    const R Ty = R(0.5) * (xy[2 * ix1(nz, el1, L1) + 1] + xy[2 * ix1(nz, el2, L1) + 1]);
                    hdiff_flux(tp, g, tr, T, n1, n2, nz, Kh, Tx, Ty, Fx, Fy);
                    c = ((dX2 - dX1) * Fy - (dY2 - dY1) * Fx) * dz;
                }
                tr.HD[t * tr.sE + ix1(nz, e, L1)] = c;
            }
        }
    }
}

// del(n) += rhs * dt / areasvol(n) for each edge of n in ascending edge order; rhs = 0 + c at
// edges(1,e), 0 - c at edges(2,e) (oce_ale_tracer.F90:1677-1684)
template <typename R>
__device__ __forceinline__ R hdiff_add(const DTopo &tp, const R *HD, R del, int n, int nz, int L1, R dt, R av) {
    for (int k = tp.ne_ptr[n]; k < tp.ne_ptr[n + 1]; k++) {
        const int code = tp.ne_idx[k];
        const int e = code >= 0 ? code : ~code;
        if (nz < tp.e_lo[e] || nz > tp.e_hi[e]) continue;
        const R c = HD[ix1(nz, e, L1)];
        const R rhs = code >= 0 ? R(0) + c : R(0) - c;
        del = del + rhs * dt / av;
    }
    return del;
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_hdiff_gather(DTopo tp, DGeom<R> g, DTracers<R> tr, R dt, R *del) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
        for (int t = 0; t < tr.ntr; t++)
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const size_t i = ix1(nz, n, L1);
                del[t * tr.sN + i] =
                    hdiff_add(tp, tr.HD + t * tr.sE, del[t * tr.sN + i], n, nz, L1, dt, g.areasvol[ixn(nz, n, nl)]);
            }
    }
}

// ---------------------------------------------------------------------------
// diff_ver_part_expl_ale (oce_ale_tracer.F90:841-902): vd(ul) = surface flux (f.bc),
// vd(nz) = Kv (T(nz-1) - T(nz)) / (Z(nz-1) - Z(nz)) area; increment of layer nz
// (vd(nz) - vd(nz+1)) / (zbar(nz) - zbar(nz+1)) dt / areasvol, at the bottom layer
// (vd(nl1) / (zbar(nl1) - zbar(nl1+1))) dt / areasvol
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R vexpl_vd(const DTopo &tp, const DGeom<R> &g, const R *Kv, const R *T, R fsurf, int n,
                                      int nz, int ul1, int nl1, int L1, int nl) {
    if (nz == ul1) return fsurf;
    if (nz > nl1) return R(0);
    const R zinv1 = R(1.0) / (g.Z3[ix1(nz - 1, n, L1)] - g.Z3[ix1(nz, n, L1)]);
    return Kv[ixn(nz, n, nl)] * (T[ix1(nz - 1, n, L1)] - T[ix1(nz, n, L1)]) * zinv1 * g.area[ixn(nz, n, nl)];
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_vexpl(DTopo tp, DGeom<R> g, DForcing<R> f, DTracers<R> tr, R dt,
                                                    R *out, int all, int add) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * kWarpsPerBlock + warp; n < tp.N2; n += gridDim.x * kWarpsPerBlock) {
        const int nl1 = tp.n_nlev[n] - 1, ul1 = tp.n_ulev[n];
        for (int t = 0; t < tr.ntr; t++) {
            if (!all && tr.cfg[t].ivd) continue;
            const R *T = tr.T + t * tr.sN;
            const R fs = f.bc ? f.bc[(size_t)t * tp.N2 + n] : R(0);
            for (int nz = ul1 + lane; nz <= nl1; nz += 32) {
                const size_t i = ix1(nz, n, L1);
                const R av = g.areasvol[ixn(nz, n, nl)];
                const R v0 = vexpl_vd(tp, g, f.Kv, T, fs, n, nz, ul1, nl1, L1, nl);
                R inc;
                if (nz <= nl1 - 1) {
                    const R v1 = vexpl_vd(tp, g, f.Kv, T, fs, n, nz + 1, ul1, nl1, L1, nl);
                    inc = (v0 - v1) / (g.zbar3[ixn(nz, n, nl)] - g.zbar3[ixn(nz + 1, n, nl)]) * dt / av;
                } else {
                    inc = (v0 / (g.zbar3[ixn(nz, n, nl)] - g.zbar3[ixn(nz + 1, n, nl)])) * dt / av;
                }
                R *o = out + t * tr.sN;
                o[i] = add ? o[i] + inc : inc;
            }
        }
    }
}

// ===========================================================================
// adv_tra_vert_impl (src/oce_adv_tra_ver.F90:90-240) on the LO values of the FCT tracers:
// implicit upwind advection by w_i, one thread per column, arithmetic in A (double); scratch
// holds cp and tp level-major
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(128) k_lo_impl(DTopo tp, DGeom<R> g, DForcing<R> f, DTracers<R> tr, double dt,
                                                 double *scratch) {
    typedef double A;
    const int L1 = tp.L1, nl = tp.nl;
    const size_t N2 = tp.N2;
    A *cps = scratch, *tps = scratch + (size_t)(L1 + 1) * N2;
#define CP(k) cps[(size_t)(k) * N2 + n]
#define TP(k) tps[(size_t)(k) * N2 + n]
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
        const R *hn = g.hnode_new + (size_t)n * L1 - 1;
        const R *ar = g.area + (size_t)n * nl - 1;
        const R *av = g.areasvol + (size_t)n * nl - 1;
        const R *wi = f.wi + (size_t)n * nl - 1;
        for (int t = 0; t < tr.ntr; t++) {
            if (!tr.cfg[t].lim) continue;
            R *Tc = tr.LO + t * tr.sN + (size_t)n * L1 - 1;
            const A zinv = 1.0 * dt;
            int nz = nzmin;
            A v = zinv * (A)ar[nz] / (A)av[nz];
            A b = (A)hn[nz] + (A)wi[nz] * v;
            v = zinv * (A)ar[nz + 1] / (A)av[nz];
            b = b - fmin(0.0, (A)wi[nz + 1]) * v;
            A c = -(fmax(0.0, (A)wi[nz + 1]) * v);
            A T0 = (A)Tc[nz], Tp1 = (A)Tc[nz + 1], Tm;
            A rhs = -((b - (A)hn[nz]) * T0) - c * Tp1;
            A cp = c / b, tpv = rhs / b;
            CP(nz) = cp;
            TP(nz) = tpv;
            for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
                v = zinv * (A)ar[nz] / (A)av[nz];
                const A a = fmin(0.0, (A)wi[nz]) * v;
                b = (A)hn[nz] + fmax(0.0, (A)wi[nz]) * v;
                v = zinv * (A)ar[nz + 1] / (A)av[nz];
                b = b - fmin(0.0, (A)wi[nz + 1]) * v;
                c = -(fmax(0.0, (A)wi[nz + 1]) * v);
                Tm = T0;
                T0 = Tp1;
                Tp1 = (A)Tc[nz + 1];
                rhs = -(a * Tm) - (b - (A)hn[nz]) * T0 - c * Tp1;
                const A m = b - cp * a;
                cp = c / m;
                tpv = (rhs - tpv * a) / m;
                CP(nz) = cp;
                TP(nz) = tpv;
            }
            nz = nzmax - 1;
            {
                v = zinv * (A)ar[nz] / (A)av[nz];
                const A a = fmin(0.0, (A)wi[nz]) * v;
                b = (A)hn[nz] + fmax(0.0, (A)wi[nz]) * v;
                Tm = T0;
                T0 = Tp1;
                rhs = -(a * Tm) - (b - (A)hn[nz]) * T0;
                const A m = b - cp * a;
                tpv = (rhs - tpv * a) / m;
            }
            A trv = tpv;
            Tc[nzmax - 1] = (R)((A)Tc[nzmax - 1] + trv);
            for (nz = nzmax - 2; nz >= nzmin; nz--) {
                trv = TP(nz) - CP(nz) * trv;
                Tc[nz] = (R)((A)Tc[nz] + trv);
            }
        }
    }
#undef CP
#undef TP
}

template <typename R>
__global__ void __launch_bounds__(128) k_vdiff(DTopo tp, DGeom<R> g, DForcing<R> f, DTracers<R> tr, double dt,
                                               double *scratch) {
    const int L1 = tp.L1, nl = tp.nl;
    const size_t N2 = tp.N2;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
        const R *hn = g.hnode_new + (size_t)n * L1 - 1;  // hn[nz], 1-based
        const R *ar = g.area + (size_t)n * nl - 1;
        const R *av = g.areasvol + (size_t)n * nl - 1;
        const R *kv = f.Kv + (size_t)n * nl - 1;
        const R *wi = f.wi + (size_t)n * nl - 1;
        const ColScratch cs{scratch + n, scratch + (size_t)(L1 + 1) * N2 + n, scratch + 2 * (size_t)(L1 + 1) * N2 + n,
                            N2};
        vdiff_col_z<R>(cs, nzmin, nzmax, (double)g.zbar_n_bot[n], hn);
        for (int t = 0; t < tr.ntr; t++) {
            if (!tr.cfg[t].ivd) continue;
            // the implicit part of a split vertical velocity joins the solve without a limiter (:961)
            const bool wimpl = f.wsplit && !tr.cfg[t].lim;
            const double bc = f.bc ? (double)f.bc[(size_t)t * N2 + n] : 0.0;
            vdiff_col_solve<R>(cs, nzmin, nzmax, hn, ar, av, kv, wimpl, wi, bc, dt, tr.T + t * tr.sN + (size_t)n * L1 - 1);
        }
    }
}

// ---------------------------------------------------------------------------
// diff_ver_part_redi_expl (oce_ale_tracer.F90:1439-1518), one thread per column, walking the
// column bottom up: node gradients (sum over the node's elements wet at nz of tr_xy
// elem_area) / 3 / areasvol; depths zbar_n, z_n from hnode and zbar_n_bot; interface flux
// vd(nz) = ((z(nz-1) - zbar(nz)) S.g(nz-1) Ki(nz-1) + (zbar(nz) - z(nz)) S.g(nz) Ki(nz))
// / (z(nz-1) - z(nz)) area(nz); increment (vd(nz) - vd(nz+1)) dt / areasvol into RV
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R redi_proj(const DTopo &tp, const DGeom<R> &g, const R *xy, const R *slope, int n, int nz) {
    const int L1 = tp.L1;
    R tx = R(0), ty = R(0);
    for (int k = tp.nie_ptr[n]; k < tp.nie_ptr[n + 1]; k++) {
        const int el = tp.nie_idx[k];
        if (nz <= tp.t_nlev[el] - 1 && nz >= tp.t_ulev[el]) {
            tx = tx + xy[2 * ix1(nz, el, L1)] * g.elem_area[el];
            ty = ty + xy[2 * ix1(nz, el, L1) + 1] * g.elem_area[el];
        }
    }
    const R av = g.areasvol[ixn(nz, n, tp.nl)];
    const R gx = tx / R(3.0) / av, gy = ty / R(3.0) / av;
    const R *s = slope + 3 * ix1(nz, n, L1);
    return s[0] * gx + s[1] * gy;
}

template <typename R>
__global__ void __launch_bounds__(128) k_redi_v(DTopo tp, DGeom<R> g, DTracers<R> tr, R dt, int add) {
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nl1 = tp.n_nlev[n] - 1, ul1 = tp.n_ulev[n];
        const R *Ki = tr.Ki;
        for (int t = 0; t < tr.ntr; t++) {
            const R *xy = tr.trxy + t * tr.sT;
            R *out = tr.RV + t * tr.sN;
            R zb = g.zbar_n_bot[n];                                  // zbar_n(nz + 1)
            R zc = zb + g.hnode[ix1(nl1, n, L1)] / R(2.0);           // z_n(nz)
            R pc = redi_proj(tp, g, xy, tr.slope, n, nl1);           // S . grad at nz
            R below = R(0);                                          // vd(nz + 1)
            for (int nz = nl1; nz >= ul1; nz--) {
                R vd = R(0);
                if (nz >= ul1 + 1) {
                    const R zbn = zb + g.hnode[ix1(nz, n, L1)];                  // zbar_n(nz)
                    const R zu = zbn + g.hnode[ix1(nz - 1, n, L1)] / R(2.0);     // z_n(nz - 1)
                    const R pu = redi_proj(tp, g, xy, tr.slope, n, nz - 1);
                    R v = (zu - zbn) * pu * Ki[ix1(nz - 1, n, L1)];
                    v = v + (zbn - zc) * pc * Ki[ix1(nz, n, L1)];
                    vd = v / (zu - zc) * g.area[ixn(nz, n, nl)];
                    zb = zbn;
                    zc = zu;
                    pc = pu;
                }
                const R inc = (vd - below) * dt / g.areasvol[ixn(nz, n, nl)];
                out[ix1(nz, n, L1)] = add ? out[ix1(nz, n, L1)] + inc : inc;
                below = vd;
            }
        }
    }
}

// K33 = Kv + Ty of diff_ver_part_impl_ale with Redi (oce_ale_tracer.F90:1099-1204) at the
// interfaces nzmin < nz < nzmax, from zbar_n / Z_n of hnode_new bottom up:
// Ty = (zbar(nz) - Z(nz)) / dZ s3(nz-1)^2 Ki(nz-1) + (Z(nz-1) - zbar(nz)) / dZ s3(nz)^2 Ki(nz),
// dZ = Z(nz-1) - Z(nz) (the Ty1 of the layer above is the same number); Kv elsewhere
template <typename R>
__global__ void __launch_bounds__(128) k_k33(DTopo tp, DGeom<R> g, const R *Kv, const R *Ki, const R *slope, R *K33) {
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
        for (int nz = 1; nz <= nl; nz++) K33[ixn(nz, n, nl)] = Kv[ixn(nz, n, nl)];
        R zb = g.zbar_n_bot[n];                                         // zbar_n(nz + 1)
        R Zc = zb + g.hnode_new[ix1(nzmax - 1, n, L1)] / R(2.0);        // Z_n(nz)
        for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
            const R zbn = zb + g.hnode_new[ix1(nz, n, L1)];             // zbar_n(nz)
            const R Zu = zbn + g.hnode_new[ix1(nz - 1, n, L1)] / R(2.0);  // Z_n(nz - 1)
            const R zinv = R(1.0) / (Zu - Zc);
            const R sa = slope[3 * ix1(nz - 1, n, L1) + 2], sb = slope[3 * ix1(nz, n, L1) + 2];
            const R Ty = (zbn - Zc) * zinv * (sa * sa) * Ki[ix1(nz - 1, n, L1)] +
                         (Zu - zbn) * zinv * (sb * sb) * Ki[ix1(nz, n, L1)];
            K33[ixn(nz, n, nl)] = Kv[ixn(nz, n, nl)] + Ty;
            zb = zbn;
            Zc = Zu;
        }
    }
}

// ===========================================================================
// Global content sum over wet node-layers of T * hnode_new * areasvol (FP64),
// deterministic: fixed per-block partials, then one ordered pass.
// ===========================================================================
template <typename R>
__global__ void __launch_bounds__(256) k_content_partial(DTopo tp, DGeom<R> g, DTracers<R> tr, double *partials) {
    __shared__ double red[256];
    const int L1 = tp.L1, nl = tp.nl;
    for (int t = 0; t < tr.ntr; t++) {
        const R *T = tr.T + t * tr.sN;
        double s = 0.0;
        for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
            for (int nz = tp.n_ulev[n]; nz <= tp.n_nlev[n] - 1; nz++) {
                const size_t i = ix1(nz, n, L1);
                s += (double)T[i] * (double)g.hnode_new[i] * (double)g.areasvol[ixn(nz, n, nl)];
            }
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[(size_t)t * gridDim.x + blockIdx.x] = red[0];
        __syncthreads();
    }
}

static __global__ void k_content_final(const double *partials, int nblk, int ntr, double *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += partials[(size_t)t * nblk + b];
    out[t] = s;
}

// ===========================================================================
// launch wrappers
// ===========================================================================
static inline int grid_for(int nent, int per_block) {
    int b = (nent + per_block - 1) / per_block;
    const int cap = 152 * 64;
    if (b > cap) b = cap;
    return b < 1 ? 1 : b;
}

template <typename R>
void Launch<R>::ab(const DTopo &tp, DTracers<R> &tr, int ab, cudaStream_t s) {
    const size_t n = (size_t)tp.L1 * tp.N2;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_ab<R><<<blocks, 256, 0, s>>>(tr, n, ab);
}
template <typename R>
void Launch<R>::trxy(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, cudaStream_t s) {
    k_trxy<R><<<grid_for(tp.T2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, tr);
}
template <typename R>
void Launch<R>::trz(const DTopo &tp, const DGeom<R> &g, const R *T, R *trz, cudaStream_t s) {
    k_trz<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, T, trz);
}
template <typename R>
void Launch<R>::edge_flux(const DTopo &tp, const DGeom<R> &g, const DForcing<R> &f, DTracers<R> &tr, int fct,
                          cudaStream_t s) {
    (void)fct;
    k_edge_flux<R><<<grid_for(tp.E2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, f, tr);
}
template <typename R>
void Launch<R>::node_lo(const DTopo &tp, const DGeom<R> &g, const DForcing<R> &f, DTracers<R> &tr, double dt, int fct,
                        cudaStream_t s) {
    (void)fct;
    k_node_lo<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, f, tr, (R)dt);
}
template <typename R>
void Launch<R>::bounds(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, cudaStream_t s) {
    const size_t sm = sizeof(R) * 2 * (tp.L1 + 2) * kWarpsPerBlock;
    k_bounds<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, sm, s>>>(tp, g, tr);
}
template <typename R>
void Launch<R>::rpm(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, double dt, cudaStream_t s) {
    k_rpm<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, tr, (R)dt);
}
template <typename R>
void Launch<R>::update(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, double dt, int fct, int mode,
                       cudaStream_t s) {
    (void)fct;
    k_update<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, tr, (R)dt, mode);
}
template <typename R>
void Launch<R>::lo_impl(const DTopo &tp, const DGeom<R> &g, const DForcing<R> &f, DTracers<R> &tr, double dt,
                        double *scratch, cudaStream_t s) {
    k_lo_impl<R><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, tr, dt, scratch);
}
template <typename R>
void Launch<R>::vdiff(const DTopo &tp, const DGeom<R> &g, const DForcing<R> &f, DTracers<R> &tr, double dt,
                      double *scratch, cudaStream_t s) {
    int blocks = (tp.N2 + 127) / 128;
    k_vdiff<R><<<blocks, 128, 0, s>>>(tp, g, f, tr, dt, scratch);
}
template <typename R>
void Launch<R>::content(const DTopo &tp, const DGeom<R> &g, const DTracers<R> &tr, double *partials, int nblk,
                        double *out, cudaStream_t s) {
    k_content_partial<R><<<nblk, 256, 0, s>>>(tp, g, tr, partials);
    k_content_final<<<(tr.ntr + 63) / 64, 64, 0, s>>>(partials, nblk, tr.ntr, out);
}

template <typename R>
void Launch<R>::hdiff(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, cudaStream_t s) {
    k_hdiff<R><<<grid_for(tp.E2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, tr);
}
template <typename R>
void Launch<R>::hdiff_gather(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, double dt, R *del, cudaStream_t s) {
    k_hdiff_gather<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, tr, (R)dt, del);
}
template <typename R>
void Launch<R>::vexpl(const DTopo &tp, const DGeom<R> &g, const DForcing<R> &f, DTracers<R> &tr, double dt, R *out,
                      int all, int add, cudaStream_t s) {
    k_vexpl<R><<<grid_for(tp.N2, kWarpsPerBlock), kThreads, 0, s>>>(tp, g, f, tr, (R)dt, out, all, add);
}
template <typename R>
void Launch<R>::redi_v(const DTopo &tp, const DGeom<R> &g, DTracers<R> &tr, double dt, int add, cudaStream_t s) {
    k_redi_v<R><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, tr, (R)dt, add);
}
template <typename R>
void Launch<R>::k33(const DTopo &tp, const DGeom<R> &g, const R *Kv, const R *Ki, const R *slope, R *K33,
                    cudaStream_t s) {
    k_k33<R><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, Kv, Ki, slope, K33);
}

}  // namespace fesom
