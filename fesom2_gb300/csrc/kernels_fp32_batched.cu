// kernels_fp32_batched.cu -- the FP32 batched form of the tracer step.
//
// All tracers of a step in one launch per stage; four tracer stages, two
// tracer-independent set-up stages:
//
//   k32_vflux     edge volume fluxes per edge-layer (oce_adv_tra_hor.F90:159-250
//                 segment rule); shared by every tracer
//   k32_vfactors  FP64 factorisation of the implicit vertical-diffusion matrix of
//                 every column (oce_ale_tracer.F90:1088-1204, 1406-1414): the
//                 pivots m = b - cp*a carry the cancellation that thin bottom cells
//                 cause, so they are formed in FP64; stored as FP32 a, c, 1/m, c/m
//   k32_lo_ad     per node: the LO solution's increment (edge gather of upwind
//                 fluxes + upwind vertical flux with w_e), the vertical
//                 antidiffusive flux (QR4C/UPW1 with w on the AB values) and the
//                 antidiffusive flux of the edges the node owns (edges(1,e) == n):
//                 MUSCL/MFCT/UPW1 on the AB values with fill_up_dn_grad inlined
//   k32_bounds    per node: FCT bounds (max/min of LO and T over the node's wet
//                 elements and the adjacent layers) and R+/R- (oce_adv_tra_fct.F90)
//   k32_update    per node: limited fluxes, flux divergence, T* update and the
//                 implicit vertical diffusion as two warp scans of affine maps over
//                 the column (the forward and back substitution with the FP64
//                 factors), written to the buffer of the oldest time level
//
// Layout: tracer-major, column-contiguous per tracer (the reference's
// a(level, node) per tracer).  One warp per node with the lanes over the levels
// of the column: every column access is coalesced, neighbour columns come
// through L1/L2.  No atomics: each edge flux is written by its owner node only,
// every node sum is a gather.  The Adams-Bashforth shift is a rotation of the
// time-level buffers (no copy).
#include <cuda_runtime.h>

#include "fesom_internal.h"

namespace fesom {

namespace {

constexpr int kW = 4;                 // warps per block
constexpr int kT = 32 * kW;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kU = 8;                 // neighbours per unrolled group
constexpr int kMaxChunks = 4;         // columns up to 128 layers

__device__ __forceinline__ size_t i1(int nz, int n, int L1) { return (size_t)n * L1 + (nz - 1); }
__device__ __forceinline__ size_t iN(int nz, int n, int nl) { return (size_t)n * nl + (nz - 1); }

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float t = s + x;
        c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
        s = t;
    }
    __device__ __forceinline__ float get() const { return s + c; }
};

// upwind vertical flux with velocity W at interface nz (statement order of
// adv_tra_ver_upw1: surface, bottom, interior), fin = 0
__device__ __forceinline__ float vupw(const float *T, const float *W, const float *area, int nz, int n, int nzmin,
                                      int nzmax, int L1, int nl) {
    if (nz == nzmin) return -(W[iN(nz, n, nl)] * T[i1(nz, n, L1)] * area[iN(nz, n, nl)]);
    if (nz == nzmax) return 0.f;
    const float w = W[iN(nz, n, nl)], aw = fabsf(w);
    return -(0.5f * (T[i1(nz, n, L1)] * (w + aw) + T[i1(nz - 1, n, L1)] * (w - aw)) * area[iN(nz, n, nl)]);
}

}  // namespace

// ---------------------------------------------------------------------------
// k32_vflux: volume flux of every edge-layer (shared by all tracers)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kT) k32_vflux(DTopo tp, DGeom<float> g, DForcing<float> f, float *VF) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1;
    for (int e = blockIdx.x * kW + warp; e < tp.E2; e += gridDim.x * kW) {
        const int el1 = tp.e_t1[e], el2 = tp.e_t2[e];
        const int nl1 = tp.t_nlev[el1] - 1, nu1 = tp.t_ulev[el1];
        int nl2 = 0, nu2 = 0;
        const float dX1 = g.ecd[4 * (size_t)e], dY1 = g.ecd[4 * (size_t)e + 1];
        float dX2 = 0.f, dY2 = 0.f;
        if (el2 >= 0) {
            nl2 = tp.t_nlev[el2] - 1;
            nu2 = tp.t_ulev[el2];
            dX2 = g.ecd[4 * (size_t)e + 2];
            dY2 = g.ecd[4 * (size_t)e + 3];
        }
        const int fnl12 = min(nl1, nl2), fnu12 = max(nu1, nu2);
        for (int nz = tp.e_lo[e] + lane; nz <= tp.e_hi[e]; nz += 32) {
            int seg = 0;
            if (nz >= nu1 && nz <= fnu12 - 1) seg = 1;
            else if (nu2 > 0 && nz >= nu2 && nz <= fnu12 - 1) seg = 2;
            else if (nz >= fnu12 && nz <= fnl12) seg = 3;
            else if (nz >= fnl12 + 1 && nz <= nl1) seg = 1;
            else if (nz >= fnl12 + 1 && nz <= nl2) seg = 2;
            float vf = 0.f;
            if (seg & 1) {
                const float u = f.uv[2 * i1(nz, el1, L1)], v = f.uv[2 * i1(nz, el1, L1) + 1];
                vf = (-(v * dX1) + u * dY1) * g.helem[i1(nz, el1, L1)];
            }
            if (seg & 2) {
                const float u = f.uv[2 * i1(nz, el2, L1)], v = f.uv[2 * i1(nz, el2, L1) + 1];
                vf += (v * dX2 - u * dY2) * g.helem[i1(nz, el2, L1)];
            }
            VF[i1(nz, e, L1)] = vf;
        }
    }
}

// ---------------------------------------------------------------------------
// k32_vfactors: FP64 factorisation of each column's tridiagonal system
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k32_vfactors(DTopo tp, DGeom<float> g, DForcing<float> f, double dt,
                                                    VFactors vf) {
    // a(k) = -Kv(k) dt/(Z_n(k-1)-Z_n(k)) area(k)/areasvol(k), c(k) = -Kv(k+1) dt/(Z_n(k)-Z_n(k+1))
    // area(k+1)/areasvol(k), b = -a - c + hnode_new (oce_ale_tracer.F90:1099-1204), with
    // Z_n(k)-Z_n(k+1) = (hnode_new(k) + hnode_new(k+1))/2 (the mid-depths of :1088-1096);
    // Thomas pivots m(k) = b(k) - cp(k-1) a(k), cp(k) = c(k)/m(k) (:1406-1414)
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
        const float *hn = g.hnode_new + (size_t)n * L1 - 1;
        const float *ar = g.area + (size_t)n * nl - 1;
        const float *av = g.areasvol + (size_t)n * nl - 1;
        const float *kv = f.Kv + (size_t)n * nl - 1;
        float *oa = vf.a + (size_t)n * L1 - 1, *oc = vf.c + (size_t)n * L1 - 1;
        float *oi = vf.inv + (size_t)n * L1 - 1, *ocp = vf.cp + (size_t)n * L1 - 1;
        double cp = 0.0, zinv1 = 0.0;
        double hcur = (double)hn[nzmin];
        for (int nz = nzmin; nz <= nzmax - 1; nz++) {
            const double hnext = nz < nzmax - 1 ? (double)hn[nz + 1] : 0.0;
            const double avz = (double)av[nz];
            const double a = nz > nzmin ? -((double)kv[nz] * zinv1 * dt * ((double)ar[nz] / avz)) : 0.0;
            double c = 0.0, zinv2 = 0.0;
            if (nz < nzmax - 1) {
                zinv2 = 2.0 / (hcur + hnext);
                c = -((double)kv[nz + 1] * zinv2 * dt * (double)ar[nz + 1] / avz);
            }
            const double b = -a - c + hcur;
            const double inv = 1.0 / (b - cp * a);
            cp = c * inv;
            oa[nz] = (float)a;
            oc[nz] = (float)c;
            oi[nz] = (float)inv;
            ocp[nz] = (float)cp;
            zinv1 = zinv2;
            hcur = hnext;
        }
    }
}

// ---------------------------------------------------------------------------
// per-node staging: the node's edge list in shared memory, once per node
// ---------------------------------------------------------------------------
struct NodeEdges {
    int e[kMaxDeg], m[kMaxDeg], lo[kMaxDeg], hi[kMaxDeg];
    unsigned own;  // bit j: the node is edges(1, e_j) (it owns the edge flux)
    int deg, nzmin, nzmax;
};

__device__ __forceinline__ void stage_node(const DTopo &tp, int n, NodeEdges &S) {
    const int k0 = tp.ne_ptr[n];
    const int deg = tp.ne_ptr[n + 1] - k0;
    if (threadIdx.x < deg && threadIdx.x < kMaxDeg) {
        const int j = threadIdx.x;
        const int code = tp.ne_idx[k0 + j];
        const int e = code >= 0 ? code : ~code;
        S.e[j] = e;
        S.m[j] = code >= 0 ? tp.e_n2[e] : tp.e_n1[e];
        S.lo[j] = tp.e_lo[e];
        S.hi[j] = tp.e_hi[e];
    }
    if (threadIdx.x == 32) {
        unsigned own = 0;
        for (int j = 0; j < deg && j < kMaxDeg; j++)
            if (tp.ne_idx[k0 + j] >= 0) own |= 1u << j;
        S.own = own;
        S.deg = deg;
        S.nzmin = tp.n_ulev[n];
        S.nzmax = tp.n_nlev[n];
    }
}

// area-weighted mean over the node's wet elements of the element gradient,
// projected on the edge: ex*a*gx + ey*R*gy (fill_up_dn_grad node means)
__device__ __noinline__ float node_grad_proj(const DTopo &tp, const DGeom<float> &g, const float *T, int node, int nz,
                                             float exa, float eyr) {
    const int L1 = tp.L1;
    float tvol = 0.f, tx = 0.f, ty = 0.f;
    for (int k = tp.nie_ptr[node]; k < tp.nie_ptr[node + 1]; k++) {
        const int el = tp.nie_idx[k];
        if (tp.t_nlev[el] - 1 < nz || nz < tp.t_ulev[el]) continue;
        const int a = tp.t_n[3 * el], b = tp.t_n[3 * el + 1], c = tp.t_n[3 * el + 2];
        const float *gs = g.gs + 6 * (size_t)el;
        const float ta = T[i1(nz, a, L1)], tb = T[i1(nz, b, L1)], tc = T[i1(nz, c, L1)];
        const float ea = g.elem_area[el];
        tvol += ea;
        tx += (gs[0] * ta + gs[1] * tb + gs[2] * tc) * ea;
        ty += (gs[3] * ta + gs[4] * tb + gs[5] * tc) * ea;
    }
    return exa * (tx / tvol) + eyr * (ty / tvol);
}

// ---------------------------------------------------------------------------
// k32_lo_ad
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kT)
k32_lo_ad(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, MusclW mw, const float *VF, float dt) {
    __shared__ NodeEdges S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    const float RE = (float)kREarth;
    for (int n = blockIdx.x; n < tp.N2; n += gridDim.x) {
        __syncthreads();
        stage_node(tp, n, S);
        __syncthreads();
        const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
        for (int t = warp; t < B.ntr; t += kW) {
            const DCfg c = B.cfg[t];
            const int fct = c.lim;
            const float *T = B.T + t * B.sN;
            const float *O1 = B.O1 + t * B.sN;
            const float *O2 = B.ab == 3 ? B.O2 + t * B.sN : nullptr;
            auto tab = [&](size_t i) {
                const float v = T[i];
                return B.ab == 2 ? -(0.6f * O1[i]) + 1.6f * v : (5.0f * O2[i] - 16.0f * O1[i] + 23.0f * v) * (1.0f / 12.0f);
            };
            for (int nz = nzmin + lane; nz <= nzmax; nz += 32) {
                float fv0 = 0.f, fv1 = 0.f;
                if (fct) {
                    fv0 = vupw(T, f.we, g.area, nz, n, nzmin, nzmax, L1, nl);
                    if (nz <= nzmax - 1) fv1 = vupw(T, f.we, g.area, nz + 1, n, nzmin, nzmax, L1, nl);
                }
                const float *pw = fct ? f.w : f.we;
                const float ar = g.area[iN(nz, n, nl)];
                float ho;
                if (nz == nzmax) {
                    ho = 0.f;
                } else if (nz == nzmin) {
                    ho = -(tab(i1(nz, n, L1)) * pw[iN(nz, n, nl)] * ar);
                } else if (c.ver != 0 || nz == nzmin + 1 || nz == nzmax - 1) {
                    const float w = pw[iN(nz, n, nl)];
                    const float t0 = tab(i1(nz, n, L1)), tm1 = tab(i1(nz - 1, n, L1));
                    if (c.ver == 0) {
                        ho = -(0.5f * (tm1 + t0) * w * ar);
                        // a two-layer column writes this row twice: flux = C - (C - flux_in)
                        if (nzmin + 1 == nzmax - 1) ho = ho - (ho - fv0) + fv0;
                    } else {
                        const float aw = fabsf(w);
                        ho = -(0.5f * (t0 * (w + aw) + tm1 * (w - aw)) * ar);
                    }
                } else {
                    const float tm2 = tab(i1(nz - 2, n, L1)), tm1 = tab(i1(nz - 1, n, L1));
                    const float t0 = tab(i1(nz, n, L1)), tp1 = tab(i1(nz + 1, n, L1));
                    const float zm2 = g.Z3[i1(nz - 2, n, L1)], zm1 = g.Z3[i1(nz - 1, n, L1)];
                    const float z0 = g.Z3[i1(nz, n, L1)], zp1 = g.Z3[i1(nz + 1, n, L1)];
                    const float qc = (tm1 - t0) / (zm1 - z0);
                    const float qu = (t0 - tp1) / (z0 - zp1);
                    const float qd = (tm2 - tm1) / (zm2 - zm1);
                    const float zb = g.zbar3[iN(nz, n, nl)];
                    const float Tm1 = t0 + (2.f * qc + qu) * (zb - z0) * (1.f / 3.f);
                    const float Tm2 = tm1 + (2.f * qc + qd) * (zb - zm1) * (1.f / 3.f);
                    const float w = pw[iN(nz, n, nl)], aw = fabsf(w);
                    const float no = (float)c.pv;
                    const float Tmean = (w + aw) * Tm1 + (w - aw) * Tm2;
                    ho = (-(0.5f * (1.f - no) * Tmean) - no * (0.5f * (Tm1 + Tm2)) * w) * ar;
                }
                B.ADv[t * B.sNI + iN(nz, n, nl)] = ho - fv0;
                if (nz > nzmax - 1) continue;
                const size_t i = i1(nz, n, L1);
                const float Tn = T[i];
                const float TAn = tab(i);
                Kahan acc;
                for (int g0 = 0; g0 < deg; g0 += kU) {
                    float vf[kU], tm[kU];
                    bool ok[kU];
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        const int j = g0 + u;
                        ok[u] = j < deg && nz >= S.lo[j] && nz <= S.hi[j];
                        vf[u] = ok[u] ? VF[i1(nz, S.e[j], L1)] : 0.f;
                        tm[u] = ok[u] ? T[i1(nz, S.m[j], L1)] : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        if (!ok[u]) continue;
                        const int j = g0 + u;
                        const bool own = (S.own >> j) & 1u;
                        const float v = vf[u], av = fabsf(v);
                        const float T1 = own ? Tn : tm[u], T2 = own ? tm[u] : Tn;
                        const float flo = fct ? -(0.5f * (T1 * (v + av) + T2 * (v - av))) : 0.f;
                        if (fct) acc.add(own ? flo : -flo);
                        if (!own) continue;
                        // owned edge: high-order flux on the AB values
                        const int e = S.e[j], m = S.m[j];
                        const float t1 = TAn, t2 = tab(i1(nz, m, L1));
                        float hf;
                        if (c.hor == 2) {
                            hf = -(0.5f * (t1 * (v + av) + t2 * (v - av)));
                        } else {
                            const int4 un = mw.un[e], dn = mw.dn[e];
                            const float4 wu = mw.wu[e], wd = mw.wd[e];
                            const int gzmin = un.w & 0xffff, gzmax = un.w >> 16;
                            float s1, s2;
                            if (nz >= gzmin && nz <= gzmax - 1) {
                                s1 = wu.x * T[i1(nz, un.x, L1)] + wu.y * T[i1(nz, un.y, L1)] + wu.z * T[i1(nz, un.z, L1)];
                                s2 = wd.x * T[i1(nz, dn.x, L1)] + wd.y * T[i1(nz, dn.y, L1)] + wd.z * T[i1(nz, dn.z, L1)];
                            } else {
                                const float exa = g.edxy[2 * (size_t)e] * wu.w;
                                const float eyr = g.edxy[2 * (size_t)e + 1] * RE;
                                s1 = node_grad_proj(tp, g, T, n, nz, exa, eyr);
                                s2 = node_grad_proj(tp, g, T, m, nz, exa, eyr);
                            }
                            float clo1 = 1.f, clo2 = 1.f;
                            if (c.hor == 0) {
                                clo1 = (tp.n_nbl[n] - nz) >= 0 ? 1.f : 0.f;
                                clo2 = (tp.n_nbl[m] - nz) >= 0 ? 1.f : 0.f;
                            }
                            const float d2 = 2.f * (t2 - t1);
                            const float Tm2 = t2 - (d2 + s2) * (1.f / 6.f) * clo2;
                            const float Tm1 = t1 + (d2 + s1) * (1.f / 6.f) * clo1;
                            const float no = (float)c.ph;
                            const float cHO = (v + av) * Tm1 + (v - av) * Tm2;
                            hf = -(0.5f * (1.f - no) * cHO) - v * no * 0.5f * (Tm1 + Tm2);
                        }
                        B.ADh[t * B.sE + i1(nz, e, L1)] = hf - flo;
                    }
                }
                if (fct) {
                    acc.add(fv0);
                    acc.add(-fv1);
                    B.LOi[t * B.sN + i] = acc.get() * dt / g.areasvol[iN(nz, n, nl)];
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// k32_bounds: FCT bounds and R+ / R- (FCT tracers only)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kT) k32_bounds(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ NodeEdges S;
    extern __shared__ __align__(16) float sm32[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    float *tvmax = sm32 + (size_t)warp * 2 * (L1 + 2);
    float *tvmin = tvmax + (L1 + 2);
    const float eps = (float)kFluxEps;
    for (int n = blockIdx.x; n < tp.N2; n += gridDim.x) {
        __syncthreads();
        stage_node(tp, n, S);
        __syncthreads();
        const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
        for (int t = warp; t < B.ntr; t += kW) {
            if (!B.cfg[t].lim) continue;
            const float *T = B.T + t * B.sN;
            const float *LOi = B.LOi + t * B.sN;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const size_t i = i1(nz, n, L1);
                const float tt = T[i];
                const float lo = (tt * g.hnode[i] + LOi[i]) / g.hnode_new[i];
                float mx = fmaxf(lo, tt), mn = fminf(lo, tt);
                for (int g0 = 0; g0 < deg; g0 += kU) {
                    float tm[kU], li[kU], hm[kU], hnm[kU];
                    bool ok[kU];
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        const int j = g0 + u;
                        ok[u] = j < deg && nz >= S.lo[j] && nz <= S.hi[j];
                        const size_t jj = ok[u] ? i1(nz, S.m[j], L1) : i;
                        tm[u] = T[jj];
                        li[u] = LOi[jj];
                        hm[u] = g.hnode[jj];
                        hnm[u] = g.hnode_new[jj];
                    }
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        if (!ok[u]) continue;
                        const float lm = (tm[u] * hm[u] + li[u]) / hnm[u];
                        mx = fmaxf(mx, fmaxf(lm, tm[u]));
                        mn = fminf(mn, fminf(lm, tm[u]));
                    }
                }
                tvmax[nz] = mx;
                tvmin[nz] = mn;
            }
            __syncwarp();
            const float *ADv = B.ADv + t * B.sNI;
            const float *ADh = B.ADh + t * B.sE;
            for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
                const size_t i = i1(nz, n, L1);
                const float lo = (T[i] * g.hnode[i] + LOi[i]) / g.hnode_new[i];
                float tup, tlo;
                if (nz == nzmin || nz == nzmax - 1) {
                    tup = tvmax[nz];
                    tlo = tvmin[nz];
                } else {
                    tup = fmaxf(fmaxf(tvmax[nz - 1], tvmax[nz]), tvmax[nz + 1]);
                    tlo = fminf(fminf(tvmin[nz - 1], tvmin[nz]), tvmin[nz + 1]);
                }
                const float bmx = tup - lo, bmn = tlo - lo;
                const float v0 = ADv[iN(nz, n, nl)], v1 = ADv[iN(nz + 1, n, nl)];
                Kahan P, M;
                P.add(fmaxf(0.f, v0) + fmaxf(0.f, -v1));
                M.add(fminf(0.f, v0) + fminf(0.f, -v1));
                for (int g0 = 0; g0 < deg; g0 += kU) {
                    float x[kU];
                    bool ok[kU];
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        const int j = g0 + u;
                        ok[u] = j < deg && nz >= S.lo[j] && nz <= S.hi[j];
                        x[u] = ok[u] ? ADh[i1(nz, S.e[j], L1)] : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        if (!ok[u]) continue;
                        const float xv = ((S.own >> (g0 + u)) & 1u) ? x[u] : -x[u];
                        P.add(fmaxf(0.f, xv));
                        M.add(fminf(0.f, xv));
                    }
                }
                const float s = dt / (g.areasvol[iN(nz, n, nl)] * g.hnode_new[i]);
                B.R[t * B.sN + i] = make_float2(fminf(1.f, bmx / (P.get() * s + eps)), fminf(1.f, bmn / (M.get() * s - eps)));
                // the bounds themselves: the update clamps the advected value into them, so
                // FP32 rounding in the limiter can never create a new extremum
                B.TB[t * B.sN + i] = make_float2(tup, tlo);
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// k32_update: limited update, T*, implicit vertical diffusion (warp scans)
// ---------------------------------------------------------------------------
// inclusive scan over lanes of affine maps y -> A*y + B, composed in lane order
__device__ __forceinline__ void scan_up(float &A, float &B, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float Ap = __shfl_up_sync(kFull, A, off), Bp = __shfl_up_sync(kFull, B, off);
        if (lane >= off) {
            B = A * Bp + B;
            A = A * Ap;
        }
    }
}
// the same, composed in reverse lane order (lane 31 first)
__device__ __forceinline__ void scan_down(float &A, float &B, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float An = __shfl_down_sync(kFull, A, off), Bn = __shfl_down_sync(kFull, B, off);
        if (lane + off < 32) {
            B = A * Bn + B;
            A = A * An;
        }
    }
}

__global__ void __launch_bounds__(kT)
k32_update(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, VFactors vf, float dt) {
    __shared__ NodeEdges S;
    extern __shared__ __align__(16) float sm32[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int L1 = tp.L1, nl = tp.nl;
    float *Ta = sm32 + (size_t)warp * (L1 + 2);
    for (int n = blockIdx.x; n < tp.N2; n += gridDim.x) {
        __syncthreads();
        stage_node(tp, n, S);
        __syncthreads();
        const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
        const int nch = (nzmax - nzmin + 31) / 32;
        for (int t = warp; t < B.ntr; t += kW) {
            const DCfg c = B.cfg[t];
            const int fct = c.lim;
            const float *T = B.T + t * B.sN;
            const float *ADv = B.ADv + t * B.sNI;
            const float *ADh = B.ADh + t * B.sE;
            const float2 *R = B.R + t * B.sN;
            float tadv[kMaxChunks];
#pragma unroll
            for (int ch = 0; ch < kMaxChunks; ch++) {
                const int nz = nzmin + 32 * ch + lane;
                tadv[ch] = 0.f;
                if (ch >= nch || nz > nzmax - 1) continue;
                const size_t i = i1(nz, n, L1);
                const float sdt = dt / g.areasvol[iN(nz, n, nl)];
                Kahan del;
                float f0 = ADv[iN(nz, n, nl)], f1 = ADv[iN(nz + 1, n, nl)];
                float2 r0 = make_float2(1.f, 1.f);
                if (fct) {
                    del.add(B.LOi[t * B.sN + i]);
                    r0 = R[i];
                    // vertical limiting (oce_adv_tra_fct.F90:425-456); the bottom interface is not limited
                    if (nz == nzmin) {
                        f0 *= f0 >= 0.f ? fminf(1.f, r0.x) : fminf(1.f, r0.y);
                    } else {
                        const float2 rm = R[i - 1];
                        f0 *= f0 >= 0.f ? fminf(fminf(1.f, rm.y), r0.x) : fminf(fminf(1.f, rm.x), r0.y);
                    }
                    if (nz + 1 <= nzmax - 1) {
                        const float2 rp = R[i + 1];
                        f1 *= f1 >= 0.f ? fminf(fminf(1.f, r0.y), rp.x) : fminf(fminf(1.f, r0.x), rp.y);
                    }
                }
                del.add(f0 * sdt);
                del.add(-(f1 * sdt));
                for (int g0 = 0; g0 < deg; g0 += kU) {
                    float x[kU];
                    float2 rm[kU];
                    bool ok[kU];
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        const int j = g0 + u;
                        ok[u] = j < deg && nz >= S.lo[j] && nz <= S.hi[j];
                        x[u] = ok[u] ? ADh[i1(nz, S.e[j], L1)] : 0.f;
                        rm[u] = (ok[u] && fct) ? R[i1(nz, S.m[j], L1)] : make_float2(1.f, 1.f);
                    }
#pragma unroll
                    for (int u = 0; u < kU; u++) {
                        if (!ok[u]) continue;
                        const bool own = (S.own >> (g0 + u)) & 1u;
                        float xv = x[u];
                        if (fct) {
                            // R of edges(1,e) and edges(2,e)
                            const float2 ra = own ? r0 : rm[u], rb = own ? rm[u] : r0;
                            xv *= xv >= 0.f ? fminf(fminf(1.f, ra.x), rb.y) : fminf(fminf(1.f, ra.y), rb.x);
                        }
                        del.add(own ? xv * sdt : -(xv * sdt));
                    }
                }
                del.add(T[i] * (g.hnode[i] - g.hnode_new[i]));
                float v = T[i] + del.get() / g.hnode_new[i];
                if (fct) {
                    const float2 tb = B.TB[t * B.sN + i];
                    const float vc = fminf(fmaxf(v, tb.y), tb.x);
                    // a clamp beyond round-off means the limiter itself failed
                    if (fabsf(vc - v) > 1e-5f * (tb.x - tb.y) + 1e-6f * fabsf(vc)) atomicOr(B.status, 2u);
                    v = vc;
                }
                tadv[ch] = v;
                Ta[nz] = v;
            }
            float *Tout = B.Tnew + t * B.sN;
            if (!c.ivd) {
#pragma unroll
                for (int ch = 0; ch < kMaxChunks; ch++) {
                    const int nz = nzmin + 32 * ch + lane;
                    if (ch < nch && nz <= nzmax - 1) {
                        Tout[i1(nz, n, L1)] = tadv[ch];
                        if (!isfinite(tadv[ch])) atomicOr(B.status, 1u);
                    }
                }
                __syncwarp();
                continue;
            }
            __syncwarp();
            // forward substitution: tp_k = inv_k*rhs_k - a_k*inv_k*tp_{k-1}
            float tpv[kMaxChunks];
            float carry = 0.f;
            const float bc = f.bc ? f.bc[(size_t)t * tp.N2 + n] : 0.f;
#pragma unroll
            for (int ch = 0; ch < kMaxChunks; ch++) {
                tpv[ch] = 0.f;
                if (ch >= nch) continue;
                const int nz = nzmin + 32 * ch + lane;
                float A = 1.f, Bv = 0.f;
                if (nz <= nzmax - 1) {
                    const size_t i = i1(nz, n, L1);
                    const float a = vf.a[i], cc = vf.c[i], inv = vf.inv[i];
                    const float t0 = tadv[ch];
                    float rhs = 0.f;
                    if (nz > nzmin) rhs -= a * (Ta[nz - 1] - t0);
                    if (nz < nzmax - 1) rhs -= cc * (Ta[nz + 1] - t0);
                    if (nz == nzmin) rhs += bc;
                    A = -(a * inv);
                    Bv = rhs * inv;
                }
                scan_up(A, Bv, lane);
                const float y = A * carry + Bv;
                tpv[ch] = y;
                carry = __shfl_sync(kFull, y, 31);
            }
            // back substitution: x_k = tp_k - cp_k * x_{k+1}
            carry = 0.f;
#pragma unroll
            for (int ch = kMaxChunks - 1; ch >= 0; ch--) {
                if (ch >= nch) continue;
                const int nz = nzmin + 32 * ch + lane;
                float A = 1.f, Bv = 0.f;
                if (nz <= nzmax - 1) {
                    A = -vf.cp[i1(nz, n, L1)];
                    Bv = tpv[ch];
                }
                scan_down(A, Bv, lane);
                const float x = A * carry + Bv;
                carry = __shfl_sync(kFull, x, 0);
                if (nz <= nzmax - 1) {
                    const float v = tadv[ch] + x;
                    Tout[i1(nz, n, L1)] = v;
                    if (!isfinite(v)) atomicOr(B.status, 1u);
                }
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
static int grid32(int nent, int per_block) {
    int b = (nent + per_block - 1) / per_block;
    const int cap = 152 * 48;
    return b > cap ? cap : (b < 1 ? 1 : b);
}

void b32_vflux(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, float *VF, cudaStream_t s) {
    k32_vflux<<<grid32(tp.E2, kW), kT, 0, s>>>(tp, g, f, VF);
}
void b32_vfactors(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, double dt, const VFactors &v,
                  cudaStream_t s) {
    k32_vfactors<<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, dt, v);
}
// node kernels: one block per node (grid-stride), the tracers split over the block's warps
static int grid_nodes(int n2) { return n2 < 152 * 32 ? n2 : 152 * 32; }

void b32_lo_ad(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, const MusclW &mw,
               const float *VF, double dt, cudaStream_t s) {
    k32_lo_ad<<<grid_nodes(tp.N2), kT, 0, s>>>(tp, g, f, B, mw, VF, (float)dt);
}
void b32_bounds(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, cudaStream_t s) {
    const size_t sm = sizeof(float) * 2 * (tp.L1 + 2) * kW;
    k32_bounds<<<grid_nodes(tp.N2), kT, sm, s>>>(tp, g, B, (float)dt);
}
void b32_update(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B,
                const VFactors &v, double dt, cudaStream_t s) {
    const size_t sm = sizeof(float) * (tp.L1 + 2) * kW;
    k32_update<<<grid_nodes(tp.N2), kT, sm, s>>>(tp, g, f, B, v, (float)dt);
}

}  // namespace fesom
