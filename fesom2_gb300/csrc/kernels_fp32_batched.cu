// kernels_fp32_batched.cu -- the FP32 batched form of the tracer step.
//
// All tracers of a launch group in one launch per stage, the whole step in one CUDA graph:
//
//   k32_vflux        edge volume fluxes per edge-layer (oce_adv_tra_hor.F90:159-250
//                    segment rule); shared by every tracer
//   k32_vfactors     FP64 factorisation of the implicit vertical-diffusion matrix of
//                    every column (oce_ale_tracer.F90:1088-1204, 1406-1414): the
//                    pivots m = b - cp*a carry the cancellation that thin bottom cells
//                    cause, so they are formed in FP64; stored as FP32 a, c, 1/m, c/m
//   k32_lo_ad        per node: the LO solution (edge gather of upwind fluxes + upwind
//                    vertical flux with w_e) and the vertical antidiffusive flux
//                    (QR4C / UPW1 / CDIFF on the AB values; PPM in k32_vppm)
//   k32_ho           per edge: the horizontal antidiffusive flux, MUSCL / MFCT / UPW1 on
//                    the AB values minus the upwind LO flux (k32_ho_nodemean: the few
//                    edge-layers whose gradients are node means)
//   k32_bounds       per node: FCT bounds (max/min of LO and T over the node's
//                    neighbours and the adjacent layers) and R+/R- (oce_adv_tra_fct.F90)
//   k32_update       per node: limited fluxes, flux divergence, T* update, written to
//                    the buffer of the oldest time level
//   k32_vdiff        per node: the implicit vertical diffusion as two warp scans of
//                    affine maps over the column (forward and back substitution with
//                    the FP64-formed factors)
//   k32_vppm, k32_lo_impl, k32_vdiff_w, k32_hdiff, k32_diff
//                    the optional parts: PPM vertical fluxes, the split vertical
//                    velocity, horizontal and explicit vertical diffusion
//
// Every tracer carries the same quantities whatever its limiter: the LO solution and
// the antidiffusive fluxes "high order minus low order" of the edges and interfaces.
// Without FCT the update adds them unlimited, which is the high-order flux divergence;
// with FCT it scales them by R+/R- first.
//
// Mapping of the node stages: one warp per node for all tracers of the launch.  The
// lanes cover a chunk of the node's column (one level per lane); consecutive chunks
// overlap by the halo levels each stage needs (the level above/below comes from the
// neighbouring lane through a shuffle), and the halo lanes compute but do not store.
// The last chunk of a column, when its levels fill at most half a warp, carries several
// tracers side by side in lane segments.  The node's edge list, the neighbour offsets
// and the tracer-independent geometry of a chunk sit in registers and serve every
// tracer, so per tracer a lane does only the gathers and the arithmetic of that tracer.
// Eight consecutive nodes per block (the node order is spatially local), so the
// neighbour columns a block gathers are mostly shared between its warps.
//
// Layout: tracer-major, column-contiguous per tracer (the reference's a(level, node)
// per tracer).  No atomics on values: each edge flux is written once and every node
// sum is a gather.  The Adams-Bashforth shift is a rotation of the time-level buffers
// (no copy).
#include <cuda_runtime.h>

#include "fesom_internal.h"

namespace fesom {

namespace {

constexpr int kWB = 8;                // warps (= nodes) per block
constexpr int kTB = 32 * kWB;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxChunks = 5;         // columns of up to 128 layers, 30 levels per chunk
// resident blocks per SM each tracer kernel is built for (3: <= 80 registers, 4: <= 64)
#ifndef FESOM_MINB_LO
#define FESOM_MINB_LO 3
#endif
#ifndef FESOM_MINB_HO
#define FESOM_MINB_HO 4
#endif
#ifndef FESOM_MINB_BOUNDS
#define FESOM_MINB_BOUNDS 4
#endif
#ifndef FESOM_MINB_UPDATE
#define FESOM_MINB_UPDATE 4
#endif
// tracers side by side in the last level chunk of a column in the multi-instance kernels too
#ifndef FESOM_PACK_MULTI
#define FESOM_PACK_MULTI true
#endif

__device__ __forceinline__ size_t i1(int nz, int n, int L1) { return (size_t)n * L1 + (nz - 1); }

// FP32 quotients of the node stages (geometry factors, limiter ratios): the fast division
// (2 ulp) instead of the correctly rounded one, 4-6 % of the bounds and lo_ad kernels' time;
// far inside the FP32 form's 1e-5, and the FCT clamp into the stored bounds keeps every
// result inside its bounds whatever the last bits of R+/R-
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }

}  // namespace

// ---------------------------------------------------------------------------
// k32_vflux: volume flux of every edge-layer (shared by all tracers)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void vflux_edge(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, float *VF,
                                           int e, int lane) {
    const int L1 = tp.L1;
    {
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

__global__ void __launch_bounds__(kTB) k32_vflux(DTopo tp, DGeom<float> g, DForcing<float> f, float *VF) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int e = blockIdx.x * kWB + warp; e < tp.E2; e += gridDim.x * kWB) vflux_edge(tp, g, f, VF, e, lane);
}

// ---------------------------------------------------------------------------
// k32_vfactors: FP64 factorisation of each column's tridiagonal system
// ---------------------------------------------------------------------------
// a(k) = -Kv(k) dt/(Z_n(k-1)-Z_n(k)) area(k)/areasvol(k), c(k) = -Kv(k+1) dt/(Z_n(k)-Z_n(k+1))
// area(k+1)/areasvol(k), b = -a - c + hnode_new (oce_ale_tracer.F90:1099-1204), with
// Z_n(k)-Z_n(k+1) = (hnode_new(k) + hnode_new(k+1))/2 (the mid-depths of :1088-1096);
// Thomas pivots m(k) = b(k) - cp(k-1) a(k), cp(k) = c(k)/m(k) (:1406-1414).
// a, b, c are formed in FP32 and used with those rounded values throughout, so all
// factors belong to one consistent system; the pivot recurrence, where thin bottom
// cells cancel most bits, runs in FP64.  One thread per column runs the recurrence; the block's columns move through shared
// memory in tiles of kVfK levels, loaded and stored with the lanes over the levels of a
// column (each column's tile is one contiguous run), so no thread walks its own column
// through the cache.
constexpr int kVfK = 8;       // levels per tile
__device__ __forceinline__ void vfactors_block(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                               double dt, const VFactors &vf, int blk) {
    // inputs for levels lev0 .. lev0 + kVfK (one extra: the next level's h, Kv, area);
    // outputs for levels lev0 .. lev0 + kVfK - 1
    __shared__ float s_hn[kVfCols][kVfK + 1], s_ar[kVfCols][kVfK + 1], s_av[kVfCols][kVfK + 1],
        s_kv[kVfCols][kVfK + 1];
    __shared__ float s_a[kVfCols][kVfK], s_c[kVfCols][kVfK], s_i[kVfCols][kVfK], s_p[kVfCols][kVfK];
    __shared__ int s_lmax;
    const int L1 = tp.L1, nl = tp.nl;
    const int c0 = blk * kVfCols, tid = threadIdx.x;
    const int ncol = min(kVfCols, tp.N2 - c0);
    const int n = c0 + tid;
    const bool mine = tid < ncol;
    const int nzmin = mine ? tp.n_ulev[n] : 1, nzmax = mine ? tp.n_nlev[n] : 1;
    if (tid == 0) s_lmax = 0;
    __syncthreads();
    if (mine) atomicMax(&s_lmax, nzmax - 1);
    __syncthreads();
    const int lmax = s_lmax;
    int lmin = 1 << 30;
    // the first tile starts at the block's shallowest top layer
    {
        __shared__ int s_lmin;
        if (tid == 0) s_lmin = 1 << 30;
        __syncthreads();
        if (mine) atomicMin(&s_lmin, nzmin);
        __syncthreads();
        lmin = s_lmin;
    }
    const float dtf = (float)dt;
    double cp = 0.0;
    float zinv1 = 0.f, hcur = 0.f;
    for (int lev0 = lmin; lev0 <= lmax; lev0 += kVfK) {
        // load: item q = column * (kVfK + 1) + k, consecutive threads on consecutive levels
        for (int q = tid; q < ncol * (kVfK + 1); q += kVfCols) {
            const int col = q / (kVfK + 1), k = q - col * (kVfK + 1);
            const int lev = lev0 + k, cn = c0 + col;
            float hv = 0.f, arv = 0.f, avv = 0.f, kvv = 0.f;
            if (lev <= L1) hv = g.hnode_new[(size_t)cn * L1 + lev - 1];
            if (lev <= nl) {
                const size_t iv = (size_t)cn * nl + lev - 1;
                arv = g.area[iv];
                avv = g.areasvol[iv];
                kvv = f.Kv[iv];
            }
            s_hn[col][k] = hv;
            s_ar[col][k] = arv;
            s_av[col][k] = avv;
            s_kv[col][k] = kvv;
        }
        __syncthreads();
        if (mine) {
            for (int k = 0; k < kVfK; k++) {
                const int nz = lev0 + k;
                float oa = 0.f, oc = 0.f, oi = 0.f, ocp = 0.f;
                if (nz >= nzmin && nz <= nzmax - 1) {
                    if (nz == nzmin) hcur = s_hn[tid][k];
                    const float hnext = nz < nzmax - 1 ? s_hn[tid][k + 1] : 0.f;
                    const float ravz = 1.f / s_av[tid][k];
                    const float a = nz > nzmin ? -(s_kv[tid][k] * zinv1 * dtf * (s_ar[tid][k] * ravz)) : 0.f;
                    float c = 0.f, zinv2 = 0.f;
                    if (nz < nzmax - 1) {
                        zinv2 = 2.f / (hcur + hnext);
                        c = -(s_kv[tid][k + 1] * zinv2 * dtf * s_ar[tid][k + 1] * ravz);
                    }
                    // pivot recurrence in FP64 on the FP32-rounded coefficients; 1/m from an FP32
                    // reciprocal and one Newton-Raphson step r = r0 (2 - m r0)
                    const double ad = (double)a;
                    const double m = ((double)(-a - c) + (double)hcur) - cp * ad;
                    const double r0 = (double)__frcp_rn((float)m);
                    const double r = r0 * (2.0 - m * r0);
                    cp = (double)c * r;
                    oa = a;
                    oc = c;
                    oi = (float)r;
                    ocp = (float)cp;
                    zinv1 = zinv2;
                    hcur = hnext;
                }
                s_a[tid][k] = oa;
                s_c[tid][k] = oc;
                s_i[tid][k] = oi;
                s_p[tid][k] = ocp;
            }
        }
        __syncthreads();
        for (int q = tid; q < ncol * kVfK; q += kVfCols) {
            const int col = q / kVfK, k = q - col * kVfK;
            const int lev = lev0 + k, cn = c0 + col;
            if (lev > L1) continue;
            const size_t i = (size_t)cn * L1 + lev - 1;
            vf.a[i] = s_a[col][k];
            vf.c[i] = s_c[col][k];
            vf.inv[i] = s_i[col][k];
            vf.cp[i] = s_p[col][k];
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kVfCols) k32_vfactors(DTopo tp, DGeom<float> g, DForcing<float> f, double dt,
                                                        VFactors vf) {
    vfactors_block(tp, g, f, dt, vf, blockIdx.x);
}

// ---------------------------------------------------------------------------
// per-warp staging of the node's edge list (one warp per node)
// ---------------------------------------------------------------------------
struct WEdges {
    int e[kMaxDeg], m[kMaxDeg], lo[kMaxDeg], hi[kMaxDeg];
    unsigned own;  // bit j: the node is edges(1, e_j) (it owns the edge flux)
    int deg, nzmin, nzmax;
};

__device__ __forceinline__ void stage_edges(const DTopo &tp, int n, int lane, WEdges &S) {
    const int k0 = tp.ne_ptr[n];
    const int deg = min(tp.ne_ptr[n + 1] - k0, kMaxDeg);
    int code = 0;
    if (lane < deg) {
        code = tp.ne_idx[k0 + lane];
        const int e = code >= 0 ? code : ~code;
        S.e[lane] = e;
        S.m[lane] = code >= 0 ? tp.e_n2[e] : tp.e_n1[e];
        S.lo[lane] = tp.e_lo[e];
        S.hi[lane] = tp.e_hi[e];
    }
    const unsigned own = __ballot_sync(kFull, lane < deg && code >= 0);
    if (lane == 0) {
        S.own = own;
        S.deg = deg;
        S.nzmin = tp.n_ulev[n];
        S.nzmax = tp.n_nlev[n];
    }
    __syncwarp();
}

// chunk ch of a column, HU halo levels above and HD below the stored levels
template <int HU, int HD>
struct Chunk {
    static constexpr int OUT = 32 - HU - HD;
    int nz;
    int q = 0;  // tracer slot of the lane (packed chunks)
    bool lvl, out;
    __device__ __forceinline__ Chunk(int nzmin, int nzmax, int ch, int lane) {
        nz = nzmin - HU + OUT * ch + lane;
        lvl = nz >= nzmin && nz <= nzmax - 1;
        out = lvl && lane >= HU && lane < 32 - HD;
    }
    // the last chunk of a column in P segments of W = (its levels + HU + HD) lanes, one
    // tracer per segment: segment q holds the lanes [q W, (q + 1) W), laid out as a whole
    // chunk, so the vertical shuffles of a stored lane stay inside its segment
    __device__ __forceinline__ Chunk(int nzmin, int nzmax, int ch, int lane, int W, int P) {
        q = lane / W;
        const int l = lane - q * W;
        nz = nzmin - HU + OUT * ch + l;
        lvl = q < P && nz >= nzmin && nz <= nzmax - 1;
        out = lvl && l >= HU && l < W - HD;
    }
    static __device__ __forceinline__ int count(int nzmin, int nzmax) { return (nzmax - nzmin + OUT - 1) / OUT; }
    // segments of the last chunk: its width, and how many fit a warp (1: not packed)
    static __device__ __forceinline__ int last_width(int nzmin, int nzmax) {
        const int nl = nzmax - nzmin;
        return nl - OUT * (count(nzmin, nzmax) - 1) + HU + HD;
    }
};

__device__ __forceinline__ float sh_up(float v, int d) { return __shfl_up_sync(kFull, v, d); }
__device__ __forceinline__ float sh_dn(float v, int d) { return __shfl_down_sync(kFull, v, d); }

// Adams-Bashforth value minus the current value: AB2 -(0.5+eps) T^{n-1} + (1.5+eps) T^n,
// AB3 (23 T^n - 16 T^{n-1} + 5 T^{n-2}) / 12 (oce_tracer_mod.F90:53, 67-68), eps = 0.1
__device__ __forceinline__ float ab_delta(int ab, float t, float o1, float o2) {
    return ab == 2 ? 0.6f * (t - o1) : (11.f * (t - o1) - 5.f * (o1 - o2)) * (1.f / 12.f);
}



// ---------------------------------------------------------------------------
// k32_lo_ad
// ---------------------------------------------------------------------------
// One chunk of a node's column for every tracer of the launch.  PACK: the column's last
// chunk with P tracers side by side in segments of W lanes; otherwise one tracer at a time
// over the whole warp.
template <int KD, bool WS, bool PACK>
__device__ __forceinline__ void lo_ad_chunk(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                            const B32View &B, const float *__restrict__ VF, float dt, int n, int lane,
                                            const WEdges &S, int ch, int W, int P) {
    using C = Chunk<2, 1>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    {
        const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
        const int nz = k.nz;
        const int i = n * L1 + nz - 1;   // layer nz of the node (valid where k.lvl)
        const int iv = n * nl + nz - 1;  // interface nz
        // ---- tracer-independent part of the chunk ----
        int off[KD];
        float am[KD];  // upwind inflow weight of each edge slot (0 where the slot is dry)
        unsigned okm = 0;
        float Dh = 0.f;  // net horizontal volume flux into the node
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
            off[u] = S.m[u] * L1 + nz - 1;
            const float v = ok ? VF[S.e[u] * L1 + nz - 1] : 0.f;
            okm |= ok ? 1u << u : 0u;
            const bool ow = (own >> u) & 1u;
            Dh += ow ? -v : v;
            am[u] = ow ? -fminf(v, 0.f) : fmaxf(v, 0.f);
        }
        float ar0 = 0.f, we0 = 0.f, w0 = 0.f, sdt = 0.f, Z0 = 0.f, hr = 0.f;
        if (k.lvl) {
            ar0 = g.area[iv];
            we0 = f.we[iv];
            w0 = f.w[iv];
            const float ihn = qdiv(1.f, g.hnode_new[i]);
            sdt = qdiv(dt, g.areasvol[iv]) * ihn;
            hr = g.hnode[i] * ihn;
            Z0 = g.Z3[i];
        }
        const float Zm1 = sh_up(Z0, 1), Zm2 = sh_up(Z0, 2), Zp1 = sh_dn(Z0, 1);
        // QR4C interior geometry, nzmin+2 <= nz <= nzmax-2 (oce_adv_tra_ver.F90:409-425)
        const bool qint = k.out && nz >= nzmin + 2 && nz <= nzmax - 2;
        float idz0 = 0.f, idzp = 0.f, idzm = 0.f, g1 = 0.f, g2 = 0.f;
        if (qint) {
            const float zb = g.zbar3[iv];
            idz0 = qdiv(1.f, Zm1 - Z0);
            idzp = qdiv(1.f, Z0 - Zp1);
            idzm = qdiv(1.f, Zm2 - Zm1);
            g1 = (zb - Z0) * (1.f / 3.f);
            g2 = (zb - Zm1) * (1.f / 3.f);
        }
        const bool twolayer = nzmin + 1 == nzmax - 1;
        // ---- per tracer ----
#pragma unroll 1
        for (int t0 = 0; t0 < B.ntr; t0 += PACK ? P : 1) {
            // the lane's tracer (packed: the tracer of its segment; idle past the last)
            const int tt = t0 + k.q;
            const bool on = tt < B.ntr;
            const int t = on ? tt : t0;
            const bool lvt = k.lvl && on;
            const unsigned okt = lvt ? okm : 0u;
            const bool lim = (B.fct_mask >> t) & 1ull;
            const int ver = B.ver[t];
            const size_t to = (size_t)t * B.sN;
            const float *__restrict__ T = B.T + to;
            const float *__restrict__ O1 = B.O1 + to;
            const float *__restrict__ O2 = B.ab == 3 ? B.O2 + to : O1;
            // every load of the tracer's chunk first
            const float Tn = lvt ? T[i] : 0.f;
            const float o1 = lvt ? O1[i] : 0.f;
            const float o2 = (lvt && B.ab == 3) ? O2[i] : 0.f;
            float tm[KD];
#pragma unroll
            for (int u = 0; u < KD; u++) tm[u] = ((okt >> u) & 1u) ? T[off[u]] : 0.f;
            const float tab = Tn + (lvt ? ab_delta(B.ab, Tn, o1, o2) : 0.f);
            const float Tu = sh_up(Tn, 1);
            const float tabu = sh_up(tab, 1), tabu2 = sh_up(tab, 2), tabd = sh_dn(tab, 1);
            // LO: upwind edge fluxes in difference form, sum_j am_j (T_j - T_n) + Dh T_n
            float hs = Dh * Tn;
#pragma unroll
            for (int u = 0; u < KD; u++)
                if ((okt >> u) & 1u) hs += am[u] * (tm[u] - Tn);
            // upwind vertical flux with w_e at interface nz (adv_tra_ver_upw1)
            float fv0 = 0.f;
            if (lvt) {
                if (nz == nzmin) {
                    fv0 = -(we0 * Tn * ar0);
                } else {
                    const float aw = fabsf(we0);
                    fv0 = -(0.5f * (Tn * (we0 + aw) + Tu * (we0 - aw)) * ar0);
                }
            }
            float fv1 = sh_dn(fv0, 1);
            if (nz == nzmax - 1) fv1 = 0.f;
            // LO = (T hnode + flux divergence dt / areasvol) / hnode_new (oce_adv_tra_driver.F90:249)
            if (k.out && on) B.LO[to + i] = Tn * hr + (hs + fv0 - fv1) * sdt;
            // with the split vertical velocity the LO part of the antidiffusive flux is the upwind
            // flux of the full w (oce_adv_tra_driver.F90:323-334)
            float fw0 = fv0;
            if (WS && f.wsplit && lvt) {
                if (nz == nzmin) {
                    fw0 = -(w0 * Tn * ar0);
                } else {
                    const float aw = fabsf(w0);
                    fw0 = -(0.5f * (Tn * (w0 + aw) + Tu * (w0 - aw)) * ar0);
                }
            }
            // vertical high-order flux on the AB values (QR4C / UPW1 / CDIFF; PPM in k32_vppm),
            // minus the LO flux
            if (k.out && on && ver != 3) {
                const float pw = lim ? w0 : we0;
                float Cf;
                if (nz == nzmin) {
                    Cf = -(tab * pw * ar0);
                } else if (ver != 0 || nz == nzmin + 1 || nz == nzmax - 1) {
                    if (ver != 1) {  // QR4C next to the ends, CDIFF everywhere
                        Cf = -(0.5f * (tabu + tab) * pw * ar0);
                    } else {
                        const float aw = fabsf(pw);
                        Cf = -(0.5f * (tab * (pw + aw) + tabu * (pw - aw)) * ar0);
                    }
                } else {
                    const float qc = (tabu - tab) * idz0;
                    const float qu = (tab - tabd) * idzp;
                    const float qd = (tabu2 - tabu) * idzm;
                    const float Tm1 = tab + (2.f * qc + qu) * g1;
                    const float Tm2 = tabu + (2.f * qc + qd) * g2;
                    const float aw = fabsf(pw), no = B.pv[t];
                    const float Tmean = (pw + aw) * Tm1 + (pw - aw) * Tm2;
                    Cf = (-(0.5f * (1.f - no) * Tmean) - no * (0.5f * (Tm1 + Tm2)) * pw) * ar0;
                }
                // flux = C - flux_in; FCT passes the LO flux in, otherwise zero
                const float fin = lim ? fw0 : 0.f;
                float F = Cf - fin;
                // a two-layer column writes its middle interface twice (statements nzmin+1, nzmax-1)
                if (ver == 0 && twolayer && nz == nzmin + 1) F = Cf - F;
                B.ADv[(size_t)t * B.sNI + iv] = lim ? F : F - fv0;
            }
        }
    }
}

template <int KD, bool WS, bool PK>
__device__ __forceinline__ void lo_ad_node(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                           const B32View &B, const float *__restrict__ VF, float dt, int n, int lane,
                                           const WEdges &S) {
    using C = Chunk<2, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    for (int ch = 0; ch < nch - 1; ch++) lo_ad_chunk<KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, ch, 32, 1);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    // packed only for nodes of at most 6 edges, as in k32_bounds
    if (PK && KD <= 6 && P > 1) lo_ad_chunk<KD, WS, true>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, W, P);
    else lo_ad_chunk<KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, 32, 1);
}

// the node of warp unit j: consecutive nodes, or (WIDE) the listed nodes of more than 8 edges
template <bool WIDE>
__device__ __forceinline__ int unit_node(const DTopo &tp, int j) {
    if (WIDE) return j < tp.n_wide ? tp.wide_nodes[j] : -1;
    return j < tp.N2 ? j : -1;
}

// WS: the split vertical velocity (a separate instantiation keeps the default path unchanged)
template <bool WIDE, bool WS, bool PK>
__device__ __forceinline__ void lo_ad_unit(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                           const B32View &B, const float *__restrict__ VF, float dt, int j, WEdges *Se) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) lo_ad_node<kMaxDeg, WS, PK>(tp, g, f, B, VF, dt, n, lane, S);
    else if (S.deg <= 6) lo_ad_node<6, WS, PK>(tp, g, f, B, VF, dt, n, lane, S);
    else lo_ad_node<8, WS, PK>(tp, g, f, B, VF, dt, n, lane, S);
}

template <bool WIDE, bool WS>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_LO)
k32_lo_ad(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, const float *__restrict__ VF, float dt) {
    __shared__ WEdges Se[kWB];
    lo_ad_unit<WIDE, WS, true>(tp, g, f, B, VF, dt, blockIdx.x * kWB + (threadIdx.x >> 5), Se);
}

// high-order minus low-order flux of one edge-layer from the two end values, their
// previous time levels and the projected gradients s1 (up) / s2 (down)
__device__ __forceinline__ float ho_minus_lo(int hor, float ph, int ab, float T1, float T2, float o1a, float o1b,
                                             float o2a, float o2b, float s1, float s2, float v, float cl1, float cl2) {
    const float vp = fmaxf(v, 0.f), vm = fminf(v, 0.f);
    const float t1 = T1 + ab_delta(ab, T1, o1a, o2a);
    const float t2 = T2 + ab_delta(ab, T2, o1b, o2b);
    const float flo = -(T1 * vp + T2 * vm);
    float hf;
    if (hor == 2) {
        hf = -(t1 * vp + t2 * vm);
    } else {
        // c_lo = 1 up to nboundary_lay (MUSCL), always 1 (MFCT)
        const float clo1 = hor == 0 ? cl1 : 1.f, clo2 = hor == 0 ? cl2 : 1.f;
        const float d2 = 2.f * (t2 - t1);
        const float Tm2 = t2 - (d2 + s2) * (1.f / 6.f) * clo2;
        const float Tm1 = t1 + (d2 + s1) * (1.f / 6.f) * clo1;
        const float cHO = 2.f * (vp * Tm1 + vm * Tm2);
        hf = -(0.5f * (1.f - ph) * cHO) - v * ph * 0.5f * (Tm1 + Tm2);
    }
    return hf - flo;
}

// ---------------------------------------------------------------------------
// k32_ho: high-order minus low-order flux of every edge-layer
// ---------------------------------------------------------------------------
// One warp per edge, the lanes over the edge's levels [nu12, nl12].  MUSCL / MFCT
// (adv_tra_hor_muscl / _mfct, oce_adv_tra_hor.F90:261-834) on the AB values with the
// gradients of fill_up_dn_grad (oce_muscl_adv.F90:356-525); UPW1 (:64-257).  The LO
// flux is the upwind flux of the current values (oce_adv_tra_driver.F90:131-190).
//
// The up triangle holds edges(1,e) and the down triangle edges(2,e); their gradients,
// projected on the edge, are wu.y (T(un.y) - T1) + wu.z (T(un.z) - T1) and the same
// for the down triangle (the three weights of a triangle sum to zero).  Those apply
// at the levels where every element around both nodes is wet, [gzmin, gzmax); the
// other edge-layers (under one percent of an ocean mesh's) take the node means in
// k32_ho_nodemean.
//
// A pass covers 32 levels of the edge; the last pass, when its levels fill at most half a
// warp, carries P tracers side by side in segments of W lanes (PACK).
template <bool PACK>
__device__ __forceinline__ void ho_pass(const DTopo &tp, const B32View &B, const MusclW &mw,
                                        const float *__restrict__ VF, int e, int nz0, int W, int P, int lane) {
    const int L1 = tp.L1;
    const int n1 = tp.e_n1[e], n2 = tp.e_n2[e];
    const int ehi = tp.e_hi[e];
    const int nbl1 = tp.n_nbl[n1], nbl2 = tp.n_nbl[n2];
    const int4 un = mw.un[e], dn = mw.dn[e];
    const float4 wu = mw.wu[e], wd = mw.wd[e];
    const int gzmin = un.w & 0xffff, gzmax = un.w >> 16;
    const int q = PACK ? lane / W : 0;
    const int nz = nz0 + lane - q * W;
    const bool tri = nz >= gzmin && nz <= gzmax - 1;
    const bool ok = nz <= ehi && q < P;
    const int ie = e * L1 + nz - 1, ia = n1 * L1 + nz - 1, ib = n2 * L1 + nz - 1;
    const float v = ok ? VF[ie] : 0.f;
    const float cl1 = (nbl1 - nz) >= 0 ? 1.f : 0.f, cl2 = (nbl2 - nz) >= 0 ? 1.f : 0.f;
    const int ua = un.y * L1 + nz - 1, ub = un.z * L1 + nz - 1;
    const int da = dn.y * L1 + nz - 1, db = dn.z * L1 + nz - 1;
    if (!ok) return;
    // two tracers per pass: their gathers in flight together (packed: tracers t0 + q and
    // t0 + P + q of the segment)
    const int step = PACK ? P : 1;
#pragma unroll 1
    for (int t0 = 0; t0 < B.ntr; t0 += 2 * step) {
        float T1[2], T2[2], o1a[2], o1b[2], o2a[2], o2b[2], ga[2], gb[2], gc[2], gd[2];
        bool grad[2], on[2];
        int tt[2];
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int tq = t0 + r * step + q;
            on[r] = tq < B.ntr;
            tt[r] = on[r] ? tq : t0;
            const size_t to = (size_t)tt[r] * B.sN;
            const float *__restrict__ T = B.T + to;
            grad[r] = on[r] && B.hor[tt[r]] != 2 && tri;
            T1[r] = on[r] ? T[ia] : 0.f;
            T2[r] = on[r] ? T[ib] : 0.f;
            o1a[r] = on[r] ? B.O1[to + ia] : 0.f;
            o1b[r] = on[r] ? B.O1[to + ib] : 0.f;
            o2a[r] = (on[r] && B.ab == 3) ? B.O2[to + ia] : 0.f;
            o2b[r] = (on[r] && B.ab == 3) ? B.O2[to + ib] : 0.f;
            ga[r] = grad[r] ? T[ua] : 0.f;
            gb[r] = grad[r] ? T[ub] : 0.f;
            gc[r] = grad[r] ? T[da] : 0.f;
            gd[r] = grad[r] ? T[db] : 0.f;
        }
#pragma unroll
        for (int r = 0; r < 2; r++) {
            if (!on[r]) continue;
            const int hor = B.hor[tt[r]];
            // MUSCL / MFCT levels outside the triangles' range: the fallback launch
            if (hor != 2 && !tri) continue;
            const float s1 = wu.y * (ga[r] - T1[r]) + wu.z * (gb[r] - T1[r]);
            const float s2 = wd.y * (gc[r] - T2[r]) + wd.z * (gd[r] - T2[r]);
            B.ADh[(size_t)tt[r] * B.sE + ie] = ho_minus_lo(hor, B.ph[tt[r]], B.ab, T1[r], T2[r], o1a[r], o1b[r],
                                                           o2a[r], o2b[r], s1, s2, v, cl1, cl2);
        }
    }
}

template <bool PK>
__device__ __forceinline__ void ho_unit(const DTopo &tp, const B32View &B, const MusclW &mw,
                                        const float *__restrict__ VF, int e) {
    const int lane = threadIdx.x & 31;
    if (e >= tp.E2) return;
    const int elo = tp.e_lo[e], ehi = tp.e_hi[e];
    int nz0 = elo;
    for (; nz0 + 32 <= ehi; nz0 += 32) ho_pass<false>(tp, B, mw, VF, e, nz0, 32, 1, lane);
    const int W = ehi - nz0 + 1;
    if (W < 1) return;
    const int P = 32 / W;
    if (PK && P > 1) ho_pass<true>(tp, B, mw, VF, e, nz0, W, P, lane);
    else ho_pass<false>(tp, B, mw, VF, e, nz0, 32, 1, lane);
}

__global__ void __launch_bounds__(kTB, FESOM_MINB_HO)
k32_ho(DTopo tp, B32View B, MusclW mw, const float *__restrict__ VF) {
    ho_unit<true>(tp, B, mw, VF, blockIdx.x * kWB + (threadIdx.x >> 5));
}

// The edge-layers of the node-mean gradients: one thread per (edge, level) item, every
// tracer, with the projected mean gradients as precomputed neighbour weights.
__device__ __forceinline__ void nodemean_item(const DTopo &tp, const B32View &B, const MusclW &mw,
                                              const float *__restrict__ VF, int j) {
    const int L1 = tp.L1;
    {
        const int e = mw.it_e[j], nz = mw.it_nz[j];
        const int p0 = mw.it_ptr[j], p1 = p0 + mw.it_n1[j], p2 = mw.it_ptr[j + 1];
        const int n1 = tp.e_n1[e], n2 = tp.e_n2[e];
        const int ie = e * L1 + nz - 1, ia = n1 * L1 + nz - 1, ib = n2 * L1 + nz - 1;
        const float v = VF[ie];
        const float cl1 = (tp.n_nbl[n1] - nz) >= 0 ? 1.f : 0.f, cl2 = (tp.n_nbl[n2] - nz) >= 0 ? 1.f : 0.f;
#pragma unroll 1
        for (int t = 0; t < B.ntr; t++) {
            const int hor = B.hor[t];
            if (hor == 2) continue;  // UPW1 has no gradients: k32_ho wrote it
            const size_t to = (size_t)t * B.sN;
            const float *__restrict__ T = B.T + to;
            const float T1 = T[ia], T2 = T[ib];
            const float o1a = B.O1[to + ia], o1b = B.O1[to + ib];
            const float o2a = B.ab == 3 ? B.O2[to + ia] : 0.f, o2b = B.ab == 3 ? B.O2[to + ib] : 0.f;
            float s1 = 0.f, s2 = 0.f;
            for (int p = p0; p < p1; p++) {
                const int2 q = mw.pairs[p];
                s1 += __int_as_float(q.y) * (T[q.x * L1 + nz - 1] - T1);
            }
            for (int p = p1; p < p2; p++) {
                const int2 q = mw.pairs[p];
                s2 += __int_as_float(q.y) * (T[q.x * L1 + nz - 1] - T2);
            }
            B.ADh[(size_t)t * B.sE + ie] = ho_minus_lo(hor, B.ph[t], B.ab, T1, T2, o1a, o1b, o2a, o2b, s1, s2, v, cl1, cl2);
        }
    }
}

__global__ void __launch_bounds__(256) k32_ho_nodemean(DTopo tp, B32View B, MusclW mw, const float *__restrict__ VF) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < mw.n_items; j += gridDim.x * blockDim.x)
        nodemean_item(tp, B, mw, VF, j);
}

// ---------------------------------------------------------------------------
// k32_bounds: FCT bounds and R+ / R- (FCT tracers only)
// ---------------------------------------------------------------------------
// One chunk of a node's column for the FCT tracers of the launch.  PACK: the column's last
// chunk with P tracers side by side in segments of W lanes (its few levels would leave most
// lanes idle); otherwise one tracer at a time over the whole warp.
template <int KD, bool PACK>
__device__ __forceinline__ void bounds_chunk(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int n,
                                             int lane, const WEdges &S, int ch, int W, int P) {
    using C = Chunk<1, 1>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const float eps = (float)kFluxEps;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
    int off[KD];
    unsigned okm = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = S.m[u] * L1 + nz - 1;
        okm |= ok ? 1u << u : 0u;
    }
    const float s = k.lvl ? qdiv(dt, g.areasvol[iv] * g.hnode_new[i]) : 0.f;
    unsigned long long todo = B.fct_mask & (B.ntr >= 64 ? ~0ull : ((1ull << B.ntr) - 1));
    int t0 = 0;
    while (PACK ? t0 < B.ntr : todo != 0ull) {
        // the lane's tracer: the next FCT tracer, or (packed) tracer t0 + q of the segment,
        // idle where that tracer has no FCT
        int t;
        if (PACK) {
            t = t0 + k.q;
            if (t >= B.ntr || !((B.fct_mask >> t) & 1ull)) t = -1;
            t0 += P;
        } else {
            t = __ffsll((long long)todo) - 1;
            todo &= todo - 1;
        }
        const bool lv = k.lvl && t >= 0;
        const unsigned okt = lv ? okm : 0u;
        const size_t to = (size_t)(t < 0 ? 0 : t) * B.sN;
        const float *__restrict__ T = B.T + to;
        const float *__restrict__ LO = B.LO + to;
        const float *__restrict__ ADh = B.ADh + (size_t)(t < 0 ? 0 : t) * B.sE;
        // every load of the tracer's chunk first
        const float Tn = lv ? T[i] : 0.f;
        const float lo = lv ? LO[i] : 0.f;
        const float v0 = lv ? B.ADv[(size_t)(t < 0 ? 0 : t) * B.sNI + iv] : 0.f;
        float tm[KD], lm[KD], x[KD];
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = (okt >> u) & 1u;
            tm[u] = ok ? T[off[u]] : 0.f;
            lm[u] = ok ? LO[off[u]] : 0.f;
            // packed chunks: the edge fluxes after the bounds (fewer values live at once)
            if (!PACK) x[u] = ok ? ADh[S.e[u] * L1 + nz - 1] : 0.f;
        }
        // bounds over the node, its neighbours and the layers above and below
        // (oce_adv_tra_fct.F90:124-248)
        float mx = fmaxf(lo, Tn), mn = fminf(lo, Tn);
        float Pp = 0.f, M = 0.f;
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = (okt >> u) & 1u;
            const float a = ok ? tm[u] : Tn, b = ok ? lm[u] : lo;
            mx = fmaxf(mx, fmaxf(a, b));
            mn = fminf(mn, fminf(a, b));
        }
        if (PACK) {
#pragma unroll
            for (int u = 0; u < KD; u++) x[u] = ((okt >> u) & 1u) ? ADh[S.e[u] * L1 + nz - 1] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const float xv = ((own >> u) & 1u) ? x[u] : -x[u];
            Pp += fmaxf(0.f, xv);
            M += fminf(0.f, xv);
        }
        const float mxu = sh_up(mx, 1), mxd = sh_dn(mx, 1), mnu = sh_up(mn, 1), mnd = sh_dn(mn, 1);
        float tup = mx, tlo = mn;
        if (nz != nzmin && nz != nzmax - 1) {
            tup = fmaxf(fmaxf(mxu, mx), mxd);
            tlo = fminf(fminf(mnu, mn), mnd);
        }
        // P / M: sums of the positive / negative antidiffusive fluxes into the node
        float v1 = sh_dn(v0, 1);
        if (nz == nzmax - 1) v1 = 0.f;
        Pp += fmaxf(0.f, v0) + fmaxf(0.f, -v1);
        M += fminf(0.f, v0) + fminf(0.f, -v1);
        if (k.out && t >= 0) {
            const float bmx = tup - lo, bmn = tlo - lo;
            B.R[to + i] = make_float2(fminf(1.f, qdiv(bmx, Pp * s + eps)), fminf(1.f, qdiv(bmn, M * s - eps)));
            // the bounds themselves: the update clamps the advected value into them, so
            // FP32 rounding in the limiter can never create a new extremum
            B.TB[to + i] = make_float2(tup, tlo);
        }
    }
}

template <int KD, bool PK>
__device__ __forceinline__ void bounds_node(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int n,
                                            int lane, const WEdges &S) {
    using C = Chunk<1, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    for (int ch = 0; ch < nch - 1; ch++) bounds_chunk<KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    // packed only for nodes of at most 6 edges (nearly all of an ocean mesh's): the wider
    // packed body would spill registers
    if (PK && KD <= 6 && P > 1) bounds_chunk<KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P);
    else bounds_chunk<KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1);
}

template <bool WIDE, bool PK>
__device__ __forceinline__ void bounds_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                            WEdges *Se) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) bounds_node<kMaxDeg, PK>(tp, g, B, dt, n, lane, S);
    else if (S.deg <= 6) bounds_node<6, PK>(tp, g, B, dt, n, lane, S);
    else bounds_node<8, PK>(tp, g, B, dt, n, lane, S);
}

template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_BOUNDS) k32_bounds(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ WEdges Se[kWB];
    bounds_unit<WIDE, true>(tp, g, B, dt, blockIdx.x * kWB + (threadIdx.x >> 5), Se);
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

template <int KD, bool PACK>
__device__ __forceinline__ void update_chunk(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt,
                                             int n, int lane, const WEdges &S, int ch, int W, int P) {
    using C = Chunk<1, 1>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
    const float sdt = k.lvl ? qdiv(dt, g.areasvol[iv] * g.hnode_new[i]) : 0.f;
    unsigned okm = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        okm |= ok ? 1u << u : 0u;
    }
#pragma unroll 1
    for (int t0 = 0; t0 < B.ntr; t0 += PACK ? P : 1) {
        // the lane's tracer (packed: the tracer of its segment)
        const int t = t0 + k.q;
        const bool on = t < B.ntr;
        const int tc = on ? t : t0;
        const bool fct = (B.fct_mask >> tc) & 1ull;
        const size_t to = (size_t)tc * B.sN;
        const float *__restrict__ ADh = B.ADh + (size_t)tc * B.sE;
        const float2 *__restrict__ R = B.R + to;
        const bool lv = k.lvl && on;
        const bool lf = lv && fct;
        const unsigned okt = lv ? okm : 0u;
        // every load of the tracer's chunk first
        const float lo = lv ? B.LO[to + i] : 0.f;
        float f0 = lv ? B.ADv[(size_t)tc * B.sNI + iv] : 0.f;
        const float2 r0 = lf ? R[i] : make_float2(1.f, 1.f);
        const float2 tb = lf ? B.TB[to + i] : make_float2(0.f, 0.f);
        float x[KD];
        float2 rm[KD];
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = (okt >> u) & 1u;
            x[u] = ok ? ADh[S.e[u] * L1 + nz - 1] : 0.f;
            rm[u] = (ok && fct) ? R[S.m[u] * L1 + nz - 1] : make_float2(1.f, 1.f);
        }
        // vertical limiting (oce_adv_tra_fct.F90:425-456): interface nz by R of layers
        // nz-1 and nz; the next interface is the lane below's
        const float rux = sh_up(r0.x, 1), ruy = sh_up(r0.y, 1);
        if (fct) {
            if (nz == nzmin) f0 *= f0 >= 0.f ? r0.x : r0.y;
            else f0 *= f0 >= 0.f ? fminf(ruy, r0.x) : fminf(rux, r0.y);
        }
        float f1 = sh_dn(f0, 1);
        if (nz == nzmax - 1) f1 = 0.f;
        // horizontal limiting (oce_adv_tra_fct.F90:468-500) seen from the node: with G the
        // antidiffusive flux into the node and m the other end, G >= 0 takes
        // min(R+(n), R-(m)), G < 0 takes min(R-(n), R+(m))
        float hs = 0.f;
#pragma unroll
        for (int u = 0; u < KD; u++) {
            float G = ((own >> u) & 1u) ? x[u] : -x[u];
            if (fct) G *= G >= 0.f ? fminf(r0.x, rm[u].y) : fminf(r0.y, rm[u].x);
            hs += G;
        }
        // del_ttf = (LO hnode_new - T hnode) + limited flux divergence dt / areasvol;
        // T* = T + (del_ttf + T (hnode - hnode_new)) / hnode_new = LO + fluxes dt / areasvol / hnode_new
        // (oce_adv_tra_driver.F90:535-620, oce_ale_tracer.F90:319-321, 743-754)
        float val = lo + (f0 - f1 + hs) * sdt;
        if (k.out && on) {
            if (fct) {
                const float vc = fminf(fmaxf(val, tb.y), tb.x);
                // a clamp beyond round-off means the limiter itself failed
                if (fabsf(vc - val) > 1e-5f * (tb.x - tb.y) + 1e-6f * fabsf(vc)) atomicOr(B.status, 2u);
                val = vc;
            }
            // the diffusion increment k32_diff parked in Tnew (the limiter acts on advection only)
            if ((B.diff_mask >> tc) & 1ull) val += B.Tnew[to + i];
            B.Tnew[to + i] = val;
            if (!isfinite(val)) atomicOr(B.status, 1u);
        }
    }
}

// Limited update of every tracer of a node: per chunk the tracer-independent part
// (which edge slots are wet, dt / (areasvol hnode_new)) once, then per tracer every gather
// of the chunk, the limiter and the T* value, written to the buffer of the oldest time level.
template <int KD, bool PK>
__device__ __forceinline__ void update_node(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt,
                                            int n, int lane, const WEdges &S) {
    using C = Chunk<1, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    for (int ch = 0; ch < nch - 1; ch++) update_chunk<KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    // packed only for nodes of at most 6 edges, as in k32_bounds
    if (PK && KD <= 6 && P > 1) update_chunk<KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P);
    else update_chunk<KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1);
}

template <bool WIDE, bool PK>
__device__ __forceinline__ void update_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                            WEdges *Se) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) update_node<kMaxDeg, PK>(tp, g, B, dt, n, lane, S);
    else if (S.deg <= 6) update_node<6, PK>(tp, g, B, dt, n, lane, S);
    else update_node<8, PK>(tp, g, B, dt, n, lane, S);
}

template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_UPDATE)
k32_update(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ WEdges Se[kWB];
    update_unit<WIDE, true>(tp, g, B, dt, blockIdx.x * kWB + (threadIdx.x >> 5), Se);
}

// ---------------------------------------------------------------------------
// k32_vppm: adv_tra_vert_ppm (oce_adv_tra_ver.F90:438-631) on the AB values of the tracers
// in ppm_mask, minus the LO flux, into ADv.  A warp per node over chunks of 27 interfaces
// with 3 levels of halo above and 2 below: the interface value tv(k) needs the layers
// k-2..k+1, the flux of interface nz the parabola of layer nz or nz-1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void vppm_node(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                          const B32View &B, float dt, int n, int lane) {
    using C = Chunk<3, 2>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
    const int nch = C::count(nzmin, nzmax);
    for (int ch = 0; ch < nch; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        const int nz = k.nz;
        const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
        float hn0 = 0.f, ho0 = 0.f, ar0 = 0.f, w0 = 0.f, we0 = 0.f;
        if (k.lvl) {
            hn0 = g.hnode_new[i];
            ho0 = g.hnode[i];
            ar0 = g.area[iv];
            w0 = f.w[iv];
            we0 = f.we[iv];
        }
        const float hm1 = sh_up(hn0, 1), hm2 = sh_up(hn0, 2), hp1 = sh_dn(hn0, 1);
        const float hom1 = sh_up(ho0, 1);
        unsigned long long todo = B.ppm_mask;
        while (todo) {
            const int t = __ffsll((long long)todo) - 1;
            todo &= todo - 1;
            const bool lim = (B.fct_mask >> t) & 1ull;
            const size_t to = (size_t)t * B.sN;
            const float Tn = k.lvl ? B.T[to + i] : 0.f;
            const float o1 = k.lvl ? B.O1[to + i] : 0.f;
            const float o2 = (k.lvl && B.ab == 3) ? B.O2[to + i] : 0.f;
            const float tab = Tn + (k.lvl ? ab_delta(B.ab, Tn, o1, o2) : 0.f);
            const float tm1 = sh_up(tab, 1), tm2 = sh_up(tab, 2), tp1 = sh_dn(tab, 1);
            const float Tu = sh_up(Tn, 1);
            // tv(nz) (:488-562): centred next to the ends, the non-uniform PPM value between
            float tv;
            if (nz == nzmax) {
                tv = tm1;
            } else if (nz == nzmin) {
                tv = tab;
            } else if (nz == nzmax - 1 || nz == nzmin + 1) {
                tv = 0.5f * (tm1 + tab);
            } else {
                // layer j = nz-1: dzjm1 = h(nz-2), dzj = h(nz-1), dzjp1 = h(nz), dzjp2 = h(nz+1)
                const float a0 = hm2, a1 = hm1, a2 = hn0, a3 = hp1;
                const float d10 = tab - tm1, d0m = tm1 - tm2, d21 = tp1 - tab;
                float dj = a1 / (a0 + a1 + a2) * ((2.f * a0 + a1) / (a2 + a1) * d10 + (a1 + 2.f * a2) / (a0 + a1) * d0m);
                float dj1 = a2 / (a1 + a2 + a3) * ((2.f * a1 + a2) / (a3 + a2) * d21 + (a2 + 2.f * a3) / (a1 + a2) * d10);
                dj = d10 * d0m > 0.f ? copysignf(fminf(fminf(fabsf(dj), 2.f * fabsf(d10)), 2.f * fabsf(d0m)), dj) : 0.f;
                dj1 = d21 * d10 > 0.f ? copysignf(fminf(fminf(fabsf(dj1), 2.f * fabsf(d21)), 2.f * fabsf(d10)), dj1) : 0.f;
                tv = tm1 + a1 / (a1 + a2) * d10 +
                     1.f / (a0 + a1 + a2 + a3) *
                         ((2.f * a2 * a1) / (a1 + a2) * ((a0 + a1) / (2.f * a1 + a2) - (a3 + a2) / (2.f * a2 + a1)) * d10 -
                          a1 * (a0 + a1) / (2.f * a1 + a2) * dj1 + a2 * (a2 + a3) / (a1 + 2.f * a2) * dj);
            }
            const float tvu = sh_up(tv, 1), tvd = sh_dn(tv, 1);
            if (!k.out) continue;
            const float pw = lim ? w0 : we0;
            float Cf = 0.f;
            if (nz == nzmin) {
                Cf = -(tv * pw * ar0);
            } else if (pw > 0.f || pw < 0.f) {
                // the parabola of the upwind layer (:564-620)
                const bool top = pw > 0.f;
                float aL = top ? tv : tvu, aR = top ? tvd : tv;
                const float tt = top ? tab : tm1, dz = top ? ho0 : hom1;
                if ((aR - tt) * (tt - aL) <= 0.f) aL = aR = tt;
                if ((aR - aL) * (tt - 0.5f * (aL + aR)) > (aR - aL) * (aR - aL) * (1.f / 6.f)) aL = 3.f * tt - 2.f * aR;
                if ((aR - aL) * (tt - 0.5f * (aR + aL)) < -((aR - aL) * (aR - aL) * (1.f / 6.f))) aR = 3.f * tt - 2.f * aL;
                const float aj = 6.f * (tt - 0.5f * (aL + aR));
                const float x = fminf(fabsf(pw) * dt / dz, 1.f);
                const float v = top ? -aL - 0.5f * x * (aR - aL + (1.f - (2.f / 3.f) * x) * aj)
                                    : -aR + 0.5f * x * (aR - aL - (1.f - (2.f / 3.f) * x) * aj);
                Cf = v * ar0 * pw;
            }
            // minus the upwind LO flux: of w_e, or of the full w for FCT with the split velocity
            const float wl = (lim && f.wsplit) ? w0 : we0;
            float fl;
            if (nz == nzmin) {
                fl = -(wl * Tn * ar0);
            } else {
                const float aw = fabsf(wl);
                fl = -(0.5f * (Tn * (wl + aw) + Tu * (wl - aw)) * ar0);
            }
            B.ADv[(size_t)t * B.sNI + iv] = Cf - fl;
        }
    }
}

__global__ void __launch_bounds__(kTB) k32_vppm(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, float dt) {
    const int n = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (n >= tp.N2) return;
    vppm_node(tp, g, f, B, dt, n, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// split vertical velocity, FP32 form: adv_tra_vert_impl by w_i on the LO values of the FCT
// tracers (oce_adv_tra_ver.F90:90-240), and the implicit vertical diffusion with the w_i
// terms for the tracers without the limiter (oce_ale_tracer.F90:907-1435, do_wimpl).  One
// thread per column, FP64 arithmetic; scratch holds Z_n, cp and tp level-major.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void lo_impl_column(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                               const B32View &B, double dt, double *scratch, int n) {
    const int L1 = tp.L1, nl = tp.nl;
    const size_t N2 = tp.N2;
    double *cps = scratch, *tps = scratch + (size_t)(L1 + 1) * N2;
#define CP(k) cps[(size_t)(k) * N2 + n]
#define TP(k) tps[(size_t)(k) * N2 + n]
    const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
    const float *hn = g.hnode_new + (size_t)n * L1 - 1;
    const float *ar = g.area + (size_t)n * nl - 1, *av = g.areasvol + (size_t)n * nl - 1;
    const float *wi = f.wi + (size_t)n * nl - 1;
    unsigned long long todo = B.fct_mask & (B.ntr >= 64 ? ~0ull : ((1ull << B.ntr) - 1));
    while (todo) {
        const int t = __ffsll((long long)todo) - 1;
        todo &= todo - 1;
        float *Tc = B.LO + (size_t)t * B.sN + (size_t)n * L1 - 1;
        int nz = nzmin;
        double v = dt * ar[nz] / av[nz];
        double b = (double)hn[nz] + (double)wi[nz] * v;
        v = dt * ar[nz + 1] / av[nz];
        b = b - fmin(0.0, (double)wi[nz + 1]) * v;
        double c = -(fmax(0.0, (double)wi[nz + 1]) * v);
        double T0 = Tc[nz], Tp1 = Tc[nz + 1], Tm;
        double rhs = -((b - hn[nz]) * T0) - c * Tp1;
        double cp = c / b, tpv = rhs / b;
        CP(nz) = cp;
        TP(nz) = tpv;
        for (nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            v = dt * ar[nz] / av[nz];
            const double a = fmin(0.0, (double)wi[nz]) * v;
            b = (double)hn[nz] + fmax(0.0, (double)wi[nz]) * v;
            c = 0.0;
            if (nz <= nzmax - 2) {
                v = dt * ar[nz + 1] / av[nz];
                b = b - fmin(0.0, (double)wi[nz + 1]) * v;
                c = -(fmax(0.0, (double)wi[nz + 1]) * v);
            }
            Tm = T0;
            T0 = Tp1;
            Tp1 = nz <= nzmax - 2 ? (double)Tc[nz + 1] : 0.0;
            rhs = -(a * Tm) - (b - hn[nz]) * T0 - c * Tp1;
            const double m = b - cp * a;
            cp = c / m;
            tpv = (rhs - tpv * a) / m;
            CP(nz) = cp;
            TP(nz) = tpv;
        }
        double x = tpv;
        Tc[nzmax - 1] = (float)(Tc[nzmax - 1] + x);
        for (nz = nzmax - 2; nz >= nzmin; nz--) {
            x = TP(nz) - CP(nz) * x;
            Tc[nz] = (float)(Tc[nz] + x);
        }
    }
#undef CP
#undef TP
}

__device__ __forceinline__ void vdiff_w_column(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                               const B32View &B, double dt, double *scratch, int n) {
    const int L1 = tp.L1, nl = tp.nl;
    const size_t N2 = tp.N2;
    double *Zs = scratch, *cps = scratch + (size_t)(L1 + 1) * N2, *tps = cps + (size_t)(L1 + 1) * N2;
#define ZN(k) Zs[(size_t)(k) * N2 + n]
#define CP(k) cps[(size_t)(k) * N2 + n]
#define TP(k) tps[(size_t)(k) * N2 + n]
    const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
    const float *hn = g.hnode_new + (size_t)n * L1 - 1;
    const float *ar = g.area + (size_t)n * nl - 1, *av = g.areasvol + (size_t)n * nl - 1;
    const float *kv = f.Kv + (size_t)n * nl - 1, *wi = f.wi + (size_t)n * nl - 1;
    double zb = g.zbar_n_bot[n];
    ZN(nzmax - 1) = zb + (double)hn[nzmax - 1] / 2.0;
    for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
        zb = zb + (double)hn[nz];
        ZN(nz - 1) = zb + (double)hn[nz - 1] / 2.0;
    }
    unsigned long long todo = B.wimpl_mask & (B.ntr >= 64 ? ~0ull : ((1ull << B.ntr) - 1));
    while (todo) {
        const int t = __ffsll((long long)todo) - 1;
        todo &= todo - 1;
        float *Tc = B.Tnew + (size_t)t * B.sN + (size_t)n * L1 - 1;
        const double bc = B.fsurf ? (double)B.fsurf[t * B.sF + n] : 0.0;
        int nz = nzmin;
        double zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1)), zinv1;
        double c = -((double)kv[nz + 1] * zinv2 * dt * ar[nz + 1] / av[nz]);
        double b = -c + hn[nz];
        double v = dt * ((double)ar[nz] / av[nz]);
        b = b + (double)wi[nz] * v;
        v = dt * ar[nz + 1] / av[nz];
        b = b - fmin(0.0, (double)wi[nz + 1]) * v;
        c = c - fmax(0.0, (double)wi[nz + 1]) * v;
        double T0 = Tc[nz], Tp1 = Tc[nz + 1], Tm;
        double rhs = -((b - hn[nz]) * T0) - c * Tp1 + bc;
        double cp = c / b, tpv = rhs / b;
        CP(nz) = cp;
        TP(nz) = tpv;
        zinv1 = zinv2;
        for (nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            const bool bot = nz == nzmax - 1;
            double a = -((double)kv[nz] * zinv1 * dt * ((double)ar[nz] / av[nz]));
            c = 0.0;
            if (!bot) {
                zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1));
                c = -((double)kv[nz + 1] * zinv2 * dt * ar[nz + 1] / av[nz]);
            }
            b = -a - c + hn[nz];
            zinv1 = zinv2;
            v = dt * ((double)ar[nz] / av[nz]);
            a = a + fmin(0.0, (double)wi[nz]) * v;
            b = b + fmax(0.0, (double)wi[nz]) * v;
            if (!bot) {
                v = dt * ar[nz + 1] / av[nz];
                b = b - fmin(0.0, (double)wi[nz + 1]) * v;
                c = c - fmax(0.0, (double)wi[nz + 1]) * v;
            }
            Tm = T0;
            T0 = Tp1;
            Tp1 = bot ? 0.0 : (double)Tc[nz + 1];
            rhs = -(a * Tm) - (b - hn[nz]) * T0 - c * Tp1;
            const double m = b - cp * a;
            cp = c / m;
            tpv = (rhs - tpv * a) / m;
            CP(nz) = cp;
            TP(nz) = tpv;
        }
        double x = tpv;
        Tc[nzmax - 1] = (float)(Tc[nzmax - 1] + x);
        for (nz = nzmax - 2; nz >= nzmin; nz--) {
            x = TP(nz) - CP(nz) * x;
            Tc[nz] = (float)(Tc[nz] + x);
        }
    }
#undef ZN
#undef CP
#undef TP
}

__global__ void __launch_bounds__(128) k32_lo_impl(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, double dt,
                                                   double *scratch) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < tp.N2) lo_impl_column(tp, g, f, B, dt, scratch, n);
}
__global__ void __launch_bounds__(128) k32_vdiff_w(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, double dt,
                                                   double *scratch) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < tp.N2) vdiff_w_column(tp, g, f, B, dt, scratch, n);
}

// ---------------------------------------------------------------------------
// diffusion of diff_tracers_ale (oce_ale_tracer.F90:560-772) in the FP32 form
// ---------------------------------------------------------------------------
// k32_hdiff: diff_part_hor_redi (:1526-1689, Redi off) flux c of every edge-layer from the
// element gradients of the current values: segments A/D (element 1), B/E (element 2), C (both)
__device__ __forceinline__ void hdiff_edge32(const DTopo &tp, const DGeom<float> &g, const B32View &B, int e) {
    const int lane = threadIdx.x & 31;
    if (e >= tp.E2 || !B.Ki) return;
    const int L1 = tp.L1;
    const int el1 = tp.e_t1[e], el2 = tp.e_t2[e], n1 = tp.e_n1[e], n2 = tp.e_n2[e];
    const int nl1 = tp.t_nlev[el1] - 1, ul1 = tp.t_ulev[el1];
    int nl2 = 0, ul2 = 0;
    const float dX1 = g.ecd[4 * (size_t)e], dY1 = g.ecd[4 * (size_t)e + 1];
    float dX2 = 0.f, dY2 = 0.f;
    const int a0 = tp.t_n[3 * el1], a1 = tp.t_n[3 * el1 + 1], a2 = tp.t_n[3 * el1 + 2];
    const float *gs1 = g.gs + 6 * (size_t)el1;
    int b0 = a0, b1 = a1, b2 = a2;
    const float *gs2 = gs1;
    if (el2 >= 0) {
        nl2 = tp.t_nlev[el2] - 1;
        ul2 = tp.t_ulev[el2];
        dX2 = g.ecd[4 * (size_t)e + 2];
        dY2 = g.ecd[4 * (size_t)e + 3];
        b0 = tp.t_n[3 * el2];
        b1 = tp.t_n[3 * el2 + 1];
        b2 = tp.t_n[3 * el2 + 2];
        gs2 = g.gs + 6 * (size_t)el2;
    }
    const float p0 = gs1[0], p1 = gs1[1], p2 = gs1[2], p3 = gs1[3], p4 = gs1[4], p5 = gs1[5];
    const float q0 = gs2[0], q1 = gs2[1], q2 = gs2[2], q3 = gs2[3], q4 = gs2[4], q5 = gs2[5];
    const int nl12 = min(nl1, nl2), ul12 = max(ul1, ul2);
    for (int nz0 = tp.e_lo[e]; nz0 <= tp.e_hi[e]; nz0 += 32) {
        const int nz = nz0 + lane;
        if (nz > tp.e_hi[e]) continue;
        int seg = 0;
        if (nz >= ul1 && nz <= ul12 - 1) seg = 1;
        else if (ul2 > 0 && nz >= ul2 && nz <= ul12 - 1) seg = 2;
        else if (nz >= ul12 && nz <= nl12) seg = 3;
        else if (nz >= nl12 + 1 && nz <= nl1) seg = 1;
        else if (nz >= nl12 + 1 && nz <= nl2) seg = 2;
        const float Kh = (B.Ki[n1 * L1 + nz - 1] + B.Ki[n2 * L1 + nz - 1]) * 0.5f;
        const float h1 = g.helem[el1 * L1 + nz - 1], h2 = seg >= 2 ? g.helem[el2 * L1 + nz - 1] : 0.f;
        const bool u1 = seg == 1 || seg == 3, u2 = seg >= 2;
#pragma unroll 1
        for (int t = 0; t < B.ntr; t++) {
            const float *__restrict__ T = B.T + (size_t)t * B.sN;
            float tx1 = 0.f, ty1 = 0.f, tx2 = 0.f, ty2 = 0.f;
            if (u1) {
                const float va = T[a0 * L1 + nz - 1], vb = T[a1 * L1 + nz - 1], vc = T[a2 * L1 + nz - 1];
                tx1 = p0 * va + p1 * vb + p2 * vc;
                ty1 = p3 * va + p4 * vb + p5 * vc;
            }
            if (u2) {
                const float va = T[b0 * L1 + nz - 1], vb = T[b1 * L1 + nz - 1], vc = T[b2 * L1 + nz - 1];
                tx2 = q0 * va + q1 * vb + q2 * vc;
                ty2 = q3 * va + q4 * vb + q5 * vc;
            }
            float c = 0.f;
            if (seg == 1) c = (-dX1 * (Kh * ty1) + dY1 * (Kh * tx1)) * h1;
            else if (seg == 2) c = (dX2 * (Kh * ty2) - dY2 * (Kh * tx2)) * h2;
            else if (seg == 3)
                c = ((dX2 - dX1) * (Kh * (0.5f * (ty1 + ty2))) - (dY2 - dY1) * (Kh * (0.5f * (tx1 + tx2)))) *
                    ((h1 + h2) * 0.5f);
            B.HD[(size_t)t * B.sE + e * L1 + nz - 1] = c;
        }
    }
}

__global__ void __launch_bounds__(kTB) k32_hdiff(DTopo tp, DGeom<float> g, B32View B) {
    hdiff_edge32(tp, g, B, blockIdx.x * kWB + (threadIdx.x >> 5));
}

// k32_diff: the diffusion increment to T* of every tracer in diff_mask, parked in Tnew:
// (sum of the node's edge fluxes +- c) dt / (areasvol hnode_new) and, without implicit vertical
// diffusion, diff_ver_part_expl_ale (:841-902): vd(ul) = surface flux, vd(nz) = Kv (T(nz-1)
// - T(nz)) / (Z(nz-1) - Z(nz)) area, increment (vd(nz) - vd(nz+1)) / (zbar(nz) - zbar(nz+1))
// dt / (areasvol hnode_new)
template <int KD>
__device__ __forceinline__ void diff_node32(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int n,
                                            int lane, const WEdges &S) {
    using C = Chunk<1, 1>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const int nch = C::count(nzmin, nzmax);
    for (int ch = 0; ch < nch; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        const int nz = k.nz;
        const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
        float sdt = 0.f, kz = 0.f, q = 0.f;
        if (k.lvl) {
            sdt = dt / (g.areasvol[iv] * g.hnode_new[i]);
            if (nz > nzmin) kz = B.Kv[iv] / (g.Z3[i - 1] - g.Z3[i]) * g.area[iv];
            q = sdt / (g.zbar3[iv] - g.zbar3[iv + 1]);
        }
        const float kzd = sh_dn(kz, 1);
        unsigned okm = 0;
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
            okm |= ok ? 1u << u : 0u;
        }
#pragma unroll 1
        for (int t = 0; t < B.ntr; t++) {
            if (!((B.diff_mask >> t) & 1ull)) continue;
            float d = 0.f;
            if (B.Ki) {
                const float *__restrict__ HD = B.HD + (size_t)t * B.sE;
#pragma unroll
                for (int u = 0; u < KD; u++) {
                    const float x = ((okm >> u) & 1u) ? HD[S.e[u] * L1 + nz - 1] : 0.f;
                    d += ((own >> u) & 1u) ? x : -x;
                }
                d *= sdt;
            }
            if (!((B.ivd_mask >> t) & 1ull)) {
                const float Tn = k.lvl ? B.T[(size_t)t * B.sN + i] : 0.f;
                const float Tu = sh_up(Tn, 1), Td = sh_dn(Tn, 1);
                const float fs = B.fsurf ? B.fsurf[t * B.sF + n] : 0.f;
                const float vd0 = nz == nzmin ? fs : kz * (Tu - Tn);
                const float vd1 = nz == nzmax - 1 ? 0.f : kzd * (Tn - Td);
                d += (vd0 - vd1) * q;
            }
            if (k.out) B.Tnew[(size_t)t * B.sN + i] = d;
        }
    }
}

template <bool WIDE>
__device__ __forceinline__ void diff_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                          WEdges *Se) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0 || !B.diff_mask) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) diff_node32<kMaxDeg>(tp, g, B, dt, n, lane, S);
    else diff_node32<8>(tp, g, B, dt, n, lane, S);
}

template <bool WIDE>
__global__ void __launch_bounds__(kTB) k32_diff(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ WEdges Se[kWB];
    diff_unit<WIDE>(tp, g, B, dt, blockIdx.x * kWB + (threadIdx.x >> 5), Se);
}

// ---------------------------------------------------------------------------
// k32_vdiff: implicit vertical diffusion of the advected columns (in Tnew)
// ---------------------------------------------------------------------------
// Forward substitution tp_k = inv_k rhs_k - a_k inv_k tp_{k-1} and back substitution
// x_k = tp_k - cp_k x_{k+1} (oce_ale_tracer.F90:1406-1422) with the column's FP64-derived
// factors, as scans of affine maps y -> A y + B over the lanes of each chunk with the carry
// passed from chunk to chunk.  The multipliers A depend on the column only: their partial
// products at each scan step are formed once per node into shared memory, so a tracer's
// scan step is one shuffle and one multiply-add.  rhs_k = -a_k (T_{k-1} - T_k)
// - c_k (T_{k+1} - T_k) (+ bc_surface at the top, :1216-1229, 1377-1383); T += x.
constexpr int kWV = 4;                    // warps (nodes) per block of the diffusion kernel
constexpr int kScan = 5;                  // steps of a 32-lane scan
constexpr int kVdiffMaxChunks = kMaxChunks;

struct VdiffWarp {
    float4 fac[130];                                  // (a, c, 1/m, c/m), 1-based levels
    float af[kVdiffMaxChunks][kScan + 1][32];         // forward: A at each step (0 below the offset), then the total
    float ab[kVdiffMaxChunks][kScan + 1][32];         // backward
};

// forward and back substitution of tracers t1 and t2 (t2 < 0: none) of a column of NCH
// chunks: the chunks' scans are independent straight-line code; only the carries between
// chunks are serial
#ifndef FESOM_VDIFF_NT
#define FESOM_VDIFF_NT 3  // tracers whose scan chains interleave in one pass (2: 12.8 ms, 3: 11.4, 4: 12.5 on the 24-tracer sphere)
#endif

// the forward and backward scans of NT tracers (the first nt of them real), interleaved
template <int NCH, int NT>
__device__ __forceinline__ void vdiff_multi(const DTopo &tp, const DForcing<float> &f, const B32View &B, int n,
                                            int lane, int nzmin, int nzmax, const int (&tt)[NT], int nt,
                                            VdiffWarp &W) {
    using C = Chunk<1, 1>;
    const int L1 = tp.L1;
    float *__restrict__ Tq[NT];
    float bc[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) {
        const int t = q < nt ? tt[q] : tt[0];
        Tq[q] = B.Tnew + (size_t)t * B.sN;
        bc[q] = (f.bc && q < nt) ? f.bc[(size_t)t * tp.N2 + n] : 0.f;
    }
    float a[NT][NCH], y[NT][NCH];
#pragma unroll
    for (int ch = 0; ch < NCH; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        const int i = n * L1 + k.nz - 1;
#pragma unroll
        for (int q = 0; q < NT; q++) a[q][ch] = (k.lvl && q < nt) ? Tq[q][i] : 0.f;
    }
#pragma unroll
    for (int ch = 0; ch < NCH; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        const int nz = k.nz;
        float b[NT];
        const float4 fz = k.out ? W.fac[nz] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int q = 0; q < NT; q++) {
            const float u = sh_up(a[q][ch], 1), d = sh_dn(a[q][ch], 1);
            float r = 0.f;
            if (nz > nzmin) r -= fz.x * (u - a[q][ch]);
            if (nz < nzmax - 1) r -= fz.y * (d - a[q][ch]);
            if (nz == nzmin) r += bc[q];
            b[q] = k.out ? r * fz.z : 0.f;
        }
#pragma unroll
        for (int s = 0, off = 1; s < kScan; s++, off <<= 1) {
            const float w = W.af[ch][s][lane];
#pragma unroll
            for (int q = 0; q < NT; q++) b[q] = fmaf(w, __shfl_up_sync(kFull, b[q], off), b[q]);
        }
#pragma unroll
        for (int q = 0; q < NT; q++) y[q][ch] = b[q];
    }
    float c[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) c[q] = 0.f;
#pragma unroll
    for (int ch = 0; ch < NCH; ch++) {
        const float w = W.af[ch][kScan][lane];
#pragma unroll
        for (int q = 0; q < NT; q++) {
            y[q][ch] = fmaf(w, c[q], y[q][ch]);
            c[q] = __shfl_sync(kFull, y[q][ch], 30);  // last stored lane (Chunk<1, 1>)
        }
    }
#pragma unroll
    for (int ch = 0; ch < NCH; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        float b[NT];
#pragma unroll
        for (int q = 0; q < NT; q++) b[q] = k.out ? y[q][ch] : 0.f;
#pragma unroll
        for (int s = 0, off = 1; s < kScan; s++, off <<= 1) {
            const float w = W.ab[ch][s][lane];
#pragma unroll
            for (int q = 0; q < NT; q++) b[q] = fmaf(w, __shfl_down_sync(kFull, b[q], off), b[q]);
        }
#pragma unroll
        for (int q = 0; q < NT; q++) y[q][ch] = b[q];
    }
#pragma unroll
    for (int q = 0; q < NT; q++) c[q] = 0.f;
#pragma unroll
    for (int ch = NCH - 1; ch >= 0; ch--) {
        const C k(nzmin, nzmax, ch, lane);
        const float w = W.ab[ch][kScan][lane];
        const int i = n * L1 + k.nz - 1;
#pragma unroll
        for (int q = 0; q < NT; q++) {
            const float x = fmaf(w, c[q], y[q][ch]);
            c[q] = __shfl_sync(kFull, x, 1);  // first stored lane (Chunk<1, 1>)
            if (k.out && q < nt) {
                const float v = a[q][ch] + x;
                Tq[q][i] = v;
                if (!isfinite(v)) atomicOr(B.status, 1u);
            }
        }
    }
}

__device__ __forceinline__ void vdiff_unit(const DTopo &tp, const DForcing<float> &f, const B32View &B,
                                           const VFactors &vf, int n, VdiffWarp &W) {
    using C = Chunk<1, 1>;
    const int lane = threadIdx.x & 31;
    if (n >= tp.N2) return;
    const int L1 = tp.L1;
    const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
    const int nch = C::count(nzmin, nzmax);
    for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
        const int i = n * L1 + nz - 1;
        W.fac[nz] = make_float4(vf.a[i], vf.c[i], vf.inv[i], vf.cp[i]);
    }
    __syncwarp();
    // the column's scan multipliers
    for (int ch = 0; ch < nch; ch++) {
        const C k(nzmin, nzmax, ch, lane);
        float A = 1.f, Ad = 1.f;
        if (k.out) {
            const float4 fz = W.fac[k.nz];
            A = -(fz.x * fz.z);
            Ad = -fz.w;
        }
#pragma unroll
        for (int s = 0, off = 1; s < kScan; s++, off <<= 1) {
            W.af[ch][s][lane] = lane >= off ? A : 0.f;
            W.ab[ch][s][lane] = lane + off < 32 ? Ad : 0.f;
            const float Ap = __shfl_up_sync(kFull, A, off), An = __shfl_down_sync(kFull, Ad, off);
            if (lane >= off) A *= Ap;
            if (lane + off < 32) Ad *= An;
        }
        W.af[ch][kScan][lane] = A;
        W.ab[ch][kScan][lane] = Ad;
    }
    __syncwarp();
    // the tracers with implicit diffusion, FESOM_VDIFF_NT per pass: their scan chains interleave
    constexpr int NT = FESOM_VDIFF_NT;
    unsigned long long todo = (B.ivd_mask & ~B.wimpl_mask) & (B.ntr >= 64 ? ~0ull : ((1ull << B.ntr) - 1));
    while (todo) {
        int tt[NT], nt = 0;
#pragma unroll
        for (int q = 0; q < NT; q++) {
            tt[q] = todo ? __ffsll((long long)todo) - 1 : (q ? tt[0] : 0);
            if (todo) {
                todo &= todo - 1;
                nt++;
            }
        }
        switch (nch) {
            case 1: vdiff_multi<1, NT>(tp, f, B, n, lane, nzmin, nzmax, tt, nt, W); break;
            case 2: vdiff_multi<2, NT>(tp, f, B, n, lane, nzmin, nzmax, tt, nt, W); break;
            case 3: vdiff_multi<3, NT>(tp, f, B, n, lane, nzmin, nzmax, tt, nt, W); break;
            case 4: vdiff_multi<4, NT>(tp, f, B, n, lane, nzmin, nzmax, tt, nt, W); break;
            default: vdiff_multi<5, NT>(tp, f, B, n, lane, nzmin, nzmax, tt, nt, W); break;
        }
    }
}

__global__ void __launch_bounds__(32 * kWV) k32_vdiff(DTopo tp, DForcing<float> f, B32View B, VFactors vf) {
    __shared__ VdiffWarp Wsm[kWV];
    const int warp = threadIdx.x >> 5;
    vdiff_unit(tp, f, B, vf, blockIdx.x * kWV + warp, Wsm[warp]);
}

// ---------------------------------------------------------------------------
// multi-instance launches: every stage over all instances of a batch at once
// ---------------------------------------------------------------------------
// Units (edges, column blocks, nodes, items) of all instances are numbered one after
// another; ix.start[i] is instance i's first unit.  A warp (or thread, or block) finds
// its instance by binary search over those offsets (kernel parameters, warp-uniform)
// and runs the single-instance body with that instance's descriptor.
__device__ __forceinline__ int find_inst(const MultiIdx &ix, int u) {
    int lo = 0, hi = ix.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ix.start[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kTB) k32m_vflux(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    vflux_edge(I[i].tp, I[i].g, I[i].f, I[i].VF, u - ix.start[i], threadIdx.x & 31);
}
__global__ void __launch_bounds__(kVfCols) k32m_vfactors(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x;
    const int i = find_inst(ix, u);
    vfactors_block(I[i].tp, I[i].g, I[i].f, I[i].dtd, I[i].vf, u - ix.start[i]);
}
// WS: some instance has the split vertical velocity (each instance checks its own switch)
template <bool WIDE, bool WS>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_LO) k32m_lo_ad(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    lo_ad_unit<WIDE, WS, FESOM_PACK_MULTI>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].VF, I[i].dt, u - ix.start[i], Se);
}
__global__ void __launch_bounds__(kTB, FESOM_MINB_HO) k32m_ho(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    ho_unit<FESOM_PACK_MULTI>(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i]);
}
__global__ void __launch_bounds__(256) k32m_ho_nodemean(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    nodemean_item(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i]);
}
template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_BOUNDS) k32m_bounds(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    bounds_unit<WIDE, FESOM_PACK_MULTI>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se);
}
template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : FESOM_MINB_UPDATE) k32m_update(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    update_unit<WIDE, FESOM_PACK_MULTI>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se);
}
__global__ void __launch_bounds__(32 * kWV) k32m_vdiff(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ VdiffWarp Wsm[kWV];
    const int u = blockIdx.x * kWV + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    vdiff_unit(I[i].tp, I[i].f, I[i].B, I[i].vf, u - ix.start[i], Wsm[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(kTB) k32m_vppm(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (I[i].B.ppm_mask) vppm_node(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dt, u - ix.start[i], threadIdx.x & 31);
}
__global__ void __launch_bounds__(128) k32m_lo_impl(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (I[i].f.wsplit) lo_impl_column(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
}
__global__ void __launch_bounds__(128) k32m_vdiff_w(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (I[i].B.wimpl_mask) vdiff_w_column(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
}

__global__ void __launch_bounds__(kTB) k32m_hdiff(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    hdiff_edge32(I[i].tp, I[i].g, I[i].B, u - ix.start[i]);
}
template <bool WIDE>
__global__ void __launch_bounds__(kTB) k32m_diff(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    const int u = blockIdx.x * kWB + (threadIdx.x >> 5);
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    diff_unit<WIDE>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se);
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
    k32_vflux<<<grid32(tp.E2, kWB), kTB, 0, s>>>(tp, g, f, VF);
}
void b32_vfactors(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, double dt, const VFactors &v,
                  cudaStream_t s) {
    k32_vfactors<<<(tp.N2 + kVfCols - 1) / kVfCols, kVfCols, 0, s>>>(tp, g, f, dt, v);
}
// node kernels: one warp per node, kWB consecutive nodes per block; the nodes of more
// than 8 edges (listed at init) take a second, small launch with 16 edge slots
static int grid_nodes(int n) { return (n + kWB - 1) / kWB; }

void b32_lo_ad(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, const float *VF,
               double dt, cudaStream_t s) {
    if (f.wsplit) {
        k32_lo_ad<false, true><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
        if (tp.n_wide) k32_lo_ad<true, true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
    } else {
        k32_lo_ad<false, false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
        if (tp.n_wide) k32_lo_ad<true, false><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
    }
}
void b32_ho(const DTopo &tp, const DGeom<float> &g, const B32View &B, const MusclW &mw, const float *VF,
            cudaStream_t s) {
    k32_ho<<<grid_nodes(tp.E2), kTB, 0, s>>>(tp, B, mw, VF);
    if (mw.n_items) {
        int blocks = (mw.n_items + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        k32_ho_nodemean<<<blocks, 256, 0, s>>>(tp, B, mw, VF);
    }
}
void b32_bounds(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, cudaStream_t s) {
    k32_bounds<false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, B, (float)dt);
    if (tp.n_wide) k32_bounds<true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
}
void b32_update(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, cudaStream_t s) {
    k32_update<false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, B, (float)dt);
    if (tp.n_wide) k32_update<true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
}
void b32_vppm(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
              cudaStream_t s) {
    k32_vppm<<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, B, (float)dt);
}
void b32_lo_impl(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
                 double *scratch, cudaStream_t s) {
    k32_lo_impl<<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
}
void b32_vdiff_w(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
                 double *scratch, cudaStream_t s) {
    k32_vdiff_w<<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
}
void b32_hdiff(const DTopo &tp, const DGeom<float> &g, const B32View &B, cudaStream_t s) {
    k32_hdiff<<<grid_nodes(tp.E2), kTB, 0, s>>>(tp, g, B);
}
void b32_diff(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, cudaStream_t s) {
    k32_diff<false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, B, (float)dt);
    if (tp.n_wide) k32_diff<true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
}
void b32_vdiff(const DTopo &tp, const DForcing<float> &f, const B32View &B, const VFactors &v, cudaStream_t s) {
    k32_vdiff<<<(tp.N2 + kWV - 1) / kWV, 32 * kWV, 0, s>>>(tp, f, B, v);
}

// multi-instance launch wrappers: ix_* hold the per-instance unit offsets of each stage
void bm32_vflux(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vflux<<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_vfactors(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vfactors<<<u, kVfCols, 0, s>>>(I, ix);
}
void bm32_lo_ad(const Inst32 *I, const MultiIdx &ix, bool wide, bool ws, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (!u) return;
    if (ws) {
        if (wide) k32m_lo_ad<true, true><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
        else k32m_lo_ad<false, true><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
    } else {
        if (wide) k32m_lo_ad<true, false><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
        else k32m_lo_ad<false, false><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
    }
}
void bm32_vppm(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vppm<<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_lo_impl(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_lo_impl<<<(u + 127) / 128, 128, 0, s>>>(I, ix);
}
void bm32_vdiff_w(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vdiff_w<<<(u + 127) / 128, 128, 0, s>>>(I, ix);
}
void bm32_ho(const Inst32 *I, const MultiIdx &ix_e, const MultiIdx &ix_items, cudaStream_t s) {
    if (ix_e.start[ix_e.n]) k32m_ho<<<grid_nodes(ix_e.start[ix_e.n]), kTB, 0, s>>>(I, ix_e);
    const int u = ix_items.start[ix_items.n];
    if (u) k32m_ho_nodemean<<<(u + 255) / 256, 256, 0, s>>>(I, ix_items);
}
void bm32_bounds(const Inst32 *I, const MultiIdx &ix, bool wide, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (!u) return;
    if (wide) k32m_bounds<true><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
    else k32m_bounds<false><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_update(const Inst32 *I, const MultiIdx &ix, bool wide, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (!u) return;
    if (wide) k32m_update<true><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
    else k32m_update<false><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_hdiff(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_hdiff<<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_diff(const Inst32 *I, const MultiIdx &ix, bool wide, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (!u) return;
    if (wide) k32m_diff<true><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
    else k32m_diff<false><<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_vdiff(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vdiff<<<(u + kWV - 1) / kWV, 32 * kWV, 0, s>>>(I, ix);
}

}  // namespace fesom
