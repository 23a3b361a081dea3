// kernels_fp32_batched.cu -- the FP32 batched form of the tracer step.
//
// All tracers of a launch group in one launch per stage, the whole step in one CUDA graph:
//
//   k32_vflux        edge volume fluxes per edge-layer (oce_adv_tra_hor.F90:159-250
//                    segment rule); shared by every tracer
//   k32_vfactors     factorisation of the implicit vertical-diffusion matrix of every
//                    column (oce_ale_tracer.F90:1088-1204, 1406-1414): the pivots
//                    m = b - cp*a, where thin bottom cells cancel most bits, are formed
//                    in FP32 from their excess over |c|, a recurrence of non-negative
//                    terms; stored as FP32 a, c, 1/m, c/m
//   k32_lo_ad        per node: the LO solution (edge gather of upwind fluxes + upwind
//                    vertical flux with w_e) and the vertical antidiffusive flux
//                    (QR4C / UPW1 / CDIFF on the AB values; PPM in k32_vppm)
//   k32_ho           per edge: the horizontal antidiffusive flux, MUSCL / MFCT / UPW1 on
//                    the AB values minus the upwind LO flux (k32_ho_nodemean: the few
//                    edge-layers whose gradients are node means)
//   k32_bounds       per node: FCT bounds (max/min of LO and T over the node's
//                    neighbours and the adjacent layers) and R+/R- (oce_adv_tra_fct.F90)
//   k32_update       per node: limited fluxes, flux divergence, T* update, written to
//                    the buffer of the oldest time level; then, by default, the same warp
//                    runs the node's implicit vertical diffusion (k32_vdiff's column solve)
//   k32_vdiff        per node: the implicit vertical diffusion as two warp scans of
//                    affine maps over the column (forward and back substitution with
//                    the factors of k32_vfactors); its own launch only when asked for
//   k32_vppm, k32_lo_impl, k32_vdiff_w, k32_hdiff, k32_diff
//                    the optional parts: PPM vertical fluxes, the split vertical
//                    velocity, horizontal and explicit vertical diffusion
//
// Tracer groups: the tracers sit in groups of G slots (G = 4, or 2) of one scheme, side by
// side in every (level, entity) entry of a field.  A lane's load of one entry is one 16-byte
// (8-byte) vector load that brings all G tracers, so the address, the wet-level predicate
// and the load of every gather are formed once for G tracers, and G independent chains of
// arithmetic follow each load.  Slots a group does not fill hold zeros and compute zeros.
//
// Every tracer carries the same quantities whatever its limiter: the LO solution and the
// antidiffusive fluxes "high order minus low order" of the edges and interfaces.  Without
// FCT the update adds them unlimited, which is the high-order flux divergence; with FCT it
// scales them by R+/R- first.
//
// Conservation: every horizontal flux a node sums is formed from the edge's own data in the
// edge's direction (edges(1,e) -> edges(2,e)) and added at one end and subtracted at the
// other, so both ends use the same bits (the upwind LO flux is recomputed at each end by the
// same expression; the antidiffusive flux is stored once per edge-layer and its limiter
// factor min(R+, R-) is the same seen from either end); a vertical flux is one value shuffled
// between the two layers it joins.  With hnode = hnode_new the LO solution is T plus the flux
// divergence (no rescaling of T that would round every value of the column).
//
// Mapping of the node stages: one warp per node for all groups of the launch.  The lanes
// cover a chunk of the node's column (one level per lane); consecutive chunks overlap by the
// halo levels each stage needs (the level above/below comes from the neighbouring lane
// through a shuffle), and the halo lanes compute but do not store.  The last chunk of a
// column, when its levels fill at most half a warp, carries several groups side by side in
// lane segments.  The node's edge list, the neighbour offsets and the tracer-independent
// geometry of a chunk sit in registers and serve every group.  Blocks of eight warps take
// consecutive nodes (the node order is spatially local), so the neighbour columns a block
// gathers are mostly shared between its warps.
//
// No atomics on values: each edge flux is written once and every node sum is a gather.  The
// Adams-Bashforth shift is a rotation of the time-level buffers (no copy).
#include <cuda_runtime.h>

#include <algorithm>

#include "fesom_internal.h"

namespace fesom {

namespace {

// The FCT clamp of the advected value into its bounds: k32_bounds stores the bounds, k32_update
// clamps into them and raises FESOM_STATUS_FCT_BOUND where the clamp moved a value by more than
// round-off.  The reference has no such clamp; the FP32 limiter keeps the values inside their
// bounds to FP32 round-off without it, and the two bound arrays cost a write and a read of 8
// bytes per tracer-DOF (7.8 ms of the 24-tracer benchmark step), so the default build leaves it
// out; -DFESOM_FCT_CLAMP=1 builds it in.
#ifndef FESOM_FCT_CLAMP
#define FESOM_FCT_CLAMP 0
#endif
constexpr bool kFctClamp = FESOM_FCT_CLAMP != 0;
// packed FP32 pairs (two slots per instruction) in the edge kernel's arithmetic
#ifndef FESOM_PACKED_PAIRS
#define FESOM_PACKED_PAIRS 1
#endif
constexpr int kWB = 8;                // warps (= nodes) per block
constexpr int kTB = 32 * kWB;
constexpr unsigned kFull = 0xffffffffu;

// resident blocks per SM each group kernel is built for (registers: 65536 / (256 * blocks))
template <int G>
struct MinB {
    // the LO stage: three blocks per SM (the staged variant's double buffer fits 3 x 74 KB);
    // two measured 1.3 ms slower per step on the 24-tracer sphere, though its own launch is faster
#ifdef FESOM_MINB_LO
    static constexpr int lo = FESOM_MINB_LO;
#else
    static constexpr int lo = 3;
#endif
#ifdef FESOM_MINB_HO
    static constexpr int ho = FESOM_MINB_HO;
#else
    static constexpr int ho = G == 4 ? 3 : 4;
#endif
    // the staged edge kernel: 80 KB (G = 4) of staging per block of eight warps
    static constexpr int ho_stg = 2;
    // bounds and update: gathers in registers (three blocks of eight warps per SM measured
    // faster than two with more registers or one with the whole pass in flight), or staged in
    // shared memory (which holds one block of the G = 4 staging per SM)
    static constexpr int node_reg = 3;
    static constexpr int node_stg = G == 4 ? 1 : 2;
#ifdef FESOM_MINB_UPDATE_REG
    static constexpr int update_reg = FESOM_MINB_UPDATE_REG;
#else
    static constexpr int update_reg = node_reg;
#endif
#ifdef FESOM_MINB_BOUNDS_REG
    static constexpr int bounds_reg = FESOM_MINB_BOUNDS_REG;
#else
    static constexpr int bounds_reg = node_reg;
#endif
};

__device__ __forceinline__ size_t i1(int nz, int n, int L1) { return (size_t)n * L1 + (nz - 1); }

// FP32 quotients of the node stages (geometry factors, limiter ratios): the fast division
// (2 ulp) instead of the correctly rounded one; far inside the FP32 form's 1e-5, and the FCT
// clamp into the stored bounds keeps every result inside its bounds whatever the last bits
// of R+/R-
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }

}  // namespace

// the value of the lane d below / above in the warp
__device__ __forceinline__ float sh_up(float v, int d) { return __shfl_up_sync(kFull, v, d); }
__device__ __forceinline__ float sh_dn(float v, int d) { return __shfl_down_sync(kFull, v, d); }

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
// k32_vfactors: factorisation of each column's tridiagonal system
// ---------------------------------------------------------------------------
// a(k) = -Kv(k) dt/(Z_n(k-1)-Z_n(k)) area(k)/areasvol(k), c(k) = -Kv(k+1) dt/(Z_n(k)-Z_n(k+1))
// area(k+1)/areasvol(k), b = -a - c + hnode_new (oce_ale_tracer.F90:1099-1204), with
// Z_n(k)-Z_n(k+1) = (hnode_new(k) + hnode_new(k+1))/2 (the mid-depths of :1088-1096);
// Thomas pivots m(k) = b(k) - cp(k-1) a(k), cp(k) = c(k)/m(k) (:1406-1414).
// With a, c <= 0 and b = |a| + |c| + h, the pivot is m(k) = |c(k)| + d(k) with the excess
// d(k) = h(k) + |a(k)| d(k-1) / (d(k-1) + |c(k-1)|) (d = h at the top layer): the textbook form
// subtracts |a| |c(k-1)| / m(k-1) from |a| + |c| + h, which cancels most bits where a thin cell
// (small h) sits under strong diffusion; every term of the excess form is non-negative, so FP32
// keeps the pivots within a few ulps of the exact ones for any cell thickness.
//
// d(k) is a linear-fractional map of d(k-1): (d, 1) -> M_k (d, 1) projectively, with the
// non-negative M_k = [[h + |a|, h |c(k-1)|], [1, |c(k-1)|]] (the top layer: [[0, h], [0, 1]]).
// A warp takes a column, its lanes over 32-level chunks (coalesced loads and stores, each value
// read once): the lanes' maps are combined by an inclusive warp scan of 2x2 products (the later
// level's map on the left; each product rescaled by a power of two, exactly), applied to the
// vector carried from the chunk above.  Products and sums of non-negative numbers do not cancel,
// so the scan keeps the same few-ulp accuracy as the sequential recurrence.
struct M22 {
    float a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ M22 m22_mul(const M22 &x, const M22 &y) {
    return {x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
// 2^-e with 2^e <= x < 2^(e+1) for a normal positive x
__device__ __forceinline__ float pow2_inv(float x) {
    const int e = ((__float_as_int(x) >> 23) & 0xff) - 127;
    return __int_as_float((127 - e) << 23);
}
__device__ __forceinline__ M22 m22_norm(const M22 &m) {
    const float s = pow2_inv(fmaxf(fmaxf(m.a, m.b), fmaxf(m.c, m.d)));
    return {m.a * s, m.b * s, m.c * s, m.d * s};
}

__device__ __forceinline__ void vfactors_col(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                             float dtf, const VFactors &vf, int n, int lane) {
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
    float cx = 1.f, cy = 1.f;       // the excess vector at the last level of the chunk above
    float h_up = 0.f, c_up = 0.f;   // h and c of that level
    for (int nz0 = nzmin; nz0 <= nzmax - 1; nz0 += 32) {
        const int nz = nz0 + lane;
        const bool ok = nz <= nzmax - 1;
        const size_t i = (size_t)n * L1 + nz - 1, iv = (size_t)n * nl + nz - 1;
        float h = 0.f, ar = 0.f, av = 1.f, kv = 0.f;
        if (ok) {
            h = g.hnode_new[i];
            ar = g.area[iv];
            av = g.areasvol[iv];
            kv = f.Kv[iv];
        }
        // the level below (c) from the next lane, the chunk's last lane loads it
        float hn = sh_dn(h, 1), arn = sh_dn(ar, 1), kvn = sh_dn(kv, 1);
        if (lane == 31 && nz + 1 <= nzmax - 1) {
            hn = g.hnode_new[i + 1];
            arn = g.area[iv + 1];
            kvn = f.Kv[iv + 1];
        }
        // the level above (a) from the previous lane, the chunk's first lane from the chunk above
        float hu = sh_up(h, 1);
        if (lane == 0) hu = h_up;
        const float ravz = 1.f / av;
        float a = 0.f, c = 0.f;
        if (ok && nz > nzmin) a = -(kv * (2.f / (hu + h)) * dtf * (ar * ravz));
        if (ok && nz < nzmax - 1) c = -(kvn * (2.f / (h + hn)) * dtf * arn * ravz);
        float cu = sh_up(c, 1);
        if (lane == 0) cu = c_up;
        M22 S;
        if (!ok) S = {1.f, 0.f, 0.f, 1.f};
        else if (nz == nzmin) S = {0.f, h, 0.f, 1.f};
        else S = {h - a, h * -cu, 1.f, -cu};
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const M22 P = {sh_up(S.a, off), sh_up(S.b, off), sh_up(S.c, off), sh_up(S.d, off)};
            if (lane >= off) S = m22_norm(m22_mul(S, P));
        }
        const float v0 = S.a * cx + S.b * cy, v1 = S.c * cx + S.d * cy;
        if (ok) {
            const float m = v0 / v1 - c;
            vf.a[i] = a;
            vf.c[i] = c;
            vf.inv[i] = 1.f / m;
            vf.cp[i] = c / m;
        }
        // past the column's end the maps are identities: lane 31 holds the chunk's last level
        const float w0 = __shfl_sync(kFull, v0, 31), w1 = __shfl_sync(kFull, v1, 31);
        const float sc = pow2_inv(fmaxf(w0, w1));
        cx = w0 * sc;
        cy = w1 * sc;
        h_up = __shfl_sync(kFull, h, 31);
        c_up = __shfl_sync(kFull, c, 31);
    }
}

__global__ void __launch_bounds__(kTB) k32_vfactors(DTopo tp, DGeom<float> g, DForcing<float> f, float dt,
                                                    VFactors vf) {
    for (int n = blockIdx.x * kWB + (threadIdx.x >> 5); n < tp.N2; n += gridDim.x * kWB)
        vfactors_col(tp, g, f, dt, vf, n, threadIdx.x & 31);
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
    __syncwarp();  // every lane is done with the previous node's list (grid-stride loops)
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
    int q = 0;  // segment of the lane (packed chunks): its group is the pass's first plus q
    bool lvl, out;
    __device__ __forceinline__ Chunk(int nzmin, int nzmax, int ch, int lane) {
        nz = nzmin - HU + OUT * ch + lane;
        lvl = nz >= nzmin && nz <= nzmax - 1;
        out = lvl && lane >= HU && lane < 32 - HD;
    }
    // the last chunk of a column in P segments of W = (its levels + HU + HD) lanes, one
    // tracer group per segment: segment q holds the lanes [q W, (q + 1) W), laid out as a whole
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



// ---------------------------------------------------------------------------
// entries of G floats
// ---------------------------------------------------------------------------
template <int G>
struct Vec {
    float c[G];
};
template <int G>
__device__ __forceinline__ Vec<G> vfill(float x) {
    Vec<G> r;
#pragma unroll
    for (int k = 0; k < G; k++) r.c[k] = x;
    return r;
}
template <int G>
__device__ __forceinline__ Vec<G> vld(const float *__restrict__ p, int i);
template <>
__device__ __forceinline__ Vec<4> vld<4>(const float *__restrict__ p, int i) {
    const float4 q = reinterpret_cast<const float4 *>(p)[i];
    return Vec<4>{{q.x, q.y, q.z, q.w}};
}
template <>
__device__ __forceinline__ Vec<2> vld<2>(const float *__restrict__ p, int i) {
    const float2 q = reinterpret_cast<const float2 *>(p)[i];
    return Vec<2>{{q.x, q.y}};
}
// entry i where ok, zeros elsewhere (no load issued where !ok)
template <int G>
__device__ __forceinline__ Vec<G> vldc(bool ok, const float *__restrict__ p, int i) {
    Vec<G> r = vfill<G>(0.f);
    if (ok) r = vld<G>(p, i);
    return r;
}
// entry i where ok, read at L2 (ld.global.cg): values the same kernel stored before a
// __syncwarp, which a load through the read-only or L1 path is not bound to see
template <int G>
__device__ __forceinline__ Vec<G> vldcg(bool ok, const float *p, int i);
template <>
__device__ __forceinline__ Vec<4> vldcg<4>(bool ok, const float *p, int i) {
    Vec<4> r = vfill<4>(0.f);
    if (ok) {
        const float4 q = __ldcg(reinterpret_cast<const float4 *>(p) + i);
        r = Vec<4>{{q.x, q.y, q.z, q.w}};
    }
    return r;
}
template <>
__device__ __forceinline__ Vec<2> vldcg<2>(bool ok, const float *p, int i) {
    Vec<2> r = vfill<2>(0.f);
    if (ok) {
        const float2 q = __ldcg(reinterpret_cast<const float2 *>(p) + i);
        r = Vec<2>{{q.x, q.y}};
    }
    return r;
}
template <int G>
__device__ __forceinline__ void vst(float *p, int i, const Vec<G> &v);
template <>
__device__ __forceinline__ void vst<4>(float *p, int i, const Vec<4> &v) {
    reinterpret_cast<float4 *>(p)[i] = make_float4(v.c[0], v.c[1], v.c[2], v.c[3]);
}
template <>
__device__ __forceinline__ void vst<2>(float *p, int i, const Vec<2> &v) {
    reinterpret_cast<float2 *>(p)[i] = make_float2(v.c[0], v.c[1]);
}
// group g of a field of `count` entries per group
template <int G>
__device__ __forceinline__ const float *grp(const float *base, int g, size_t count) {
    return base + (size_t)g * count * G;
}
template <int G>
__device__ __forceinline__ float *grp(float *base, int g, size_t count) {
    return base + (size_t)g * count * G;
}

// ---------------------------------------------------------------------------
// per-lane asynchronous staging of a pass's gathers in shared memory
// ---------------------------------------------------------------------------
// The node stages gather, per pass (one chunk of a column for one tracer group), a few dozen
// entries per lane: the node's own and every neighbour's.  Held in registers, only a part of
// them can be in flight at once; staged with cp.async (one G-float copy per lane and entry,
// zero-filled where the lane has nothing to gather) they all are, and the next pass's copies
// run while the current pass computes.  Each lane reads back only what it copied, so the
// staging needs no barrier: cp.async.wait_group orders a lane's copies before its reads.
// Staging of a warp: [2 buffers][NS entries][32 lanes][G floats].
template <int G>
__device__ __forceinline__ void cpa(float *sdst, const float *gsrc, bool pred) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(sdst);
    const size_t a = __cvta_generic_to_global(gsrc);
    if constexpr (G == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(a), "r"(pred ? 16 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(a), "r"(pred ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
// entry s of the lane in a staging buffer
template <int G>
__device__ __forceinline__ float *stg(float *buf, int s, int lane) {
    return buf + ((size_t)s * 32 + lane) * G;
}
template <int G>
__device__ __forceinline__ Vec<G> lds(const float *p) {
    if constexpr (G == 4) {
        const float4 q = *reinterpret_cast<const float4 *>(p);
        return Vec<4>{{q.x, q.y, q.z, q.w}};
    } else {
        const float2 q = *reinterpret_cast<const float2 *>(p);
        return Vec<2>{{q.x, q.y}};
    }
}

// Adams-Bashforth value minus the current value: AB2 -(0.5+eps) T^{n-1} + (1.5+eps) T^n,
// AB3 (23 T^n - 16 T^{n-1} + 5 T^{n-2}) / 12 (oce_tracer_mod.F90:53, 67-68), eps = 0.1
__device__ __forceinline__ float ab_delta(int ab, float t, float o1, float o2) {
    return ab == 2 ? 0.6f * (t - o1) : (11.f * (t - o1) - 5.f * (o1 - o2)) * (1.f / 12.f);
}

// upwind flux of an edge-layer in the edge's direction, -(T1 v+ + T2 v-)
// (oce_adv_tra_hor.F90:174-177, 0.5 (v +- |v|) = v+ / v-), both products rounded and then
// summed: the rounding k32_lo_ad's node sums use for the same flux
__device__ __forceinline__ float upw_flux(float T1, float T2, float v) {
    return -__fadd_rn(__fmul_rn(T1, fmaxf(v, 0.f)), __fmul_rn(T2, fminf(v, 0.f)));
}

// vertical high-order flux of interface nz on the AB values (QR4C / UPW1 / CDIFF,
// oce_adv_tra_ver.F90:332-434, 635-695) minus the LO flux, for one slot
__device__ __forceinline__ float ver_ad(int ver, bool lim, float pv, int nz, int nzmin, int nzmax, bool twolayer,
                                        float tab, float tabu, float tabu2, float tabd, float pw, float ar0, float fv0,
                                        float fw0, float idz0, float idzp, float idzm, float g1, float g2) {
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
        const float aw = fabsf(pw);
        const float Tmean = (pw + aw) * Tm1 + (pw - aw) * Tm2;
        Cf = (-(0.5f * (1.f - pv) * Tmean) - pv * (0.5f * (Tm1 + Tm2)) * pw) * ar0;
    }
    // flux = C - flux_in; FCT passes the LO flux in, otherwise zero
    float F = Cf - (lim ? fw0 : 0.f);
    // a two-layer column writes its middle interface twice (statements nzmin+1, nzmax-1)
    if (ver == 0 && twolayer && nz == nzmin + 1) F = Cf - F;
    return lim ? F : F - fv0;
}

// Packed FP32 pairs: two slots of a group in one instruction (Blackwell's two-wide FP32 add,
// multiply and fused multiply-add).  Each element rounds as the scalar
// operation does; a - b is formed as fma(b, -1, a), which rounds once, like the subtraction.
__device__ __forceinline__ float2 pk(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
template <int G>
__device__ __forceinline__ float2 pr(const Vec<G> &a, int j) {
    return make_float2(a.c[2 * j], a.c[2 * j + 1]);
}

// The per-group arithmetic of k32_lo_ad for two slots at once: the AB value, the upwind
// vertical flux with w_e, LO from the edge-flux sum hs, and the vertical antidiffusive flux
// (ver_ad's branches, taken per lane and group, so both slots of a pair share them).
template <bool WS>
__device__ __forceinline__ void lo_ad_pair(const DForcing<float> &f, int ab, int ver, bool lim, bool lvt, float2 pv,
                                           int nz, int nzmin, int nzmax, bool twolayer, float ar0, float we0, float w0,
                                           float sdt, float dhr, float idz0, float idzp, float idzm, float g1,
                                           float g2, float2 tn, float2 o1, float2 o2, float2 hs, float2 &lo,
                                           float2 &ad) {
    float2 tab = tn;
    if (lvt)
        tab = ab == 2 ? pfma(pk(0.6f), psub(tn, o1), tn)
                      : pfma(pfma(pk(11.f), psub(tn, o1), pmul(pk(-5.f), psub(o1, o2))), pk(1.f / 12.f), tn);
    const float2 Tu = make_float2(sh_up(tn.x, 1), sh_up(tn.y, 1));
    const float2 tabu = make_float2(sh_up(tab.x, 1), sh_up(tab.y, 1));
    const float2 tabu2 = make_float2(sh_up(tab.x, 2), sh_up(tab.y, 2));
    const float2 tabd = make_float2(sh_dn(tab.x, 1), sh_dn(tab.y, 1));
    float2 fv0 = pk(0.f);
    if (lvt) {
        if (nz == nzmin) {
            fv0 = pmul(tn, pk(-(we0 * ar0)));
        } else {
            const float aw = fabsf(we0);
            fv0 = pmul(pfma(tn, pk(we0 + aw), pmul(Tu, pk(we0 - aw))), pk(-0.5f * ar0));
        }
    }
    float2 fv1 = make_float2(sh_dn(fv0.x, 1), sh_dn(fv0.y, 1));
    if (nz == nzmax - 1) fv1 = pk(0.f);
    lo = padd(tn, pfma(tn, pk(dhr), pmul(padd(hs, psub(fv0, fv1)), pk(sdt))));
    float2 fw0 = fv0;
    if (WS && f.wsplit && lvt) {
        if (nz == nzmin) {
            fw0 = pmul(tn, pk(-(w0 * ar0)));
        } else {
            const float aw = fabsf(w0);
            fw0 = pmul(pfma(tn, pk(w0 + aw), pmul(Tu, pk(w0 - aw))), pk(-0.5f * ar0));
        }
    }
    const float pw = lim ? w0 : we0;
    float2 Cf;
    if (nz == nzmin) {
        Cf = pmul(tab, pk(-(pw * ar0)));
    } else if (ver != 0 || nz == nzmin + 1 || nz == nzmax - 1) {
        if (ver != 1) {
            Cf = pmul(padd(tabu, tab), pk(-0.5f * pw * ar0));
        } else {
            const float aw = fabsf(pw);
            Cf = pmul(pfma(tab, pk(pw + aw), pmul(tabu, pk(pw - aw))), pk(-0.5f * ar0));
        }
    } else {
        const float2 qc = pmul(psub(tabu, tab), pk(idz0));
        const float2 qu = pmul(psub(tab, tabd), pk(idzp));
        const float2 qd = pmul(psub(tabu2, tabu), pk(idzm));
        const float2 Tm1 = pfma(pfma(pk(2.f), qc, qu), pk(g1), tab);
        const float2 Tm2 = pfma(pfma(pk(2.f), qc, qd), pk(g2), tabu);
        const float aw = fabsf(pw);
        const float2 Tmean = pfma(pk(pw + aw), Tm1, pmul(pk(pw - aw), Tm2));
        // (-(0.5 (1 - pv) Tmean) - pv (0.5 (Tm1 + Tm2)) pw) ar0
        const float2 a1 = pmul(pk(-0.5f), psub(pk(1.f), pv)), a2 = pmul(pk(-0.5f * pw), pv);
        Cf = pmul(pfma(a1, Tmean, pmul(a2, padd(Tm1, Tm2))), pk(ar0));
    }
    float2 F = lim ? psub(Cf, fw0) : Cf;
    if (ver == 0 && twolayer && nz == nzmin + 1) F = psub(Cf, F);
    ad = lim ? F : psub(F, fv0);
}

// ---------------------------------------------------------------------------
// k32_lo_ad
// ---------------------------------------------------------------------------
// One chunk of a node's column for every group of the launch.  PACK: the column's last
// chunk with P groups side by side in segments of W lanes; otherwise one group at a time
// over the whole warp.
template <int G, int KD, bool WS, bool PACK>
__device__ __forceinline__ void lo_ad_chunk(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                            const B32View &B, const float *__restrict__ VF, float dt, int n, int lane,
                                            const WEdges &S, int ch, int W, int P) {
    using C = Chunk<2, 1>;
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1;   // layer nz of the node (valid where k.lvl)
    const int iv = n * nl + nz - 1;  // interface nz
    // ---- tracer-independent part of the chunk ----
    // The node's share of edge slot u's upwind flux F = -(T1 v+ + T2 v-) (+F at edges(1,e),
    // -F at edges(2,e)) is rn(rn(T_n p_u) + rn(T_m q_u)) with (p, q) = (-v+, -v-) at edges(1,e)
    // and (v-, v+) at edges(2,e): the same two products and the same sum as at the other end,
    // so the two ends add exactly opposite values.  A dry slot has p = q = 0 and gathers the
    // node's own entry, so it adds zero without a per-tracer test.
    int off[KD];
    float pq[KD], qq[KD];
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : i;
        const float v = ok ? VF[S.e[u] * L1 + nz - 1] : 0.f;
        const float vp = fmaxf(v, 0.f), vm = fminf(v, 0.f);
        const bool ow = (own >> u) & 1u;
        pq[u] = ow ? -vp : vm;
        qq[u] = ow ? -vm : vp;
    }
    float ar0 = 0.f, we0 = 0.f, w0 = 0.f, sdt = 0.f, Z0 = 0.f, dhr = 0.f;
    if (k.lvl) {
        ar0 = g.area[iv];
        we0 = f.we[iv];
        w0 = f.w[iv];
        const float hn = g.hnode_new[i];
        sdt = qdiv(dt, g.areasvol[iv] * hn);
        dhr = qdiv(g.hnode[i] - hn, hn);
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
    // ---- per group ----
#pragma unroll 1
    for (int g0 = 0; g0 < B.ng; g0 += PACK ? P : 1) {
        // the lane's group (packed: the group of its segment; idle past the last)
        const int gg = g0 + k.q;
        const bool on = gg < B.ng;
        const int gi = on ? gg : g0;
        const bool lvt = k.lvl && on;
        const bool lim = (B.fct >> gi) & 1ull;
        const int ver = B.ver[gi];
        const float *__restrict__ T = grp<G>(B.T, gi, B.sN);
        const float *__restrict__ O1 = grp<G>(B.O1, gi, B.sN);
        const float *__restrict__ O2 = B.ab == 3 ? grp<G>(B.O2, gi, B.sN) : O1;
        // every load of the group's chunk first
        const Vec<G> Tn = vldc<G>(lvt, T, i);
        const Vec<G> o1 = vldc<G>(lvt, O1, i);
        const Vec<G> o2 = vldc<G>(lvt && B.ab == 3, O2, i);
        Vec<G> tm[KD];
#pragma unroll
        for (int u = 0; u < KD; u++) tm[u] = vldc<G>(lvt, T, off[u]);
        Vec<G> lo, ad;
#if FESOM_PACKED_PAIRS
#pragma unroll
        for (int j = 0; j < G / 2; j++) {
            const float2 tn = pr(Tn, j);
            float2 hs = pk(0.f);
#pragma unroll
            for (int u = 0; u < KD; u++) hs = padd(hs, padd(pmul(tn, pk(pq[u])), pmul(pr(tm[u], j), pk(qq[u]))));
            float2 l2, a2;
            lo_ad_pair<WS>(f, B.ab, ver, lim, lvt, make_float2(B.pv[gi * G + 2 * j], B.pv[gi * G + 2 * j + 1]), nz,
                           nzmin, nzmax, twolayer, ar0, we0, w0, sdt, dhr, idz0, idzp, idzm, g1, g2, tn, pr(o1, j),
                           pr(o2, j), hs, l2, a2);
            lo.c[2 * j] = l2.x;
            lo.c[2 * j + 1] = l2.y;
            ad.c[2 * j] = a2.x;
            ad.c[2 * j + 1] = a2.y;
        }
#else
#pragma unroll
        for (int c = 0; c < G; c++) {
            const float tn = Tn.c[c];
            const float tab = tn + (lvt ? ab_delta(B.ab, tn, o1.c[c], o2.c[c]) : 0.f);
            const float Tu = sh_up(tn, 1);
            const float tabu = sh_up(tab, 1), tabu2 = sh_up(tab, 2), tabd = sh_dn(tab, 1);
            // LO: the upwind edge fluxes, + at edges(1,e), - at edges(2,e), in ascending edge
            // order (oce_adv_tra_driver.F90:131-190)
            float hs = 0.f;
#pragma unroll
            for (int u = 0; u < KD; u++) hs += __fadd_rn(__fmul_rn(tn, pq[u]), __fmul_rn(tm[u].c[c], qq[u]));
            // upwind vertical flux with w_e at interface nz (adv_tra_ver_upw1)
            float fv0 = 0.f;
            if (lvt) {
                if (nz == nzmin) {
                    fv0 = -(we0 * tn * ar0);
                } else {
                    const float aw = fabsf(we0);
                    fv0 = -(0.5f * (tn * (we0 + aw) + Tu * (we0 - aw)) * ar0);
                }
            }
            float fv1 = sh_dn(fv0, 1);
            if (nz == nzmax - 1) fv1 = 0.f;
            // LO = (T hnode + flux divergence dt / areasvol) / hnode_new (oce_adv_tra_driver.F90:249),
            // as T + T (hnode - hnode_new) / hnode_new + flux divergence dt / (areasvol hnode_new)
            lo.c[c] = tn + fmaf(tn, dhr, (hs + (fv0 - fv1)) * sdt);
            // with the split vertical velocity the LO part of the antidiffusive flux is the upwind
            // flux of the full w (oce_adv_tra_driver.F90:323-334)
            float fw0 = fv0;
            if (WS && f.wsplit && lvt) {
                if (nz == nzmin) {
                    fw0 = -(w0 * tn * ar0);
                } else {
                    const float aw = fabsf(w0);
                    fw0 = -(0.5f * (tn * (w0 + aw) + Tu * (w0 - aw)) * ar0);
                }
            }
            ad.c[c] = ver_ad(ver, lim, B.pv[gi * G + c], nz, nzmin, nzmax, twolayer, tab, tabu, tabu2, tabd,
                             lim ? w0 : we0, ar0, fv0, fw0, idz0, idzp, idzm, g1, g2);
        }
#endif
        if (k.out && on) {
            vst<G>(grp<G>(B.LO, gi, B.sN), i, lo);
            // PPM fluxes come from k32_vppm
            if (ver != 3) vst<G>(grp<G>(B.ADv, gi, B.sNI), iv, ad);
        }
    }
}

// The same chunk with each pass's gathers staged in shared memory: entries T and the previous
// levels of the node, then T of every edge slot (a dry slot stages the node's own T).
constexpr int kNsLoAd = 3 + 6;
template <int G, int KD, bool WS, bool PACK>
__device__ __forceinline__ void lo_ad_chunk_pf(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                               const B32View &B, const float *__restrict__ VF, float dt, int n,
                                               int lane, const WEdges &S, int ch, int W, int P, float *sb) {
    using C = Chunk<2, 1>;
    constexpr int NS = 3 + KD;
    static_assert(NS <= kNsLoAd, "staging sized for six edge slots");
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1;
    const int iv = n * nl + nz - 1;
    // tracer-independent part of the chunk (as in lo_ad_chunk)
    int off[KD];
    float pq[KD], qq[KD];
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : (k.lvl ? i : 0);
        const float v = ok ? VF[S.e[u] * L1 + nz - 1] : 0.f;
        const float vp = fmaxf(v, 0.f), vm = fminf(v, 0.f);
        const bool ow = (own >> u) & 1u;
        pq[u] = ow ? -vp : vm;
        qq[u] = ow ? -vm : vp;
    }
    float ar0 = 0.f, we0 = 0.f, w0 = 0.f, sdt = 0.f, Z0 = 0.f, dhr = 0.f;
    if (k.lvl) {
        ar0 = g.area[iv];
        we0 = f.we[iv];
        w0 = f.w[iv];
        const float hn = g.hnode_new[i];
        sdt = qdiv(dt, g.areasvol[iv] * hn);
        dhr = qdiv(g.hnode[i] - hn, hn);
        Z0 = g.Z3[i];
    }
    const float Zm1 = sh_up(Z0, 1), Zm2 = sh_up(Z0, 2), Zp1 = sh_dn(Z0, 1);
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
    const int npass = PACK ? (B.ng + P - 1) / P : B.ng;
    auto grp_of = [&](int p) { return PACK ? p * P + k.q : p; };
    auto issue = [&](int p, float *buf) {
        const int gg = grp_of(p);
        const bool lvt = k.lvl && gg < B.ng;
        const int gi = gg < B.ng ? gg : 0;
        const float *T = grp<G>(B.T, gi, B.sN);
        const int ii = lvt ? i : 0;
        cpa<G>(stg<G>(buf, 0, lane), T + (size_t)ii * G, lvt);
        cpa<G>(stg<G>(buf, 1, lane), grp<G>(B.O1, gi, B.sN) + (size_t)ii * G, lvt);
        cpa<G>(stg<G>(buf, 2, lane), (B.ab == 3 ? grp<G>(B.O2, gi, B.sN) : T) + (size_t)ii * G, lvt && B.ab == 3);
#pragma unroll
        for (int u = 0; u < KD; u++) cpa<G>(stg<G>(buf, 3 + u, lane), T + (size_t)off[u] * G, lvt);
        cpa_commit();
    };
    auto compute = [&](int p, float *buf) {
        const int gg = grp_of(p);
        const bool on = gg < B.ng;
        const int gi = on ? gg : 0;
        const bool lvt = k.lvl && on;
        const bool lim = (B.fct >> gi) & 1ull;
        const int ver = B.ver[gi];
        const Vec<G> Tn = lds<G>(stg<G>(buf, 0, lane));
        const Vec<G> o1 = lds<G>(stg<G>(buf, 1, lane));
        const Vec<G> o2 = lds<G>(stg<G>(buf, 2, lane));
#if FESOM_PACKED_PAIRS
        Vec<G> lo, ad;
        float2 hsp[G / 2];
#pragma unroll
        for (int j = 0; j < G / 2; j++) hsp[j] = pk(0.f);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> tm = lds<G>(stg<G>(buf, 3 + u, lane));
#pragma unroll
            for (int j = 0; j < G / 2; j++)
                hsp[j] = padd(hsp[j], padd(pmul(pr(Tn, j), pk(pq[u])), pmul(pr(tm, j), pk(qq[u]))));
        }
#pragma unroll
        for (int j = 0; j < G / 2; j++) {
            const float2 tn = pr(Tn, j), hs = hsp[j];
            float2 l2, a2;
            lo_ad_pair<WS>(f, B.ab, ver, lim, lvt, make_float2(B.pv[gi * G + 2 * j], B.pv[gi * G + 2 * j + 1]), nz,
                           nzmin, nzmax, twolayer, ar0, we0, w0, sdt, dhr, idz0, idzp, idzm, g1, g2, tn, pr(o1, j),
                           pr(o2, j), hs, l2, a2);
            lo.c[2 * j] = l2.x;
            lo.c[2 * j + 1] = l2.y;
            ad.c[2 * j] = a2.x;
            ad.c[2 * j + 1] = a2.y;
        }
#else
        Vec<G> hs = vfill<G>(0.f);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> tm = lds<G>(stg<G>(buf, 3 + u, lane));
#pragma unroll
            for (int c = 0; c < G; c++)
                hs.c[c] += __fadd_rn(__fmul_rn(Tn.c[c], pq[u]), __fmul_rn(tm.c[c], qq[u]));
        }
        Vec<G> lo, ad;
#pragma unroll
        for (int c = 0; c < G; c++) {
            const float tn = Tn.c[c];
            const float tab = tn + (lvt ? ab_delta(B.ab, tn, o1.c[c], o2.c[c]) : 0.f);
            const float Tu = sh_up(tn, 1);
            const float tabu = sh_up(tab, 1), tabu2 = sh_up(tab, 2), tabd = sh_dn(tab, 1);
            float fv0 = 0.f;
            if (lvt) {
                if (nz == nzmin) {
                    fv0 = -(we0 * tn * ar0);
                } else {
                    const float aw = fabsf(we0);
                    fv0 = -(0.5f * (tn * (we0 + aw) + Tu * (we0 - aw)) * ar0);
                }
            }
            float fv1 = sh_dn(fv0, 1);
            if (nz == nzmax - 1) fv1 = 0.f;
            lo.c[c] = tn + fmaf(tn, dhr, (hs.c[c] + (fv0 - fv1)) * sdt);
            float fw0 = fv0;
            if (WS && f.wsplit && lvt) {
                if (nz == nzmin) {
                    fw0 = -(w0 * tn * ar0);
                } else {
                    const float aw = fabsf(w0);
                    fw0 = -(0.5f * (tn * (w0 + aw) + Tu * (w0 - aw)) * ar0);
                }
            }
            ad.c[c] = ver_ad(ver, lim, B.pv[gi * G + c], nz, nzmin, nzmax, twolayer, tab, tabu, tabu2, tabd,
                             lim ? w0 : we0, ar0, fv0, fw0, idz0, idzp, idzm, g1, g2);
        }
#endif
        if (k.out && on) {
            vst<G>(grp<G>(B.LO, gi, B.sN), i, lo);
            if (ver != 3) vst<G>(grp<G>(B.ADv, gi, B.sNI), iv, ad);
        }
    };
    issue(0, sb);
    float *cur = sb, *nxt = sb + (size_t)NS * 32 * G;
    for (int p = 0; p < npass; p++) {
        if (p + 1 < npass) {
            issue(p + 1, nxt);
            cpa_wait<1>();
        } else {
            cpa_wait<0>();
        }
        compute(p, cur);
        float *t = cur;
        cur = nxt;
        nxt = t;
    }
}

template <int G, int KD, bool WS, bool PK>
__device__ __forceinline__ void lo_ad_node(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                           const B32View &B, const float *__restrict__ VF, float dt, int n, int lane,
                                           const WEdges &S, float *sb) {
    using C = Chunk<2, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    if constexpr (KD == 6) {
        if (sb) {
            for (int ch = 0; ch < nch - 1; ch++)
                lo_ad_chunk_pf<G, KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, ch, 32, 1, sb);
            if (PK && P > 1) lo_ad_chunk_pf<G, KD, WS, true>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, W, P, sb);
            else lo_ad_chunk_pf<G, KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, 32, 1, sb);
            return;
        }
    }
    for (int ch = 0; ch < nch - 1; ch++) lo_ad_chunk<G, KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, ch, 32, 1);
    // packed only for nodes of at most 6 edges (the wider packed bodies would spill)
    if (PK && KD <= 6 && P > 1) lo_ad_chunk<G, KD, WS, true>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, W, P);
    else lo_ad_chunk<G, KD, WS, false>(tp, g, f, B, VF, dt, n, lane, S, nch - 1, 32, 1);
}

// the node of warp unit j: consecutive nodes, or (WIDE) the listed nodes of more than 8 edges
template <bool WIDE>
__device__ __forceinline__ int unit_node(const DTopo &tp, int j) {
    if (WIDE) return j < tp.n_wide ? tp.wide_nodes[j] : -1;
    return j < tp.N2 ? j : -1;
}
template <bool WIDE>
__device__ __forceinline__ int node_units(const DTopo &tp) {
    return WIDE ? tp.n_wide : tp.N2;
}

// WS: the split vertical velocity (a separate instantiation keeps the default path unchanged)
template <int G, bool WIDE, bool WS, bool PK>
__device__ __forceinline__ void lo_ad_unit(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                           const B32View &B, const float *__restrict__ VF, float dt, int j, WEdges *Se,
                                           float *sb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) lo_ad_node<G, kMaxDeg, WS, PK>(tp, g, f, B, VF, dt, n, lane, S, nullptr);
    else if (S.deg <= 6) lo_ad_node<G, 6, WS, PK>(tp, g, f, B, VF, dt, n, lane, S, sb);
    else lo_ad_node<G, 8, WS, PK>(tp, g, f, B, VF, dt, n, lane, S, nullptr);
}

template <int G>
__host__ __device__ constexpr int stage_bytes_lo_ad() { return 2 * kNsLoAd * 32 * G * 4; }

// grid-stride loop of the warps over the units (one launch may hold fewer blocks than units)
#define FOR_WARP_UNITS(j, count)                                                               \
    for (int j = blockIdx.x * kWB + (threadIdx.x >> 5); j < (count); j += gridDim.x * kWB)

template <int G, bool WIDE, bool WS, bool STG>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : MinB<G>::lo)
k32_lo_ad(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, const float *__restrict__ VF, float dt) {
    __shared__ WEdges Se[kWB];
    extern __shared__ __align__(16) float dsm[];
    float *sb = (WIDE || !STG) ? nullptr : dsm + (size_t)(threadIdx.x >> 5) * (stage_bytes_lo_ad<G>() / 4);
    FOR_WARP_UNITS(j, node_units<WIDE>(tp)) lo_ad_unit<G, WIDE, WS, true>(tp, g, f, B, VF, dt, j, Se, sb);
}

// high-order minus low-order flux of one edge-layer from the two end values, their
// previous time levels and the projected gradients s1 (up) / s2 (down)
__device__ __forceinline__ float ho_minus_lo(int hor, float ph, int ab, float T1, float T2, float o1a, float o1b,
                                             float o2a, float o2b, float s1, float s2, float v, float cl1, float cl2) {
    const float vp = fmaxf(v, 0.f), vm = fminf(v, 0.f);
    const float t1 = T1 + ab_delta(ab, T1, o1a, o2a);
    const float t2 = T2 + ab_delta(ab, T2, o1b, o2b);
    const float flo = upw_flux(T1, T2, v);
    float hf;
    if (hor == 2) {
        hf = upw_flux(t1, t2, v);
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

// hor, ab uniform over the pair; q1 = 1 - ph, q2 = v ph / 2 per slot; vp, vm the upwind parts of v
__device__ __forceinline__ float2 ho_minus_lo2(int hor, int ab, float2 q1, float2 q2, float2 T1, float2 T2,
                                               float2 o1a, float2 o1b, float2 o2a, float2 o2b, float2 s1,
                                               float2 s2, float vp, float vm, float cl1, float cl2) {
    float2 t1, t2;
    if (ab == 2) {
        t1 = pfma(pk(0.6f), psub(T1, o1a), T1);
        t2 = pfma(pk(0.6f), psub(T2, o1b), T2);
    } else {
        t1 = pfma(pfma(pk(11.f), psub(T1, o1a), pmul(pk(-5.f), psub(o1a, o2a))), pk(1.f / 12.f), T1);
        t2 = pfma(pfma(pk(11.f), psub(T2, o1b), pmul(pk(-5.f), psub(o1b, o2b))), pk(1.f / 12.f), T2);
    }
    // minus the LO flux: + (T1 v+ + T2 v-), both products rounded, then summed
    const float2 lo = padd(pmul(T1, pk(vp)), pmul(T2, pk(vm)));
    if (hor == 2) return psub(lo, padd(pmul(t1, pk(vp)), pmul(t2, pk(vm))));
    const float clo1 = hor == 0 ? cl1 : 1.f, clo2 = hor == 0 ? cl2 : 1.f;
    const float2 d2 = pmul(pk(2.f), psub(t2, t1));
    const float2 Tm2 = pfma(pmul(padd(d2, s2), pk(1.f / 6.f)), pk(-clo2), t2);
    const float2 Tm1 = pfma(pmul(padd(d2, s1), pk(1.f / 6.f)), pk(clo1), t1);
    // hf = -(1 - ph) (v+ Tm1 + v- Tm2) - (v ph / 2) (Tm1 + Tm2)
    const float2 c = pfma(pk(vp), Tm1, pmul(pk(vm), Tm2));
    return psub(lo, pfma(q1, c, pmul(q2, padd(Tm1, Tm2))));
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
// warp, carries P groups side by side in segments of W lanes (PACK).
// the group's high-minus-low fluxes of one edge-layer from its gathered entries
template <int G>
__device__ __forceinline__ Vec<G> ho_group(const B32View &B, int gq, int hor, const Vec<G> &T1, const Vec<G> &T2,
                                           const Vec<G> &o1a, const Vec<G> &o1b, const Vec<G> &o2a, const Vec<G> &o2b,
                                           const Vec<G> &ga, const Vec<G> &gb, const Vec<G> &gc, const Vec<G> &gd,
                                           const float4 &wu, const float4 &wd, float v, float cl1, float cl2) {
    Vec<G> out;
#if FESOM_PACKED_PAIRS
    const float vp = fmaxf(v, 0.f), vm = fminf(v, 0.f);
#pragma unroll
    for (int j = 0; j < G / 2; j++) {
        const float2 ph = make_float2(B.ph[gq * G + 2 * j], B.ph[gq * G + 2 * j + 1]);
        const float2 q1 = psub(pk(1.f), ph), q2 = pmul(pk(0.5f * v), ph);
        const float2 t1 = pr(T1, j), t2 = pr(T2, j);
        const float2 s1 = pfma(pk(wu.y), psub(pr(ga, j), t1), pmul(pk(wu.z), psub(pr(gb, j), t1)));
        const float2 s2 = pfma(pk(wd.y), psub(pr(gc, j), t2), pmul(pk(wd.z), psub(pr(gd, j), t2)));
        const float2 r = ho_minus_lo2(hor, B.ab, q1, q2, t1, t2, pr(o1a, j), pr(o1b, j), pr(o2a, j), pr(o2b, j), s1,
                                      s2, vp, vm, cl1, cl2);
        out.c[2 * j] = r.x;
        out.c[2 * j + 1] = r.y;
    }
#else
#pragma unroll
    for (int c = 0; c < G; c++) {
        const float s1 = wu.y * (ga.c[c] - T1.c[c]) + wu.z * (gb.c[c] - T1.c[c]);
        const float s2 = wd.y * (gc.c[c] - T2.c[c]) + wd.z * (gd.c[c] - T2.c[c]);
        out.c[c] = ho_minus_lo(hor, B.ph[gq * G + c], B.ab, T1.c[c], T2.c[c], o1a.c[c], o1b.c[c], o2a.c[c], o2b.c[c],
                               s1, s2, v, cl1, cl2);
    }
#endif
    return out;
}

template <int G, bool PACK>
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
    if (!ok) return;
    const int ie = e * L1 + nz - 1, ia = n1 * L1 + nz - 1, ib = n2 * L1 + nz - 1;
    const float v = VF[ie];
    const float cl1 = (nbl1 - nz) >= 0 ? 1.f : 0.f, cl2 = (nbl2 - nz) >= 0 ? 1.f : 0.f;
    const int ua = un.y * L1 + nz - 1, ub = un.z * L1 + nz - 1;
    const int da = dn.y * L1 + nz - 1, db = dn.z * L1 + nz - 1;
#pragma unroll 1
    for (int g0 = 0; g0 < B.ng; g0 += PACK ? P : 1) {
        const int gq = g0 + q;
        if (gq >= B.ng) break;
        const int hor = B.hor[gq];
        // MUSCL / MFCT levels outside the triangles' range: the node-mean launch
        if (hor != 2 && !tri) continue;
        const bool grad = hor != 2;
        const float *__restrict__ T = grp<G>(B.T, gq, B.sN);
        const float *__restrict__ O1 = grp<G>(B.O1, gq, B.sN);
        const float *__restrict__ O2 = B.ab == 3 ? grp<G>(B.O2, gq, B.sN) : O1;
        const Vec<G> T1 = vld<G>(T, ia), T2 = vld<G>(T, ib);
        const Vec<G> o1a = vld<G>(O1, ia), o1b = vld<G>(O1, ib);
        const Vec<G> o2a = vldc<G>(B.ab == 3, O2, ia), o2b = vldc<G>(B.ab == 3, O2, ib);
        const Vec<G> ga = vldc<G>(grad, T, ua), gb = vldc<G>(grad, T, ub);
        const Vec<G> gc = vldc<G>(grad, T, da), gd = vldc<G>(grad, T, db);
        vst<G>(grp<G>(B.ADh, gq, B.sE), ie,
               ho_group<G>(B, gq, hor, T1, T2, o1a, o1b, o2a, o2b, ga, gb, gc, gd, wu, wd, v, cl1, cl2));
    }
}

// The same pass with each group's gathers (T and the previous levels at both ends, T at the
// four triangle vertices) copied into shared memory by cp.async, double-buffered across the
// groups: the next group's copies are in flight while the current one computes.  Each lane reads
// back only its own copies, so the staging needs no barrier.  Staging of a warp:
// [2 buffers][kNsHo entries][32 lanes][G floats].
constexpr int kNsHo = 10;
template <int G>
__host__ __device__ constexpr int stage_bytes_ho() { return 2 * kNsHo * 32 * G * 4; }

template <int G, bool PACK>
__device__ __forceinline__ void ho_pass_pf(const DTopo &tp, const B32View &B, const MusclW &mw,
                                           const float *__restrict__ VF, int e, int nz0, int W, int P, int lane,
                                           float *sb) {
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
    if (!ok) return;
    const int ie = e * L1 + nz - 1, ia = n1 * L1 + nz - 1, ib = n2 * L1 + nz - 1;
    const float v = VF[ie];
    const float cl1 = (nbl1 - nz) >= 0 ? 1.f : 0.f, cl2 = (nbl2 - nz) >= 0 ? 1.f : 0.f;
    // the triangle vertices' entries where the gradients apply (elsewhere the edge's own, unread)
    const int ua = tri ? un.y * L1 + nz - 1 : ia, ub = tri ? un.z * L1 + nz - 1 : ia;
    const int da = tri ? dn.y * L1 + nz - 1 : ib, db = tri ? dn.z * L1 + nz - 1 : ib;
    const int npass = PACK ? (B.ng + P - 1) / P : B.ng;
    auto issue = [&](int p, float *buf) {
        const int gq = PACK ? p * P + q : p;
        const bool on = gq < B.ng;
        const int gi = on ? gq : 0;
        const int hor = B.hor[gi];
        const bool act = on && (hor == 2 || tri);
        const bool grad = act && hor != 2;
        const float *T = grp<G>(B.T, gi, B.sN), *O1 = grp<G>(B.O1, gi, B.sN);
        const float *O2 = B.ab == 3 ? grp<G>(B.O2, gi, B.sN) : O1;
        cpa<G>(stg<G>(buf, 0, lane), T + (size_t)ia * G, act);
        cpa<G>(stg<G>(buf, 1, lane), T + (size_t)ib * G, act);
        cpa<G>(stg<G>(buf, 2, lane), O1 + (size_t)ia * G, act);
        cpa<G>(stg<G>(buf, 3, lane), O1 + (size_t)ib * G, act);
        cpa<G>(stg<G>(buf, 4, lane), O2 + (size_t)ia * G, act && B.ab == 3);
        cpa<G>(stg<G>(buf, 5, lane), O2 + (size_t)ib * G, act && B.ab == 3);
        cpa<G>(stg<G>(buf, 6, lane), T + (size_t)ua * G, grad);
        cpa<G>(stg<G>(buf, 7, lane), T + (size_t)ub * G, grad);
        cpa<G>(stg<G>(buf, 8, lane), T + (size_t)da * G, grad);
        cpa<G>(stg<G>(buf, 9, lane), T + (size_t)db * G, grad);
        cpa_commit();
    };
    auto compute = [&](int p, const float *buf) {
        const int gq = PACK ? p * P + q : p;
        if (gq >= B.ng) return;
        const int hor = B.hor[gq];
        if (hor != 2 && !tri) return;  // MUSCL / MFCT outside the triangles' range: the node-mean launch
        const Vec<G> r = ho_group<G>(B, gq, hor, lds<G>(stg<G>((float *)buf, 0, lane)),
                                     lds<G>(stg<G>((float *)buf, 1, lane)), lds<G>(stg<G>((float *)buf, 2, lane)),
                                     lds<G>(stg<G>((float *)buf, 3, lane)), lds<G>(stg<G>((float *)buf, 4, lane)),
                                     lds<G>(stg<G>((float *)buf, 5, lane)), lds<G>(stg<G>((float *)buf, 6, lane)),
                                     lds<G>(stg<G>((float *)buf, 7, lane)), lds<G>(stg<G>((float *)buf, 8, lane)),
                                     lds<G>(stg<G>((float *)buf, 9, lane)), wu, wd, v, cl1, cl2);
        vst<G>(grp<G>(B.ADh, gq, B.sE), ie, r);
    };
    issue(0, sb);
    float *cur = sb, *nxt = sb + (size_t)kNsHo * 32 * G;
    for (int p = 0; p < npass; p++) {
        if (p + 1 < npass) {
            issue(p + 1, nxt);
            cpa_wait<1>();
        } else {
            cpa_wait<0>();
        }
        compute(p, cur);
        float *t = cur;
        cur = nxt;
        nxt = t;
    }
}

template <int G, bool PK, bool STG>
__device__ __forceinline__ void ho_unit(const DTopo &tp, const B32View &B, const MusclW &mw,
                                        const float *__restrict__ VF, int e, float *sb) {
    const int lane = threadIdx.x & 31;
    if (e >= tp.E2) return;
    const int elo = tp.e_lo[e], ehi = tp.e_hi[e];
    int nz0 = elo;
    for (; nz0 + 32 <= ehi; nz0 += 32) {
        if (STG) ho_pass_pf<G, false>(tp, B, mw, VF, e, nz0, 32, 1, lane, sb);
        else ho_pass<G, false>(tp, B, mw, VF, e, nz0, 32, 1, lane);
    }
    const int W = ehi - nz0 + 1;
    if (W < 1) return;
    const int P = 32 / W;
    if (STG) {
        if (PK && P > 1) ho_pass_pf<G, true>(tp, B, mw, VF, e, nz0, W, P, lane, sb);
        else ho_pass_pf<G, false>(tp, B, mw, VF, e, nz0, 32, 1, lane, sb);
    } else {
        if (PK && P > 1) ho_pass<G, true>(tp, B, mw, VF, e, nz0, W, P, lane);
        else ho_pass<G, false>(tp, B, mw, VF, e, nz0, 32, 1, lane);
    }
}

template <int G, bool STG>
__global__ void __launch_bounds__(kTB, STG ? MinB<G>::ho_stg : MinB<G>::ho)
k32_ho(DTopo tp, B32View B, MusclW mw, const float *__restrict__ VF) {
    extern __shared__ __align__(16) float dsm[];
    float *sb = STG ? dsm + (size_t)(threadIdx.x >> 5) * (stage_bytes_ho<G>() / 4) : nullptr;
    FOR_WARP_UNITS(e, tp.E2) ho_unit<G, true, STG>(tp, B, mw, VF, e, sb);
}

// The edge-layers of the node-mean gradients: one thread per (edge, level) item, every
// group, with the projected mean gradients as precomputed neighbour weights.
template <int G>
__device__ __forceinline__ void nodemean_item(const DTopo &tp, const B32View &B, const MusclW &mw,
                                              const float *__restrict__ VF, int j) {
    const int L1 = tp.L1;
    const int e = mw.it_e[j], nz = mw.it_nz[j];
    const int p0 = mw.it_ptr[j], p1 = p0 + mw.it_n1[j], p2 = mw.it_ptr[j + 1];
    const int n1 = tp.e_n1[e], n2 = tp.e_n2[e];
    const int ie = e * L1 + nz - 1, ia = n1 * L1 + nz - 1, ib = n2 * L1 + nz - 1;
    const float v = VF[ie];
    const float cl1 = (tp.n_nbl[n1] - nz) >= 0 ? 1.f : 0.f, cl2 = (tp.n_nbl[n2] - nz) >= 0 ? 1.f : 0.f;
#pragma unroll 1
    for (int gq = 0; gq < B.ng; gq++) {
        const int hor = B.hor[gq];
        if (hor == 2) continue;  // UPW1 has no gradients: k32_ho wrote it
        const float *__restrict__ T = grp<G>(B.T, gq, B.sN);
        const float *__restrict__ O1 = grp<G>(B.O1, gq, B.sN);
        const Vec<G> T1 = vld<G>(T, ia), T2 = vld<G>(T, ib);
        const Vec<G> o1a = vld<G>(O1, ia), o1b = vld<G>(O1, ib);
        const Vec<G> o2a = vldc<G>(B.ab == 3, grp<G>(B.O2, gq, B.sN), ia);
        const Vec<G> o2b = vldc<G>(B.ab == 3, grp<G>(B.O2, gq, B.sN), ib);
        Vec<G> s1 = vfill<G>(0.f), s2 = vfill<G>(0.f);
        for (int p = p0; p < p1; p++) {
            const int2 q = mw.pairs[p];
            const Vec<G> t = vld<G>(T, q.x * L1 + nz - 1);
#pragma unroll
            for (int c = 0; c < G; c++) s1.c[c] += __int_as_float(q.y) * (t.c[c] - T1.c[c]);
        }
        for (int p = p1; p < p2; p++) {
            const int2 q = mw.pairs[p];
            const Vec<G> t = vld<G>(T, q.x * L1 + nz - 1);
#pragma unroll
            for (int c = 0; c < G; c++) s2.c[c] += __int_as_float(q.y) * (t.c[c] - T2.c[c]);
        }
        Vec<G> out;
#pragma unroll
        for (int c = 0; c < G; c++)
            out.c[c] = ho_minus_lo(hor, B.ph[gq * G + c], B.ab, T1.c[c], T2.c[c], o1a.c[c], o1b.c[c], o2a.c[c],
                                   o2b.c[c], s1.c[c], s2.c[c], v, cl1, cl2);
        vst<G>(grp<G>(B.ADh, gq, B.sE), ie, out);
    }
}

template <int G>
__global__ void __launch_bounds__(256) k32_ho_nodemean(DTopo tp, B32View B, MusclW mw, const float *__restrict__ VF) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < mw.n_items; j += gridDim.x * blockDim.x)
        nodemean_item<G>(tp, B, mw, VF, j);
}

// ---------------------------------------------------------------------------
// k32_bounds: FCT bounds and R+ / R- (FCT groups only)
// ---------------------------------------------------------------------------
// One chunk of a node's column for the FCT groups of the launch.  PACK: the column's last
// chunk with P groups side by side in segments of W lanes; otherwise one group at a time
// over the whole warp.
template <int G, int KD, bool PACK>
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
    // a dry slot gathers the node's own T and LO (neutral for the bounds); its ADh is not loaded
    int off[KD], eo[KD];
    unsigned okx = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : i;
        eo[u] = ok ? S.e[u] * L1 + nz - 1 : 0;
        okx |= ok ? 1u << u : 0u;
    }
    const float s = k.lvl ? qdiv(dt, g.areasvol[iv] * g.hnode_new[i]) : 0.f;
    unsigned long long todo = B.fct & (B.ng >= 64 ? ~0ull : ((1ull << B.ng) - 1));
    int g0 = 0;
    while (PACK ? g0 < B.ng : todo != 0ull) {
        // the lane's group: the next FCT group, or (packed) group g0 + q of the segment, idle
        // where that group has no FCT
        int gq;
        if (PACK) {
            gq = g0 + k.q;
            if (gq >= B.ng || !((B.fct >> gq) & 1ull)) gq = -1;
            g0 += P;
        } else {
            gq = __ffsll((long long)todo) - 1;
            todo &= todo - 1;
        }
        const bool lv = k.lvl && gq >= 0;
        const int gs = gq < 0 ? 0 : gq;
        const float *__restrict__ T = grp<G>(B.T, gs, B.sN);
        const float *__restrict__ LO = grp<G>(B.LO, gs, B.sN);
        const float *__restrict__ ADh = grp<G>(B.ADh, gs, B.sE);
        const Vec<G> Tn = vldc<G>(lv, T, i);
        const Vec<G> lo = vldc<G>(lv, LO, i);
        const Vec<G> v0 = vldc<G>(lv, grp<G>(B.ADv, gs, B.sNI), iv);
        // bounds over the node, its neighbours and the layers above and below
        // (oce_adv_tra_fct.F90:124-248)
        Vec<G> mx, mn;
#pragma unroll
        for (int c = 0; c < G; c++) {
            mx.c[c] = fmaxf(lo.c[c], Tn.c[c]);
            mn.c[c] = fminf(lo.c[c], Tn.c[c]);
        }
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> tm = vldc<G>(lv, T, off[u]);
            const Vec<G> lm = vldc<G>(lv, LO, off[u]);
#pragma unroll
            for (int c = 0; c < G; c++) {
                mx.c[c] = fmaxf(mx.c[c], fmaxf(tm.c[c], lm.c[c]));
                mn.c[c] = fminf(mn.c[c], fminf(tm.c[c], lm.c[c]));
            }
        }
        // P / M: sums of the positive / negative antidiffusive fluxes into the node
        Vec<G> Pp = vfill<G>(0.f), M = vfill<G>(0.f);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> x = vldc<G>(lv && ((okx >> u) & 1u), ADh, eo[u]);
            const bool ow = (own >> u) & 1u;
#pragma unroll
            for (int c = 0; c < G; c++) {
                const float xv = ow ? x.c[c] : -x.c[c];
                Pp.c[c] += fmaxf(0.f, xv);
                M.c[c] += fminf(0.f, xv);
            }
        }
        Vec<G> rp, rm, bp, bm;
#pragma unroll
        for (int c = 0; c < G; c++) {
            const float mxu = sh_up(mx.c[c], 1), mxd = sh_dn(mx.c[c], 1);
            const float mnu = sh_up(mn.c[c], 1), mnd = sh_dn(mn.c[c], 1);
            float tup = mx.c[c], tlo = mn.c[c];
            if (nz != nzmin && nz != nzmax - 1) {
                tup = fmaxf(fmaxf(mxu, mx.c[c]), mxd);
                tlo = fminf(fminf(mnu, mn.c[c]), mnd);
            }
            float v1 = sh_dn(v0.c[c], 1);
            if (nz == nzmax - 1) v1 = 0.f;
            const float pp = Pp.c[c] + (fmaxf(0.f, v0.c[c]) + fmaxf(0.f, -v1));
            const float mm = M.c[c] + (fminf(0.f, v0.c[c]) + fminf(0.f, -v1));
            const float bmx = tup - lo.c[c], bmn = tlo - lo.c[c];
            rp.c[c] = fminf(1.f, qdiv(bmx, pp * s + eps));
            rm.c[c] = fminf(1.f, qdiv(bmn, mm * s - eps));
            // the bounds themselves: the update clamps the advected value into them, so FP32
            // rounding in the limiter can never create a new extremum
            bp.c[c] = tup;
            bm.c[c] = tlo;
        }
        if (k.out && gq >= 0) {
            vst<G>(grp<G>(B.Rp, gq, B.sN), i, rp);
            vst<G>(grp<G>(B.Rm, gq, B.sN), i, rm);
            if (kFctClamp) {
                vst<G>(grp<G>(B.Bp, gq, B.sN), i, bp);
                vst<G>(grp<G>(B.Bm, gq, B.sN), i, bm);
            }
        }
    }
}

// The same chunk with each pass's gathers staged in shared memory (sb: the warp's staging):
// entries T, LO, ADv of the node, then T, LO, ADh of every edge slot.
constexpr int kNsBounds = 3 + 3 * 6;
template <int G, int KD, bool PACK>
__device__ __forceinline__ void bounds_chunk_pf(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt,
                                                int n, int lane, const WEdges &S, int ch, int W, int P, float *sb) {
    using C = Chunk<1, 1>;
    constexpr int NS = 3 + 3 * KD;
    static_assert(NS <= kNsBounds, "staging sized for six edge slots");
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const float eps = (float)kFluxEps;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
    // a dry slot stages the node's own T and LO (neutral for the bounds) and zeros for ADh
    int off[KD], eo[KD];
    unsigned okx = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : (k.lvl ? i : 0);
        eo[u] = ok ? S.e[u] * L1 + nz - 1 : 0;
        okx |= ok ? 1u << u : 0u;
    }
    const float s = k.lvl ? qdiv(dt, g.areasvol[iv] * g.hnode_new[i]) : 0.f;
    unsigned todo = (unsigned)(B.fct & (B.ng >= 32 ? 0xffffffffull : ((1ull << B.ng) - 1)));
    int g0 = 0;
    // the lane's group of the next pass (-1: idle); false when no pass is left
    auto next = [&](int &gq) -> bool {
        if (PACK) {
            if (g0 >= B.ng) return false;
            gq = g0 + k.q;
            if (gq >= B.ng || !((B.fct >> gq) & 1ull)) gq = -1;
            g0 += P;
            return true;
        }
        if (!todo) return false;
        gq = __ffs(todo) - 1;
        todo &= todo - 1;
        return true;
    };
    auto issue = [&](int gq, float *buf) {
        const bool lv = k.lvl && gq >= 0;
        const int gs = gq < 0 ? 0 : gq;
        const float *T = grp<G>(B.T, gs, B.sN), *LO = grp<G>(B.LO, gs, B.sN);
        const float *ADh = grp<G>(B.ADh, gs, B.sE), *ADv = grp<G>(B.ADv, gs, B.sNI);
        cpa<G>(stg<G>(buf, 0, lane), T + (size_t)(lv ? i : 0) * G, lv);
        cpa<G>(stg<G>(buf, 1, lane), LO + (size_t)(lv ? i : 0) * G, lv);
        cpa<G>(stg<G>(buf, 2, lane), ADv + (size_t)(lv ? iv : 0) * G, lv);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            cpa<G>(stg<G>(buf, 3 + 3 * u, lane), T + (size_t)off[u] * G, lv);
            cpa<G>(stg<G>(buf, 4 + 3 * u, lane), LO + (size_t)off[u] * G, lv);
            cpa<G>(stg<G>(buf, 5 + 3 * u, lane), ADh + (size_t)eo[u] * G, lv && ((okx >> u) & 1u));
        }
        cpa_commit();
    };
    auto compute = [&](int gq, float *buf) {
        const Vec<G> Tn = lds<G>(stg<G>(buf, 0, lane));
        const Vec<G> lo = lds<G>(stg<G>(buf, 1, lane));
        const Vec<G> v0 = lds<G>(stg<G>(buf, 2, lane));
        Vec<G> mx, mn, Pp = vfill<G>(0.f), M = vfill<G>(0.f);
#pragma unroll
        for (int c = 0; c < G; c++) {
            mx.c[c] = fmaxf(lo.c[c], Tn.c[c]);
            mn.c[c] = fminf(lo.c[c], Tn.c[c]);
        }
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> tm = lds<G>(stg<G>(buf, 3 + 3 * u, lane));
            const Vec<G> lm = lds<G>(stg<G>(buf, 4 + 3 * u, lane));
            const Vec<G> x = lds<G>(stg<G>(buf, 5 + 3 * u, lane));
            const bool ow = (own >> u) & 1u;
#pragma unroll
            for (int c = 0; c < G; c++) {
                mx.c[c] = fmaxf(mx.c[c], fmaxf(tm.c[c], lm.c[c]));
                mn.c[c] = fminf(mn.c[c], fminf(tm.c[c], lm.c[c]));
                const float xv = ow ? x.c[c] : -x.c[c];
                Pp.c[c] += fmaxf(0.f, xv);
                M.c[c] += fminf(0.f, xv);
            }
        }
        Vec<G> rp, rm, bp, bm;
#pragma unroll
        for (int c = 0; c < G; c++) {
            const float mxu = sh_up(mx.c[c], 1), mxd = sh_dn(mx.c[c], 1);
            const float mnu = sh_up(mn.c[c], 1), mnd = sh_dn(mn.c[c], 1);
            float tup = mx.c[c], tlo = mn.c[c];
            if (nz != nzmin && nz != nzmax - 1) {
                tup = fmaxf(fmaxf(mxu, mx.c[c]), mxd);
                tlo = fminf(fminf(mnu, mn.c[c]), mnd);
            }
            float v1 = sh_dn(v0.c[c], 1);
            if (nz == nzmax - 1) v1 = 0.f;
            const float pp = Pp.c[c] + (fmaxf(0.f, v0.c[c]) + fmaxf(0.f, -v1));
            const float mm = M.c[c] + (fminf(0.f, v0.c[c]) + fminf(0.f, -v1));
            const float bmx = tup - lo.c[c], bmn = tlo - lo.c[c];
            rp.c[c] = fminf(1.f, qdiv(bmx, pp * s + eps));
            rm.c[c] = fminf(1.f, qdiv(bmn, mm * s - eps));
            bp.c[c] = tup;
            bm.c[c] = tlo;
        }
        if (k.out && gq >= 0) {
            vst<G>(grp<G>(B.Rp, gq, B.sN), i, rp);
            vst<G>(grp<G>(B.Rm, gq, B.sN), i, rm);
            if (kFctClamp) {
                vst<G>(grp<G>(B.Bp, gq, B.sN), i, bp);
                vst<G>(grp<G>(B.Bm, gq, B.sN), i, bm);
            }
        }
    };
    int gq;
    if (!next(gq)) return;
    float *cur = sb, *nxt = sb + (size_t)NS * 32 * G;
    issue(gq, cur);
    for (;;) {
        int gn;
        const bool more = next(gn);
        if (more) {
            issue(gn, nxt);
            cpa_wait<1>();
        } else {
            cpa_wait<0>();
        }
        compute(gq, cur);
        if (!more) break;
        float *t = cur;
        cur = nxt;
        nxt = t;
        gq = gn;
    }
}

template <int G, int KD, bool PK>
__device__ __forceinline__ void bounds_node(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int n,
                                            int lane, const WEdges &S, float *sb) {
    using C = Chunk<1, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    if constexpr (KD == 6) {
        if (sb) {
            for (int ch = 0; ch < nch - 1; ch++) bounds_chunk_pf<G, KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1, sb);
            if (PK && P > 1) bounds_chunk_pf<G, KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P, sb);
            else bounds_chunk_pf<G, KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1, sb);
            return;
        }
    }
    for (int ch = 0; ch < nch - 1; ch++) bounds_chunk<G, KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1);
    if (PK && KD <= 6 && P > 1) bounds_chunk<G, KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P);
    else bounds_chunk<G, KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1);
}

// sb: the warp's shared-memory staging (null: the gathers go to registers)
template <int G, bool WIDE, bool PK>
__device__ __forceinline__ void bounds_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                            WEdges *Se, float *sb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) bounds_node<G, kMaxDeg, PK>(tp, g, B, dt, n, lane, S, nullptr);
    else if (S.deg <= 6) bounds_node<G, 6, PK>(tp, g, B, dt, n, lane, S, sb);
    else bounds_node<G, 8, PK>(tp, g, B, dt, n, lane, S, nullptr);
}

// staging bytes per warp of the bounds kernel (two buffers of NS entries)
template <int G>
__host__ __device__ constexpr int stage_bytes_bounds() { return 2 * kNsBounds * 32 * G * 4; }

// STG: each pass's gathers staged in shared memory (fewer resident warps) instead of registers
template <int G, bool WIDE, bool STG>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : (STG ? MinB<G>::node_stg : MinB<G>::bounds_reg))
k32_bounds(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ WEdges Se[kWB];
    extern __shared__ __align__(16) float dsm[];
    float *sb = (WIDE || !STG) ? nullptr : dsm + (size_t)(threadIdx.x >> 5) * (stage_bytes_bounds<G>() / 4);
    FOR_WARP_UNITS(j, node_units<WIDE>(tp)) bounds_unit<G, WIDE, true>(tp, g, B, dt, j, Se, sb);
}

// ---------------------------------------------------------------------------
// k32_vdiff: implicit vertical diffusion of the advected columns (in Tnew)
// ---------------------------------------------------------------------------
// Forward substitution tp_k = inv_k rhs_k - a_k inv_k tp_{k-1} and back substitution
// x_k = tp_k - cp_k x_{k+1} (oce_ale_tracer.F90:1406-1422) with the column's k32_vfactors
// factors, as scans of affine maps y -> A y + B.  Each lane holds K consecutive levels of the
// column (K = ceil(layers / 32): one warp covers the whole column): it composes its K maps in
// registers, the warp scans the lane maps (five shuffles), and each lane then runs its K
// levels from the carry it receives.  The multipliers A depend on the column only: the lane
// products and their partial products at each scan step are formed once per node (shared
// memory), so a slot's scan step is one shuffle and one multiply-add, and a column costs a slot
// 14 shuffles whatever its depth.  rhs_k = -a_k (T_{k-1} - T_k) - c_k (T_{k+1} - T_k)
// (+ bc_surface at the top, :1216-1229, 1377-1383); T += x.
// CG: the column was stored by the same kernel (the update with the diffusion as its epilogue):
// its values are read at L2.
constexpr int kWV = 4;                    // warps (nodes) per block of the diffusion kernel
constexpr int kScan = 5;                  // steps of a 32-lane scan

struct VdiffWarp {
    float4 fac[130];                      // (a, c, 1/m, c/m), 1-based levels
    float af[kScan][32];                  // forward: lane-map product of the window at each step (0 below the offset)
    float ab[kScan][32];                  // backward (0 past the offset)
};

// per-lane column data of a node: the factors of the lane's K levels
template <int K>
struct VdiffLane {
    float a[K], c[K], inv[K], A[K], Ad[K];
    bool ok[K];
};

// a group's column values of the lane's K levels and its surface flux
template <int K, int G>
struct VdiffCol {
    Vec<G> a[K];
    Vec<G> bc;
};

template <int K, int G, bool CG>
__device__ __forceinline__ void vdiff_load(const DTopo &tp, const B32View &B, int n, int lane, int nzmin, int gq,
                                           const VdiffLane<K> &V, VdiffCol<K, G> &x) {
    const int L1 = tp.L1;
    const int nz0 = nzmin + lane * K;  // the lane's first level
    const float *Tg = grp<G>(B.Tnew, gq, B.sN);
    x.bc = B.fsurf ? vld<G>(B.fsurf, gq * tp.N2 + n) : vfill<G>(0.f);
#pragma unroll
    for (int t = 0; t < K; t++)
        x.a[t] = CG ? vldcg<G>(V.ok[t], Tg, n * L1 + nz0 + t - 1) : vldc<G>(V.ok[t], Tg, n * L1 + nz0 + t - 1);
}

template <int K, int G>
__device__ __forceinline__ void vdiff_group(const DTopo &tp, const B32View &B, int n, int lane, int nzmin, int nzmax,
                                            int gq, const VdiffLane<K> &V, const VdiffWarp &W,
                                            const VdiffCol<K, G> &x) {
    const int L1 = tp.L1;
    const int nz0 = nzmin + lane * K;  // the lane's first level
    float *__restrict__ Tg = grp<G>(B.Tnew, gq, B.sN);
    const Vec<G>(&a)[K] = x.a;
    const Vec<G> &bc = x.bc;
    Vec<G> y[K];
#pragma unroll
    for (int c = 0; c < G; c++) {
        // the levels next to the lane's ends come from the neighbouring lanes
        const float up = sh_up(a[K - 1].c[c], 1), dn = sh_dn(a[0].c[c], 1);
        float bl = 0.f;  // the lane's composed forward map applied to 0
#pragma unroll
        for (int t = 0; t < K; t++) {
            const int nz = nz0 + t;
            const float tu = t > 0 ? a[t - 1].c[c] : up, td = t < K - 1 ? a[t + 1].c[c] : dn;
            const float tc = a[t].c[c];
            float r = 0.f;
            if (nz > nzmin) r -= V.a[t] * (tu - tc);
            if (nz < nzmax - 1) r -= V.c[t] * (td - tc);
            if (nz == nzmin) r += bc.c[c];
            y[t].c[c] = V.ok[t] ? r * V.inv[t] : 0.f;
            bl = fmaf(V.A[t], bl, y[t].c[c]);
        }
        // inclusive scan of the lane maps: bl = tp at the lane's last level
#pragma unroll
        for (int s = 0, off = 1; s < kScan; s++, off <<= 1) bl = fmaf(W.af[s][lane], __shfl_up_sync(kFull, bl, off), bl);
        float yv = __shfl_up_sync(kFull, bl, 1);
        if (lane == 0) yv = 0.f;
#pragma unroll
        for (int t = 0; t < K; t++) {
            yv = fmaf(V.A[t], yv, y[t].c[c]);
            y[t].c[c] = yv;
        }
        // back substitution: the lane's composed backward map, the suffix scan, the lane's levels
        float xl = 0.f;
#pragma unroll
        for (int t = K - 1; t >= 0; t--) xl = fmaf(V.Ad[t], xl, y[t].c[c]);
#pragma unroll
        for (int s = 0, off = 1; s < kScan; s++, off <<= 1)
            xl = fmaf(W.ab[s][lane], __shfl_down_sync(kFull, xl, off), xl);
        float xv = __shfl_down_sync(kFull, xl, 1);
        if (lane == 31) xv = 0.f;
#pragma unroll
        for (int t = K - 1; t >= 0; t--) {
            xv = fmaf(V.Ad[t], xv, y[t].c[c]);
            y[t].c[c] = a[t].c[c] + xv;
        }
    }
#pragma unroll
    for (int t = 0; t < K; t++) {
        if (!V.ok[t]) continue;
        bool fin = true;
#pragma unroll
        for (int c = 0; c < G; c++) fin = fin && isfinite(y[t].c[c]);
        vst<G>(Tg, n * L1 + nz0 + t - 1, y[t]);
        if (!fin) atomicOr(B.status, 1u);
    }
}

template <int K, int G, bool CG>
__device__ __forceinline__ void vdiff_node(const DTopo &tp, const B32View &B, int n, int lane, int nzmin, int nzmax,
                                           VdiffWarp &W) {
    VdiffLane<K> V;
    float A = 1.f, Ad = 1.f;
#pragma unroll
    for (int t = 0; t < K; t++) {
        const int nz = nzmin + lane * K + t;
        V.ok[t] = nz <= nzmax - 1;
        const float4 fz = V.ok[t] ? W.fac[nz] : make_float4(0.f, 0.f, 0.f, 0.f);
        V.a[t] = fz.x;
        V.c[t] = fz.y;
        V.inv[t] = fz.z;
        // levels past the column's end are identity maps
        V.A[t] = V.ok[t] ? -(fz.x * fz.z) : 1.f;
        V.Ad[t] = V.ok[t] ? -fz.w : 1.f;
        A *= V.A[t];
        Ad *= V.Ad[t];
    }
    // partial products of the lane maps at each scan step
#pragma unroll
    for (int s = 0, off = 1; s < kScan; s++, off <<= 1) {
        W.af[s][lane] = lane >= off ? A : 0.f;
        W.ab[s][lane] = lane + off < 32 ? Ad : 0.f;
        const float Ap = __shfl_up_sync(kFull, A, off), An = __shfl_down_sync(kFull, Ad, off);
        if (lane >= off) A *= Ap;
        if (lane + off < 32) Ad *= An;
    }
    __syncwarp();
    unsigned long long todo = (B.ivd & ~B.wimpl) & (B.ng >= 64 ? ~0ull : ((1ull << B.ng) - 1));
    // (loading the next group's column during the current solve measured slower after the
    // update: the extra registers spill)
    while (todo) {
        const int gq = __ffsll((long long)todo) - 1;
        todo &= todo - 1;
        VdiffCol<K, G> x;
        vdiff_load<K, G, CG>(tp, B, n, lane, nzmin, gq, V, x);
        vdiff_group<K, G>(tp, B, n, lane, nzmin, nzmax, gq, V, W, x);
    }
}

template <int G, bool CG = false>
__device__ __forceinline__ void vdiff_unit(const DTopo &tp, const B32View &B, const VFactors &vf, int n,
                                           VdiffWarp &W) {
    const int lane = threadIdx.x & 31;
    if (n >= tp.N2) return;
    const int L1 = tp.L1;
    const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
    const int K = (nzmax - nzmin + 31) / 32;
    __syncwarp();  // the previous node's reads of W are done
    for (int nz = nzmin + lane; nz <= nzmax - 1; nz += 32) {
        const int i = n * L1 + nz - 1;
        W.fac[nz] = make_float4(vf.a[i], vf.c[i], vf.inv[i], vf.cp[i]);
    }
    __syncwarp();
    switch (K) {
        case 1: vdiff_node<1, G, CG>(tp, B, n, lane, nzmin, nzmax, W); break;
        case 2: vdiff_node<2, G, CG>(tp, B, n, lane, nzmin, nzmax, W); break;
        case 3: vdiff_node<3, G, CG>(tp, B, n, lane, nzmin, nzmax, W); break;
        default: vdiff_node<4, G, CG>(tp, B, n, lane, nzmin, nzmax, W); break;
    }
}

// ---------------------------------------------------------------------------
// k32_update: limited update, T*
// ---------------------------------------------------------------------------
template <int G, int KD, bool PACK>
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
    // a dry slot gathers the node's own R (finite); its ADh is not loaded (zero)
    int off[KD], eo[KD];
    unsigned okx = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : i;
        eo[u] = ok ? S.e[u] * L1 + nz - 1 : 0;
        okx |= ok ? 1u << u : 0u;
    }
#pragma unroll 1
    for (int g0 = 0; g0 < B.ng; g0 += PACK ? P : 1) {
        // the lane's group (packed: the group of its segment)
        const int gq = g0 + k.q;
        const bool on = gq < B.ng;
        const int gc = on ? gq : g0;
        const bool fct = (B.fct >> gc) & 1ull;
        const bool dif = (B.diff >> gc) & 1ull;
        const bool lv = k.lvl && on;
        const bool lf = lv && fct;
        const float *__restrict__ Rp = grp<G>(B.Rp, gc, B.sN);
        const float *__restrict__ Rm = grp<G>(B.Rm, gc, B.sN);
        const float *__restrict__ ADh = grp<G>(B.ADh, gc, B.sE);
        float *__restrict__ Tn = grp<G>(B.Tnew, gc, B.sN);
        // every load of the group's chunk first
        const Vec<G> lo = vldc<G>(lv, grp<G>(B.LO, gc, B.sN), i);
        const Vec<G> f0 = vldc<G>(lv, grp<G>(B.ADv, gc, B.sNI), iv);
        const Vec<G> r0p = lf ? vld<G>(Rp, i) : vfill<G>(1.f);
        const Vec<G> r0m = lf ? vld<G>(Rm, i) : vfill<G>(1.f);
        const Vec<G> tbp = vldc<G>(lf && kFctClamp, grp<G>(B.Bp, gc, B.sN), i);
        const Vec<G> tbm = vldc<G>(lf && kFctClamp, grp<G>(B.Bm, gc, B.sN), i);
        // the diffusion increment k32_diff parked in Tnew (the limiter acts on advection only)
        const Vec<G> dd = vldc<G>(lv && dif, Tn, i);
        Vec<G> hs = vfill<G>(0.f);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> x = vldc<G>(lv && ((okx >> u) & 1u), ADh, eo[u]);
            const Vec<G> rmp = lf ? vld<G>(Rp, off[u]) : vfill<G>(1.f);
            const Vec<G> rmm = lf ? vld<G>(Rm, off[u]) : vfill<G>(1.f);
            const bool ow = (own >> u) & 1u;
            // horizontal limiting (oce_adv_tra_fct.F90:468-500) seen from the node: with G the
            // antidiffusive flux into the node and m the other end, G >= 0 takes
            // min(R+(n), R-(m)), G < 0 takes min(R-(n), R+(m))
#pragma unroll
            for (int c = 0; c < G; c++) {
                float Gf = ow ? x.c[c] : -x.c[c];
                if (fct) Gf *= Gf >= 0.f ? fminf(r0p.c[c], rmm.c[c]) : fminf(r0m.c[c], rmp.c[c]);
                hs.c[c] += Gf;
            }
        }
        Vec<G> out;
#pragma unroll
        for (int c = 0; c < G; c++) {
            // vertical limiting (oce_adv_tra_fct.F90:425-456): interface nz by R of layers
            // nz-1 and nz; the next interface is the lane below's
            const float rux = sh_up(r0p.c[c], 1), ruy = sh_up(r0m.c[c], 1);
            float fz = f0.c[c];
            if (fct) {
                if (nz == nzmin) fz *= fz >= 0.f ? r0p.c[c] : r0m.c[c];
                else fz *= fz >= 0.f ? fminf(ruy, r0p.c[c]) : fminf(rux, r0m.c[c]);
            }
            float f1 = sh_dn(fz, 1);
            if (nz == nzmax - 1) f1 = 0.f;
            // del_ttf = (LO hnode_new - T hnode) + limited flux divergence dt / areasvol;
            // T* = T + (del_ttf + T (hnode - hnode_new)) / hnode_new = LO + fluxes dt / areasvol / hnode_new
            // (oce_adv_tra_driver.F90:535-620, oce_ale_tracer.F90:319-321, 743-754)
            float val = lo.c[c] + ((fz - f1) + hs.c[c]) * sdt;
            if (kFctClamp && k.out && on && fct) {
                const float vc = fminf(fmaxf(val, tbm.c[c]), tbp.c[c]);
                // a clamp beyond round-off means the limiter itself failed
                if (fabsf(vc - val) > 1e-5f * (tbp.c[c] - tbm.c[c]) + 1e-6f * fabsf(vc)) atomicOr(B.status, 2u);
                val = vc;
            }
            if (dif) val += dd.c[c];
            out.c[c] = val;
        }
        if (k.out && on) {
            vst<G>(Tn, i, out);
#pragma unroll
            for (int c = 0; c < G; c++)
                if (!isfinite(out.c[c])) atomicOr(B.status, 1u);
        }
    }
}

// The same chunk with each pass's gathers staged in shared memory: entries LO, ADv, R+, R-, the
// two bounds and the parked diffusion increment of the node, then ADh, R+, R- of every slot
// (a dry slot stages zeros for ADh and the node's own R).
constexpr int kNsUpdate = 7 + 3 * 6;
template <int G, int KD, bool PACK>
__device__ __forceinline__ void update_chunk_pf(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt,
                                                int n, int lane, const WEdges &S, int ch, int W, int P, float *sb) {
    using C = Chunk<1, 1>;
    constexpr int NS = 7 + 3 * KD;
    static_assert(NS <= kNsUpdate, "staging sized for six edge slots");
    const int L1 = tp.L1, nl = tp.nl;
    const int nzmin = S.nzmin, nzmax = S.nzmax, deg = S.deg;
    const unsigned own = S.own;
    const C k = PACK ? C(nzmin, nzmax, ch, lane, W, P) : C(nzmin, nzmax, ch, lane);
    const int nz = k.nz;
    const int i = n * L1 + nz - 1, iv = n * nl + nz - 1;
    const float sdt = k.lvl ? qdiv(dt, g.areasvol[iv] * g.hnode_new[i]) : 0.f;
    int off[KD], eo[KD];
    unsigned okx = 0;
#pragma unroll
    for (int u = 0; u < KD; u++) {
        const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
        off[u] = ok ? S.m[u] * L1 + nz - 1 : (k.lvl ? i : 0);
        eo[u] = ok ? S.e[u] * L1 + nz - 1 : 0;
        okx |= ok ? 1u << u : 0u;
    }
    const int npass = PACK ? (B.ng + P - 1) / P : B.ng;
    // the lane's group in pass p (packed: the group of its segment)
    auto grp_of = [&](int p) { return PACK ? p * P + k.q : p; };
    auto issue = [&](int p, float *buf) {
        const int gq = grp_of(p);
        const bool on = gq < B.ng;
        const int gc = on ? gq : 0;
        const bool lv = k.lvl && on;
        const bool lf = lv && ((B.fct >> gc) & 1ull);
        const bool ld = lv && ((B.diff >> gc) & 1ull);
        const int ii = lv ? i : 0;
        const float *Rp = grp<G>(B.Rp, gc, B.sN), *Rm = grp<G>(B.Rm, gc, B.sN);
        const float *ADh = grp<G>(B.ADh, gc, B.sE);
        cpa<G>(stg<G>(buf, 0, lane), grp<G>(B.LO, gc, B.sN) + (size_t)ii * G, lv);
        cpa<G>(stg<G>(buf, 1, lane), grp<G>(B.ADv, gc, B.sNI) + (size_t)(lv ? iv : 0) * G, lv);
        cpa<G>(stg<G>(buf, 2, lane), Rp + (size_t)ii * G, lf);
        cpa<G>(stg<G>(buf, 3, lane), Rm + (size_t)ii * G, lf);
        // (without the clamp the bounds are not allocated: the zero-filled copies name LO)
        cpa<G>(stg<G>(buf, 4, lane), grp<G>(kFctClamp ? B.Bp : B.LO, gc, B.sN) + (size_t)ii * G, lf && kFctClamp);
        cpa<G>(stg<G>(buf, 5, lane), grp<G>(kFctClamp ? B.Bm : B.LO, gc, B.sN) + (size_t)ii * G, lf && kFctClamp);
        cpa<G>(stg<G>(buf, 6, lane), grp<G>(B.Tnew, gc, B.sN) + (size_t)ii * G, ld);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            cpa<G>(stg<G>(buf, 7 + 3 * u, lane), ADh + (size_t)eo[u] * G, lv && ((okx >> u) & 1u));
            cpa<G>(stg<G>(buf, 8 + 3 * u, lane), Rp + (size_t)off[u] * G, lf);
            cpa<G>(stg<G>(buf, 9 + 3 * u, lane), Rm + (size_t)off[u] * G, lf);
        }
        cpa_commit();
    };
    auto compute = [&](int p, float *buf) {
        const int gq = grp_of(p);
        const bool on = gq < B.ng;
        const int gc = on ? gq : 0;
        const bool fct = (B.fct >> gc) & 1ull;
        const bool dif = (B.diff >> gc) & 1ull;
        const Vec<G> lo = lds<G>(stg<G>(buf, 0, lane));
        const Vec<G> f0 = lds<G>(stg<G>(buf, 1, lane));
        const Vec<G> r0p = lds<G>(stg<G>(buf, 2, lane));
        const Vec<G> r0m = lds<G>(stg<G>(buf, 3, lane));
        Vec<G> hs = vfill<G>(0.f);
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const Vec<G> x = lds<G>(stg<G>(buf, 7 + 3 * u, lane));
            const bool ow = (own >> u) & 1u;
            if (fct) {
                const Vec<G> rmp = lds<G>(stg<G>(buf, 8 + 3 * u, lane));
                const Vec<G> rmm = lds<G>(stg<G>(buf, 9 + 3 * u, lane));
#pragma unroll
                for (int c = 0; c < G; c++) {
                    float Gf = ow ? x.c[c] : -x.c[c];
                    Gf *= Gf >= 0.f ? fminf(r0p.c[c], rmm.c[c]) : fminf(r0m.c[c], rmp.c[c]);
                    hs.c[c] += Gf;
                }
            } else {
#pragma unroll
                for (int c = 0; c < G; c++) hs.c[c] += ow ? x.c[c] : -x.c[c];
            }
        }
        const Vec<G> tbp = lds<G>(stg<G>(buf, 4, lane));
        const Vec<G> tbm = lds<G>(stg<G>(buf, 5, lane));
        const Vec<G> dd = lds<G>(stg<G>(buf, 6, lane));
        Vec<G> out;
#pragma unroll
        for (int c = 0; c < G; c++) {
            const float rux = sh_up(r0p.c[c], 1), ruy = sh_up(r0m.c[c], 1);
            float fz = f0.c[c];
            if (fct) {
                if (nz == nzmin) fz *= fz >= 0.f ? r0p.c[c] : r0m.c[c];
                else fz *= fz >= 0.f ? fminf(ruy, r0p.c[c]) : fminf(rux, r0m.c[c]);
            }
            float f1 = sh_dn(fz, 1);
            if (nz == nzmax - 1) f1 = 0.f;
            float val = lo.c[c] + ((fz - f1) + hs.c[c]) * sdt;
            if (kFctClamp && k.out && on && fct) {
                const float vc = fminf(fmaxf(val, tbm.c[c]), tbp.c[c]);
                if (fabsf(vc - val) > 1e-5f * (tbp.c[c] - tbm.c[c]) + 1e-6f * fabsf(vc)) atomicOr(B.status, 2u);
                val = vc;
            }
            if (dif) val += dd.c[c];
            out.c[c] = val;
        }
        if (k.out && on) {
            vst<G>(grp<G>(B.Tnew, gc, B.sN), i, out);
#pragma unroll
            for (int c = 0; c < G; c++)
                if (!isfinite(out.c[c])) atomicOr(B.status, 1u);
        }
    };
    issue(0, sb);
    float *cur = sb, *nxt = sb + (size_t)NS * 32 * G;
    for (int p = 0; p < npass; p++) {
        if (p + 1 < npass) {
            issue(p + 1, nxt);
            cpa_wait<1>();
        } else {
            cpa_wait<0>();
        }
        compute(p, cur);
        float *t = cur;
        cur = nxt;
        nxt = t;
    }
}

template <int G, int KD, bool PK>
__device__ __forceinline__ void update_node(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt,
                                            int n, int lane, const WEdges &S, float *sb) {
    using C = Chunk<1, 1>;
    const int nch = C::count(S.nzmin, S.nzmax);
    const int W = C::last_width(S.nzmin, S.nzmax), P = 32 / W;
    if constexpr (KD == 6) {
        if (sb) {
            for (int ch = 0; ch < nch - 1; ch++) update_chunk_pf<G, KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1, sb);
            if (PK && P > 1) update_chunk_pf<G, KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P, sb);
            else update_chunk_pf<G, KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1, sb);
            return;
        }
    }
    for (int ch = 0; ch < nch - 1; ch++) update_chunk<G, KD, false>(tp, g, B, dt, n, lane, S, ch, 32, 1);
    if (PK && KD <= 6 && P > 1) update_chunk<G, KD, true>(tp, g, B, dt, n, lane, S, nch - 1, W, P);
    else update_chunk<G, KD, false>(tp, g, B, dt, n, lane, S, nch - 1, 32, 1);
}

// VD: the implicit vertical diffusion of the node's column follows its update in the same warp
// (the diffusion is column-local: it reads only the column's own T*, which the warp has just
// stored and reads back at L2), so T* is not written to and read back from HBM between two
// launches.  Vw: the warp's diffusion workspace.
template <int G, bool WIDE, bool PK, bool VD = false>
__device__ __forceinline__ void update_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                            WEdges *Se, float *sb, const VFactors *vf = nullptr,
                                            VdiffWarp *Vw = nullptr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) update_node<G, kMaxDeg, PK>(tp, g, B, dt, n, lane, S, nullptr);
    else if (S.deg <= 6) update_node<G, 6, PK>(tp, g, B, dt, n, lane, S, sb);
    else update_node<G, 8, PK>(tp, g, B, dt, n, lane, S, nullptr);
    // (vdiff_unit opens with a __syncwarp: every lane's T* stores are ordered before the reads)
    if constexpr (VD) vdiff_unit<G, true>(tp, B, *vf, n, *Vw);
}

template <int G>
__host__ __device__ constexpr int stage_bytes_update() { return 2 * kNsUpdate * 32 * G * 4; }

// VD: with the implicit vertical diffusion of the groups in ivd & ~wimpl as the epilogue of each
// node (factors vf); its workspace is the warp's staging buffer in the staged variant (idle once
// the node's last pass has landed), static shared memory otherwise
template <int G, bool WIDE, bool STG, bool VD>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : (STG ? MinB<G>::node_stg : MinB<G>::update_reg))
k32_update(DTopo tp, DGeom<float> g, B32View B, float dt, VFactors vf) {
    __shared__ WEdges Se[kWB];
    extern __shared__ __align__(16) float dsm[];
    constexpr bool kStaged = STG && !WIDE;
    static_assert(sizeof(VdiffWarp) <= stage_bytes_update<G>(), "diffusion workspace inside the staging");
    float *sb = kStaged ? dsm + (size_t)(threadIdx.x >> 5) * (stage_bytes_update<G>() / 4) : nullptr;
    VdiffWarp *Vw = nullptr;
    if constexpr (VD) {
        if constexpr (kStaged) {
            Vw = reinterpret_cast<VdiffWarp *>(sb);
        } else {
            __shared__ VdiffWarp Wsm[kWB];
            Vw = &Wsm[threadIdx.x >> 5];
        }
    }
    FOR_WARP_UNITS(j, node_units<WIDE>(tp)) update_unit<G, WIDE, true, VD>(tp, g, B, dt, j, Se, sb, &vf, Vw);
}

// ---------------------------------------------------------------------------
// k32_vppm: adv_tra_vert_ppm (oce_adv_tra_ver.F90:438-631) on the AB values of the groups
// in the ppm mask, minus the LO flux, into ADv.  A warp per node over chunks of 27 interfaces
// with 3 levels of halo above and 2 below: the interface value tv(k) needs the layers
// k-2..k+1, the flux of interface nz the parabola of layer nz or nz-1.
// ---------------------------------------------------------------------------
template <int G>
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
        unsigned long long todo = B.ppm & (B.ng >= 64 ? ~0ull : ((1ull << B.ng) - 1));
        while (todo) {
            const int gq = __ffsll((long long)todo) - 1;
            todo &= todo - 1;
            const bool lim = (B.fct >> gq) & 1ull;
            const Vec<G> Tv = vldc<G>(k.lvl, grp<G>(B.T, gq, B.sN), i);
            const Vec<G> o1 = vldc<G>(k.lvl, grp<G>(B.O1, gq, B.sN), i);
            const Vec<G> o2 = vldc<G>(k.lvl && B.ab == 3, grp<G>(B.O2, gq, B.sN), i);
            Vec<G> out;
#pragma unroll
            for (int c = 0; c < G; c++) {
                const float Tn = Tv.c[c];
                const float tab = Tn + (k.lvl ? ab_delta(B.ab, Tn, o1.c[c], o2.c[c]) : 0.f);
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
                    float dj = a1 / (a0 + a1 + a2) *
                               ((2.f * a0 + a1) / (a2 + a1) * d10 + (a1 + 2.f * a2) / (a0 + a1) * d0m);
                    float dj1 = a2 / (a1 + a2 + a3) *
                                ((2.f * a1 + a2) / (a3 + a2) * d21 + (a2 + 2.f * a3) / (a1 + a2) * d10);
                    dj = d10 * d0m > 0.f ? copysignf(fminf(fminf(fabsf(dj), 2.f * fabsf(d10)), 2.f * fabsf(d0m)), dj)
                                         : 0.f;
                    dj1 = d21 * d10 > 0.f
                              ? copysignf(fminf(fminf(fabsf(dj1), 2.f * fabsf(d21)), 2.f * fabsf(d10)), dj1)
                              : 0.f;
                    tv = tm1 + a1 / (a1 + a2) * d10 +
                         1.f / (a0 + a1 + a2 + a3) *
                             ((2.f * a2 * a1) / (a1 + a2) * ((a0 + a1) / (2.f * a1 + a2) - (a3 + a2) / (2.f * a2 + a1)) *
                                  d10 -
                              a1 * (a0 + a1) / (2.f * a1 + a2) * dj1 + a2 * (a2 + a3) / (a1 + 2.f * a2) * dj);
                }
                const float tvu = sh_up(tv, 1), tvd = sh_dn(tv, 1);
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
                    if ((aR - aL) * (tt - 0.5f * (aR + aL)) < -((aR - aL) * (aR - aL) * (1.f / 6.f)))
                        aR = 3.f * tt - 2.f * aL;
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
                out.c[c] = Cf - fl;
            }
            if (k.out) vst<G>(grp<G>(B.ADv, gq, B.sNI), iv, out);
        }
    }
}

template <int G>
__global__ void __launch_bounds__(kTB) k32_vppm(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, float dt) {
    FOR_WARP_UNITS(n, tp.N2) vppm_node<G>(tp, g, f, B, dt, n, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// split vertical velocity, FP32 form: adv_tra_vert_impl by w_i on the LO values of the FCT
// groups (oce_adv_tra_ver.F90:90-240), and the implicit vertical diffusion with the w_i
// terms for the groups without the limiter (oce_ale_tracer.F90:907-1435, do_wimpl).  One
// thread per column, FP64 arithmetic; scratch holds Z_n, cp and tp level-major.
// ---------------------------------------------------------------------------
// one slot's column of a group field (1-based levels)
struct SlotCol {
    float *p;
    int G;
    __device__ __forceinline__ float &operator[](int nz) const { return p[(size_t)(nz - 1) * G]; }
};

__device__ __forceinline__ void lo_impl_slot(const float *hn, const float *ar, const float *av, const float *wi,
                                             double dt, double *cps, double *tps, size_t N2, int n, int nzmin,
                                             int nzmax, SlotCol Tc) {
#define CP(k) cps[(size_t)(k) * N2 + n]
#define TP(k) tps[(size_t)(k) * N2 + n]
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
#undef CP
#undef TP
}

template <int G>
__device__ __forceinline__ void lo_impl_column(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f,
                                               const B32View &B, double dt, double *scratch, int n) {
    const int L1 = tp.L1, nl = tp.nl;
    const size_t N2 = tp.N2;
    double *cps = scratch, *tps = scratch + (size_t)(L1 + 1) * N2;
    const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
    const float *hn = g.hnode_new + (size_t)n * L1 - 1;
    const float *ar = g.area + (size_t)n * nl - 1, *av = g.areasvol + (size_t)n * nl - 1;
    const float *wi = f.wi + (size_t)n * nl - 1;
    unsigned long long todo = B.fct & (B.ng >= 64 ? ~0ull : ((1ull << B.ng) - 1));
    while (todo) {
        const int gq = __ffsll((long long)todo) - 1;
        todo &= todo - 1;
        float *base = grp<G>(B.LO, gq, B.sN) + (size_t)n * L1 * G;
        for (int c = 0; c < G; c++)
            lo_impl_slot(hn, ar, av, wi, dt, cps, tps, N2, n, nzmin, nzmax, SlotCol{base + c, G});
    }
}

template <int G>
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
    unsigned long long todo = B.wimpl & (B.ng >= 64 ? ~0ull : ((1ull << B.ng) - 1));
    while (todo) {
        const int gq = __ffsll((long long)todo) - 1;
        todo &= todo - 1;
        float *base = grp<G>(B.Tnew, gq, B.sN) + (size_t)n * L1 * G;
        for (int cs = 0; cs < G; cs++) {
            const SlotCol Tc{base + cs, G};
            const double bc = B.fsurf ? (double)B.fsurf[((size_t)gq * N2 + n) * G + cs] : 0.0;
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
    }
#undef ZN
#undef CP
#undef TP
}

template <int G>
__global__ void __launch_bounds__(128) k32_lo_impl(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, double dt,
                                                   double *scratch) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < tp.N2) lo_impl_column<G>(tp, g, f, B, dt, scratch, n);
}
template <int G>
__global__ void __launch_bounds__(128) k32_vdiff_w(DTopo tp, DGeom<float> g, DForcing<float> f, B32View B, double dt,
                                                   double *scratch) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < tp.N2) vdiff_w_column<G>(tp, g, f, B, dt, scratch, n);
}

// ---------------------------------------------------------------------------
// diffusion of diff_tracers_ale (oce_ale_tracer.F90:560-772) in the FP32 form
// ---------------------------------------------------------------------------
// k32_hdiff: diff_part_hor_redi (:1526-1689) flux c of every edge-layer from the element
// gradients of the current values: segments A/D (element 1), B/E (element 2), C (both); with
// Redi the gradient gains S_xy Tz: Tz at each edge node the layer mean of the vertical gradient
// (tracer_gradient_z, 0 at the column's top and bottom interfaces), S_xy Tz = (Tz(n1) S(n1)
// + Tz(n2) S(n2)) / 2 (:1583-1595)
//
// 1 / dz of the vertical gradient at interface nz of node n (0 where tr_z is 0)
__device__ __forceinline__ float trz_rdz(const DTopo &tp, const DGeom<float> &g, int n, int nz) {
    if (nz <= tp.n_ulev[n] || nz >= tp.n_nlev[n]) return 0.f;
    const int i = n * tp.L1 + nz - 1;
    return 2.f / (g.hnode[i - 1] + g.hnode[i]);
}

template <int G>
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
    const bool redi = B.slope != nullptr;
    for (int nz0 = tp.e_lo[e]; nz0 <= tp.e_hi[e]; nz0 += 32) {
        const int nz = nz0 + lane;
        if (nz > tp.e_hi[e]) continue;
        // Redi: 1/dz of the gradients above and below the layer at both nodes, the slopes
        float ru1 = 0.f, rd1 = 0.f, ru2 = 0.f, rd2 = 0.f, sx1 = 0.f, sy1 = 0.f, sx2 = 0.f, sy2 = 0.f;
        if (redi) {
            ru1 = trz_rdz(tp, g, n1, nz);
            rd1 = trz_rdz(tp, g, n1, nz + 1);
            ru2 = trz_rdz(tp, g, n2, nz);
            rd2 = trz_rdz(tp, g, n2, nz + 1);
            const float *s1 = B.slope + 3 * (size_t)(n1 * L1 + nz - 1), *s2 = B.slope + 3 * (size_t)(n2 * L1 + nz - 1);
            sx1 = s1[0];
            sy1 = s1[1];
            sx2 = s2[0];
            sy2 = s2[1];
        }
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
        for (int gq = 0; gq < B.ng; gq++) {
            const float *__restrict__ T = grp<G>(B.T, gq, B.sN);
            const Vec<G> va = vldc<G>(u1, T, a0 * L1 + nz - 1), vb = vldc<G>(u1, T, a1 * L1 + nz - 1),
                         vc = vldc<G>(u1, T, a2 * L1 + nz - 1);
            const Vec<G> wa = vldc<G>(u2, T, b0 * L1 + nz - 1), wb = vldc<G>(u2, T, b1 * L1 + nz - 1),
                         wc = vldc<G>(u2, T, b2 * L1 + nz - 1);
            Vec<G> tz1 = vfill<G>(0.f), tz2 = vfill<G>(0.f);
            if (redi) {
                // the column neighbours of both edge nodes (rd = 0 where nz + 1 is not a gradient
                // interface, ru = 0 likewise, so the loads stay inside the columns)
                const Vec<G> m0 = vldc<G>(ru1 != 0.f, T, n1 * L1 + nz - 2), m1 = vld<G>(T, n1 * L1 + nz - 1),
                             m2 = vldc<G>(rd1 != 0.f, T, n1 * L1 + nz);
                const Vec<G> o0 = vldc<G>(ru2 != 0.f, T, n2 * L1 + nz - 2), o1 = vld<G>(T, n2 * L1 + nz - 1),
                             o2 = vldc<G>(rd2 != 0.f, T, n2 * L1 + nz);
#pragma unroll
                for (int c = 0; c < G; c++) {
                    tz1.c[c] = 0.5f * ((m0.c[c] - m1.c[c]) * ru1 + (m1.c[c] - m2.c[c]) * rd1);
                    tz2.c[c] = 0.5f * ((o0.c[c] - o1.c[c]) * ru2 + (o1.c[c] - o2.c[c]) * rd2);
                }
            }
            Vec<G> out;
#pragma unroll
            for (int c = 0; c < G; c++) {
                float tx1 = 0.f, ty1 = 0.f, tx2 = 0.f, ty2 = 0.f;
                if (u1) {
                    tx1 = p0 * va.c[c] + p1 * vb.c[c] + p2 * vc.c[c];
                    ty1 = p3 * va.c[c] + p4 * vb.c[c] + p5 * vc.c[c];
                }
                if (u2) {
                    tx2 = q0 * wa.c[c] + q1 * wb.c[c] + q2 * wc.c[c];
                    ty2 = q3 * wa.c[c] + q4 * wb.c[c] + q5 * wc.c[c];
                }
                if (redi) {
                    const float sx = 0.5f * (tz1.c[c] * sx1 + tz2.c[c] * sx2);
                    const float sy = 0.5f * (tz1.c[c] * sy1 + tz2.c[c] * sy2);
                    tx1 += sx;
                    ty1 += sy;
                    tx2 += sx;
                    ty2 += sy;
                }
                float cf = 0.f;
                if (seg == 1) cf = (-dX1 * (Kh * ty1) + dY1 * (Kh * tx1)) * h1;
                else if (seg == 2) cf = (dX2 * (Kh * ty2) - dY2 * (Kh * tx2)) * h2;
                else if (seg == 3)
                    cf = ((dX2 - dX1) * (Kh * (0.5f * (ty1 + ty2))) - (dY2 - dY1) * (Kh * (0.5f * (tx1 + tx2)))) *
                         ((h1 + h2) * 0.5f);
                out.c[c] = cf;
            }
            vst<G>(grp<G>(B.HD, gq, B.sE), e * L1 + nz - 1, out);
        }
    }
}

template <int G>
__global__ void __launch_bounds__(kTB) k32_hdiff(DTopo tp, DGeom<float> g, B32View B) {
    FOR_WARP_UNITS(e, tp.E2) hdiff_edge32<G>(tp, g, B, e);
}

// k32_diff: the diffusion increment to T* of every group in the diff mask, parked in Tnew:
// (sum of the node's edge fluxes +- c) dt / (areasvol hnode_new) and, without implicit vertical
// diffusion, diff_ver_part_expl_ale (:841-902): vd(ul) = surface flux, vd(nz) = Kv (T(nz-1)
// - T(nz)) / (Z(nz-1) - Z(nz)) area, increment (vd(nz) - vd(nz+1)) / (zbar(nz) - zbar(nz+1))
// dt / (areasvol hnode_new).  With Redi, diff_ver_part_redi_expl (:1439-1518): the node
// gradient g(nz) = sum over the node's elements wet at nz of grad T elem_area / 3 / areasvol,
// p = S_xy . g, interface flux vd(nz) = (h(nz-1) p(nz-1) Ki(nz-1) + h(nz) p(nz) Ki(nz)) /
// (h(nz-1) + h(nz)) area(nz) with h = hnode (the reference's depth differences z(nz-1) -
// zbar(nz) = h(nz-1)/2 etc. in exact arithmetic), increment (vd(nz) - vd(nz+1)) dt / (areasvol
// hnode_new)
template <int G, int KD>
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
        // Redi: weights of p above and at the interface nz, 1 / (3 areasvol), the slopes
        float cu = 0.f, cd = 0.f, r3 = 0.f, sx = 0.f, sy = 0.f;
        if (B.slope && k.lvl) {
            r3 = 1.f / (3.f * g.areasvol[iv]);
            sx = B.slope[3 * (size_t)i];
            sy = B.slope[3 * (size_t)i + 1];
            if (nz > nzmin) {
                const float hu = g.hnode[i - 1], hd = g.hnode[i];
                const float w = g.area[iv] / (hu + hd);
                cu = hu * B.Ki[i - 1] * w;
                cd = hd * B.Ki[i] * w;
            }
        }
        unsigned okm = 0;
#pragma unroll
        for (int u = 0; u < KD; u++) {
            const bool ok = u < deg && k.lvl && nz >= S.lo[u] && nz <= S.hi[u];
            okm |= ok ? 1u << u : 0u;
        }
#pragma unroll 1
        for (int gq = 0; gq < B.ng; gq++) {
            if (!((B.diff >> gq) & 1ull)) continue;
            Vec<G> d = vfill<G>(0.f);
            if (B.Ki) {
                const float *__restrict__ HD = grp<G>(B.HD, gq, B.sE);
#pragma unroll
                for (int u = 0; u < KD; u++) {
                    const Vec<G> x = vldc<G>((okm >> u) & 1u, HD, S.e[u] * L1 + nz - 1);
                    const bool ow = (own >> u) & 1u;
#pragma unroll
                    for (int c = 0; c < G; c++) d.c[c] += ow ? x.c[c] : -x.c[c];
                }
#pragma unroll
                for (int c = 0; c < G; c++) d.c[c] *= sdt;
            }
            if (!((B.ivd >> gq) & 1ull)) {
                const Vec<G> Tv = vldc<G>(k.lvl, grp<G>(B.T, gq, B.sN), i);
                const Vec<G> fs = B.fsurf ? vld<G>(B.fsurf, gq * tp.N2 + n) : vfill<G>(0.f);
#pragma unroll
                for (int c = 0; c < G; c++) {
                    const float Tn = Tv.c[c];
                    const float Tu = sh_up(Tn, 1), Td = sh_dn(Tn, 1);
                    const float vd0 = nz == nzmin ? fs.c[c] : kz * (Tu - Tn);
                    const float vd1 = nz == nzmax - 1 ? 0.f : kzd * (Tn - Td);
                    d.c[c] += (vd0 - vd1) * q;
                }
            }
            if (B.slope) {
                const float *__restrict__ T = grp<G>(B.T, gq, B.sN);
                Vec<G> gx = vfill<G>(0.f), gy = vfill<G>(0.f);
                for (int kk = tp.nie_ptr[n]; kk < tp.nie_ptr[n + 1]; kk++) {
                    const int el = tp.nie_idx[kk];
                    const bool wet = k.lvl && nz >= tp.t_ulev[el] && nz <= tp.t_nlev[el] - 1;
                    const float *gs = g.gs + 6 * (size_t)el;
                    const float ea = g.elem_area[el];
                    const Vec<G> ta = vldc<G>(wet, T, tp.t_n[3 * el] * L1 + nz - 1),
                                 tb = vldc<G>(wet, T, tp.t_n[3 * el + 1] * L1 + nz - 1),
                                 tc = vldc<G>(wet, T, tp.t_n[3 * el + 2] * L1 + nz - 1);
#pragma unroll
                    for (int c = 0; c < G; c++) {
                        gx.c[c] += (gs[0] * ta.c[c] + gs[1] * tb.c[c] + gs[2] * tc.c[c]) * ea;
                        gy.c[c] += (gs[3] * ta.c[c] + gs[4] * tb.c[c] + gs[5] * tc.c[c]) * ea;
                    }
                }
#pragma unroll
                for (int c = 0; c < G; c++) {
                    const float pz = (sx * gx.c[c] + sy * gy.c[c]) * r3;
                    const float vd = cu * sh_up(pz, 1) + cd * pz;
                    const float vdn = sh_dn(vd, 1);
                    d.c[c] += (vd - vdn) * sdt;
                }
            }
            if (k.out) vst<G>(grp<G>(B.Tnew, gq, B.sN), i, d);
        }
    }
}

template <int G, bool WIDE>
__device__ __forceinline__ void diff_unit(const DTopo &tp, const DGeom<float> &g, const B32View &B, float dt, int j,
                                          WEdges *Se) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = unit_node<WIDE>(tp, j);
    if (n < 0 || !B.diff) return;
    WEdges &S = Se[warp];
    stage_edges(tp, n, lane, S);
    if ((S.deg > 8) != WIDE) return;
    if (WIDE) diff_node32<G, kMaxDeg>(tp, g, B, dt, n, lane, S);
    else diff_node32<G, 8>(tp, g, B, dt, n, lane, S);
}

template <int G, bool WIDE>
__global__ void __launch_bounds__(kTB) k32_diff(DTopo tp, DGeom<float> g, B32View B, float dt) {
    __shared__ WEdges Se[kWB];
    FOR_WARP_UNITS(j, node_units<WIDE>(tp)) diff_unit<G, WIDE>(tp, g, B, dt, j, Se);
}

template <int G>
__global__ void __launch_bounds__(32 * kWV) k32_vdiff(DTopo tp, B32View B, VFactors vf) {
    __shared__ VdiffWarp Wsm[kWV];
    const int warp = threadIdx.x >> 5;
    for (int n = blockIdx.x * kWV + warp; n < tp.N2; n += gridDim.x * kWV) vdiff_unit<G, false>(tp, B, vf, n, Wsm[warp]);
}

// ---------------------------------------------------------------------------
// content sums and layout conversions
// ---------------------------------------------------------------------------
// FP64 content of every slot of ng groups: block b sums its nodes [b*per, (b+1)*per) in a
// fixed order (threads over nodes, then a tree over the block), out = ordered sum of blocks
template <int G>
__global__ void __launch_bounds__(256) k32_content_partial(DTopo tp, DGeom<float> g, const float *T, int ng,
                                                           double *partials) {
    __shared__ double red[256];
    const int L1 = tp.L1, nl = tp.nl;
    const int per = (tp.N2 + gridDim.x - 1) / gridDim.x;
    const int n0 = blockIdx.x * per, n1 = min(tp.N2, n0 + per);
    for (int gq = 0; gq < ng; gq++) {
        double acc[G];
#pragma unroll
        for (int c = 0; c < G; c++) acc[c] = 0.0;
        const float *Tg = grp<G>(T, gq, (size_t)tp.N2 * L1);
        for (int n = n0 + threadIdx.x; n < n1; n += blockDim.x) {
            const int nzmin = tp.n_ulev[n], nzmax = tp.n_nlev[n];
            for (int nz = nzmin; nz <= nzmax - 1; nz++) {
                const Vec<G> t = vld<G>(Tg, n * L1 + nz - 1);
                const double w = (double)g.hnode_new[n * L1 + nz - 1] * (double)g.areasvol[n * nl + nz - 1];
#pragma unroll
                for (int c = 0; c < G; c++) acc[c] += (double)t.c[c] * w;
            }
        }
#pragma unroll
        for (int c = 0; c < G; c++) {
            red[threadIdx.x] = acc[c];
            __syncthreads();
            for (int s = 128; s > 0; s >>= 1) {
                if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
                __syncthreads();
            }
            if (threadIdx.x == 0) partials[((size_t)blockIdx.x * ng + gq) * G + c] = red[0];
            __syncthreads();
        }
    }
}
__global__ void k32_content_final(const double *partials, int nblk, int nslots, double *out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    double a = 0.0;
    for (int b = 0; b < nblk; b++) a += partials[(size_t)b * nslots + s];
    out[s] = a;
}

template <typename S>
__global__ void k32_put_slot(const S *src, float *grpf, int G, int c, size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        grpf[i * G + c] = (float)src[i];
}
template <typename S>
__global__ void k32_get_slot(const float *grpf, int G, int c, size_t count, S *dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (S)grpf[i * G + c];
}
template <typename S>
__global__ void k32_put_slot_pair(const S *src, float *g1, float *g2, int G, int c, size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        g1[i * G + c] = (float)src[2 * i];
        g2[i * G + c] = (float)src[2 * i + 1];
    }
}
template <typename S>
__global__ void k32_get_slot_pair(const float *g1, const float *g2, int G, int c, size_t count, S *dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        dst[2 * i] = (S)g1[i * G + c];
        dst[2 * i + 1] = (S)g2[i * G + c];
    }
}
// element i of slot c's source is src.p[c][i * stride + off] (stride 2: one level of AB3's
// interleaved valuesold); a null source fills its slot with zeros
template <int G, typename S>
__global__ void k32_pack_group(SlotSrc<S> src, float *grpf, size_t count, int stride, int off) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        Vec<G> v;
#pragma unroll
        for (int c = 0; c < G; c++) v.c[c] = src.p[c] ? (float)src.p[c][i * stride + off] : 0.f;
        vst<G>(grpf, (int)i, v);
    }
}
template <int G, typename S>
__global__ void k32_unpack_group(const float *grpf, size_t count, SlotDst<S> dst, int stride, int off) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const Vec<G> v = vld<G>(grpf, (int)i);
#pragma unroll
        for (int c = 0; c < G; c++)
            if (dst.p[c]) dst.p[c][i * stride + off] = (S)v.c[c];
    }
}

// ---------------------------------------------------------------------------
// multi-instance launches: every stage over all instances of a batch at once
// ---------------------------------------------------------------------------
// Units (edges, column blocks, nodes, items) of all instances are numbered one after
// another; ix.start[i] is instance i's first unit.  A warp (or thread, or block) finds
// its instance by binary search over those offsets (kernel parameters, warp-uniform)
// and runs the single-instance body with that instance's descriptor and its group width.
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
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        vflux_edge(I[i].tp, I[i].g, I[i].f, I[i].VF, u - ix.start[i], threadIdx.x & 31);
    }
}
__global__ void __launch_bounds__(kTB) k32m_vfactors(const Inst32 *__restrict__ I, MultiIdx ix) {
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        vfactors_col(I[i].tp, I[i].g, I[i].f, I[i].dt, I[i].vf, u - ix.start[i], threadIdx.x & 31);
    }
}
// WS: some instance has the split vertical velocity (each instance checks its own switch)
template <bool WIDE, bool WS>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : MinB<4>::lo) k32m_lo_ad(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.G == 4)
            lo_ad_unit<4, WIDE, WS, true>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].VF, I[i].dt, u - ix.start[i], Se, nullptr);
        else
            lo_ad_unit<2, WIDE, WS, true>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].VF, I[i].dt, u - ix.start[i], Se, nullptr);
    }
}
__global__ void __launch_bounds__(kTB, MinB<4>::ho) k32m_ho(const Inst32 *__restrict__ I, MultiIdx ix) {
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.G == 4) ho_unit<4, true, false>(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i], nullptr);
        else ho_unit<2, true, false>(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i], nullptr);
    }
}
__global__ void __launch_bounds__(256) k32m_ho_nodemean(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (I[i].B.G == 4) nodemean_item<4>(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i]);
    else nodemean_item<2>(I[i].tp, I[i].B, I[i].mw, I[i].VF, u - ix.start[i]);
}
template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : MinB<4>::node_reg) k32m_bounds(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.G == 4) bounds_unit<4, WIDE, true>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se, nullptr);
        else bounds_unit<2, WIDE, true>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se, nullptr);
    }
}
// each node's column is then diffused by the same warp where its instance has groups in
// ivd & ~wimpl (as k32_update with the diffusion epilogue)
template <bool WIDE>
__global__ void __launch_bounds__(kTB, WIDE ? 1 : MinB<4>::node_reg) k32m_update(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    __shared__ VdiffWarp Wsm[kWB];
    VdiffWarp *Vw = &Wsm[threadIdx.x >> 5];
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        const Inst32 &d = I[i];
        const bool vd = (d.B.ivd & ~d.B.wimpl) != 0;
        const int j = u - ix.start[i];
        if (d.B.G == 4) {
            if (vd) update_unit<4, WIDE, true, true>(d.tp, d.g, d.B, d.dt, j, Se, nullptr, &d.vf, Vw);
            else update_unit<4, WIDE, true>(d.tp, d.g, d.B, d.dt, j, Se, nullptr);
        } else {
            if (vd) update_unit<2, WIDE, true, true>(d.tp, d.g, d.B, d.dt, j, Se, nullptr, &d.vf, Vw);
            else update_unit<2, WIDE, true>(d.tp, d.g, d.B, d.dt, j, Se, nullptr);
        }
    }
}
__global__ void __launch_bounds__(kTB) k32m_vppm(const Inst32 *__restrict__ I, MultiIdx ix) {
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.ppm && I[i].B.G == 4) vppm_node<4>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dt, u - ix.start[i], threadIdx.x & 31);
        else if (I[i].B.ppm) vppm_node<2>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dt, u - ix.start[i], threadIdx.x & 31);
    }
}
__global__ void __launch_bounds__(128) k32m_lo_impl(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (!I[i].f.wsplit) return;
    if (I[i].B.G == 4) lo_impl_column<4>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
    else lo_impl_column<2>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
}
__global__ void __launch_bounds__(128) k32m_vdiff_w(const Inst32 *__restrict__ I, MultiIdx ix) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ix.start[ix.n]) return;
    const int i = find_inst(ix, u);
    if (!I[i].B.wimpl) return;
    if (I[i].B.G == 4) vdiff_w_column<4>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
    else vdiff_w_column<2>(I[i].tp, I[i].g, I[i].f, I[i].B, I[i].dtd, I[i].scratch, u - ix.start[i]);
}

__global__ void __launch_bounds__(kTB) k32m_hdiff(const Inst32 *__restrict__ I, MultiIdx ix) {
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.G == 4) hdiff_edge32<4>(I[i].tp, I[i].g, I[i].B, u - ix.start[i]);
        else hdiff_edge32<2>(I[i].tp, I[i].g, I[i].B, u - ix.start[i]);
    }
}
template <bool WIDE>
__global__ void __launch_bounds__(kTB) k32m_diff(const Inst32 *__restrict__ I, MultiIdx ix) {
    __shared__ WEdges Se[kWB];
    FOR_WARP_UNITS(u, ix.start[ix.n]) {
        const int i = find_inst(ix, u);
        if (I[i].B.G == 4) diff_unit<4, WIDE>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se);
        else diff_unit<2, WIDE>(I[i].tp, I[i].g, I[i].B, I[i].dt, u - ix.start[i], Se);
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
// warp-per-unit kernels: one warp per unit, or at most blocks_per_sm blocks per SM looping
static int grid_units(int units, const LaunchShape &sh) {
    int b = (units + kWB - 1) / kWB;
    if (sh.blocks_per_sm > 0 && b > 152 * sh.blocks_per_sm) b = 152 * sh.blocks_per_sm;
    return b < 1 ? 1 : b;
}
static int grid_nodes(int n) { return (n + kWB - 1) / kWB; }
static int grid_flat(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 32); }

void b32_vflux(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, float *VF, cudaStream_t s) {
    k32_vflux<<<grid32(tp.E2, kWB), kTB, 0, s>>>(tp, g, f, VF);
}
void b32_vfactors(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, double dt, const VFactors &v,
                  cudaStream_t s) {
    k32_vfactors<<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, (float)dt, v);
}

// dynamic shared memory of the staged node kernels: kWB warps' staging
template <int G>
constexpr int smem_lo_ad() { return kWB * stage_bytes_lo_ad<G>(); }
template <int G>
constexpr int smem_bounds() { return kWB * stage_bytes_bounds<G>(); }
template <int G>
constexpr int smem_update() { return kWB * stage_bytes_update<G>(); }
template <int G>
constexpr int smem_ho() { return kWB * stage_bytes_ho<G>(); }

template <int G>
static cudaError_t prepare_g() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void *fn, int bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    };
    set((const void *)k32_lo_ad<G, false, false, true>, smem_lo_ad<G>());
    set((const void *)k32_lo_ad<G, false, true, true>, smem_lo_ad<G>());
    set((const void *)k32_bounds<G, false, true>, smem_bounds<G>());
    set((const void *)k32_update<G, false, true, false>, smem_update<G>());
    set((const void *)k32_update<G, false, true, true>, smem_update<G>());
    set((const void *)k32_ho<G, true>, smem_ho<G>());
    return e;
}
bool b32_fct_clamp() { return kFctClamp; }

cudaError_t b32_prepare() {
    static cudaError_t done = cudaErrorNotReady;
    if (done == cudaSuccess) return done;
    cudaError_t e = prepare_g<4>();
    if (e == cudaSuccess) e = prepare_g<2>();
    done = e;
    return e;
}

template <int G, bool WS>
static void lo_ad_gw(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B,
                     const float *VF, double dt, const LaunchShape &sh, cudaStream_t s) {
    if (sh.staged)
        k32_lo_ad<G, false, WS, true><<<grid_units(tp.N2, sh), kTB, smem_lo_ad<G>(), s>>>(tp, g, f, B, VF, (float)dt);
    else
        k32_lo_ad<G, false, WS, false><<<grid_units(tp.N2, sh), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
    if (tp.n_wide) k32_lo_ad<G, true, WS, false><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, f, B, VF, (float)dt);
}
template <int G>
static void lo_ad_g(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, const float *VF,
                    double dt, const LaunchShape &sh, cudaStream_t s) {
    if (f.wsplit) lo_ad_gw<G, true>(tp, g, f, B, VF, dt, sh, s);
    else lo_ad_gw<G, false>(tp, g, f, B, VF, dt, sh, s);
}
template <int G>
static void bounds_g(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, const LaunchShape &sh,
                     cudaStream_t s) {
    if (sh.staged) k32_bounds<G, false, true><<<grid_units(tp.N2, sh), kTB, smem_bounds<G>(), s>>>(tp, g, B, (float)dt);
    else k32_bounds<G, false, false><<<grid_units(tp.N2, sh), kTB, 0, s>>>(tp, g, B, (float)dt);
    if (tp.n_wide) k32_bounds<G, true, false><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
}
template <int G, bool VD>
static void update_gv(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, const LaunchShape &sh,
                      const VFactors &vf, cudaStream_t s) {
    const float d = (float)dt;
    if (sh.staged) k32_update<G, false, true, VD><<<grid_units(tp.N2, sh), kTB, smem_update<G>(), s>>>(tp, g, B, d, vf);
    else k32_update<G, false, false, VD><<<grid_units(tp.N2, sh), kTB, 0, s>>>(tp, g, B, d, vf);
    if (tp.n_wide) k32_update<G, true, false, VD><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, d, vf);
}
template <int G>
static void update_g(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, const LaunchShape &sh,
                     const VFactors *vf, cudaStream_t s) {
    if (vf) update_gv<G, true>(tp, g, B, dt, sh, *vf, s);
    else update_gv<G, false>(tp, g, B, dt, sh, VFactors{}, s);
}
void b32_lo_ad(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, const float *VF,
               double dt, const LaunchShape &sh, cudaStream_t s) {
    if (B.G == 4) lo_ad_g<4>(tp, g, f, B, VF, dt, sh, s);
    else lo_ad_g<2>(tp, g, f, B, VF, dt, sh, s);
}
template <int G>
static void ho_g(const DTopo &tp, const B32View &B, const MusclW &mw, const float *VF, const LaunchShape &sh,
                 cudaStream_t s) {
    if (sh.staged) k32_ho<G, true><<<grid_units(tp.E2, sh), kTB, smem_ho<G>(), s>>>(tp, B, mw, VF);
    else k32_ho<G, false><<<grid_units(tp.E2, sh), kTB, 0, s>>>(tp, B, mw, VF);
    if (mw.n_items) {
        int blocks = (mw.n_items + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        k32_ho_nodemean<G><<<blocks, 256, 0, s>>>(tp, B, mw, VF);
    }
}
void b32_ho(const DTopo &tp, const DGeom<float> &, const B32View &B, const MusclW &mw, const float *VF,
            const LaunchShape &sh, cudaStream_t s) {
    if (B.G == 4) ho_g<4>(tp, B, mw, VF, sh, s);
    else ho_g<2>(tp, B, mw, VF, sh, s);
}
void b32_bounds(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, const LaunchShape &sh,
                cudaStream_t s) {
    if (B.G == 4) bounds_g<4>(tp, g, B, dt, sh, s);
    else bounds_g<2>(tp, g, B, dt, sh, s);
}
void b32_update(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, const LaunchShape &sh,
                const VFactors *vf, cudaStream_t s) {
    if (B.G == 4) update_g<4>(tp, g, B, dt, sh, vf, s);
    else update_g<2>(tp, g, B, dt, sh, vf, s);
}
void b32_vdiff(const DTopo &tp, const DForcing<float> &, const B32View &B, const VFactors &v, cudaStream_t s) {
    if (B.G == 4) k32_vdiff<4><<<(tp.N2 + kWV - 1) / kWV, 32 * kWV, 0, s>>>(tp, B, v);
    else k32_vdiff<2><<<(tp.N2 + kWV - 1) / kWV, 32 * kWV, 0, s>>>(tp, B, v);
}
void b32_vppm(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
              cudaStream_t s) {
    if (B.G == 4) k32_vppm<4><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, B, (float)dt);
    else k32_vppm<2><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, f, B, (float)dt);
}
void b32_lo_impl(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
                 double *scratch, cudaStream_t s) {
    if (B.G == 4) k32_lo_impl<4><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
    else k32_lo_impl<2><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
}
void b32_vdiff_w(const DTopo &tp, const DGeom<float> &g, const DForcing<float> &f, const B32View &B, double dt,
                 double *scratch, cudaStream_t s) {
    if (B.G == 4) k32_vdiff_w<4><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
    else k32_vdiff_w<2><<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, f, B, dt, scratch);
}
// Redi K33 = Kv + Ty (oce_ale_tracer.F90:1099-1204) of every interface nzmin < nz < nzmax, one
// thread per column, in FP64 from the FP32 inputs: Ty = (zbar(nz) - Z(nz)) / dZ s3(nz-1)^2
// Ki(nz-1) + (Z(nz-1) - zbar(nz)) / dZ s3(nz)^2 Ki(nz), dZ = Z(nz-1) - Z(nz), zbar / Z of
// hnode_new from zbar_n_bot upward; Kv elsewhere
__global__ void __launch_bounds__(128) k32_k33(DTopo tp, DGeom<float> g, const float *Kv, const float *Ki,
                                               const float *slope, float *K33) {
    const int L1 = tp.L1, nl = tp.nl;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < tp.N2; n += gridDim.x * blockDim.x) {
        const int nzmax = tp.n_nlev[n], nzmin = tp.n_ulev[n];
        const size_t b = (size_t)n * nl, c = (size_t)n * L1;
        for (int nz = 1; nz <= nl; nz++) K33[b + nz - 1] = Kv[b + nz - 1];
        double zb = g.zbar_n_bot[n];
        double Zc = zb + (double)g.hnode_new[c + nzmax - 2] / 2.0;
        for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
            const double zbn = zb + (double)g.hnode_new[c + nz - 1];
            const double Zu = zbn + (double)g.hnode_new[c + nz - 2] / 2.0;
            const double zinv = 1.0 / (Zu - Zc);
            const double sa = slope[3 * (c + nz - 2) + 2], sb = slope[3 * (c + nz - 1) + 2];
            const double Ty = (zbn - Zc) * zinv * (sa * sa) * (double)Ki[c + nz - 2] +
                              (Zu - zbn) * zinv * (sb * sb) * (double)Ki[c + nz - 1];
            K33[b + nz - 1] = (float)((double)Kv[b + nz - 1] + Ty);
            zb = zbn;
            Zc = Zu;
        }
    }
}

void b32_k33(const DTopo &tp, const DGeom<float> &g, const float *Kv, const float *Ki, const float *slope, float *K33,
             cudaStream_t s) {
    k32_k33<<<(tp.N2 + 127) / 128, 128, 0, s>>>(tp, g, Kv, Ki, slope, K33);
}

void b32_hdiff(const DTopo &tp, const DGeom<float> &g, const B32View &B, cudaStream_t s) {
    if (B.G == 4) k32_hdiff<4><<<grid_nodes(tp.E2), kTB, 0, s>>>(tp, g, B);
    else k32_hdiff<2><<<grid_nodes(tp.E2), kTB, 0, s>>>(tp, g, B);
}
void b32_diff(const DTopo &tp, const DGeom<float> &g, const B32View &B, double dt, cudaStream_t s) {
    if (B.G == 4) {
        k32_diff<4, false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, B, (float)dt);
        if (tp.n_wide) k32_diff<4, true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
    } else {
        k32_diff<2, false><<<grid_nodes(tp.N2), kTB, 0, s>>>(tp, g, B, (float)dt);
        if (tp.n_wide) k32_diff<2, true><<<grid_nodes(tp.n_wide), kTB, 0, s>>>(tp, g, B, (float)dt);
    }
}
void b32_content(const DTopo &tp, const DGeom<float> &g, const float *T, int ng, int G, double *partials, int nblk,
                 double *out, cudaStream_t s) {
    if (G == 4) k32_content_partial<4><<<nblk, 256, 0, s>>>(tp, g, T, ng, partials);
    else k32_content_partial<2><<<nblk, 256, 0, s>>>(tp, g, T, ng, partials);
    const int nslots = ng * G;
    k32_content_final<<<(nslots + 63) / 64, 64, 0, s>>>(partials, nblk, nslots, out);
}
void b32_put_slot(const double *src, float *grpf, int G, int c, size_t count, cudaStream_t s) {
    k32_put_slot<double><<<grid_flat(count), 256, 0, s>>>(src, grpf, G, c, count);
}
void b32_put_slot_f(const float *src, float *grpf, int G, int c, size_t count, cudaStream_t s) {
    k32_put_slot<float><<<grid_flat(count), 256, 0, s>>>(src, grpf, G, c, count);
}
void b32_get_slot(const float *grpf, int G, int c, size_t count, double *dst, cudaStream_t s) {
    k32_get_slot<double><<<grid_flat(count), 256, 0, s>>>(grpf, G, c, count, dst);
}
void b32_get_slot_f(const float *grpf, int G, int c, size_t count, float *dst, cudaStream_t s) {
    k32_get_slot<float><<<grid_flat(count), 256, 0, s>>>(grpf, G, c, count, dst);
}
void b32_put_slot_pair(const double *src, float *g1, float *g2, int G, int c, size_t count, cudaStream_t s) {
    k32_put_slot_pair<double><<<grid_flat(count), 256, 0, s>>>(src, g1, g2, G, c, count);
}
void b32_put_slot_pair_f(const float *src, float *g1, float *g2, int G, int c, size_t count, cudaStream_t s) {
    k32_put_slot_pair<float><<<grid_flat(count), 256, 0, s>>>(src, g1, g2, G, c, count);
}
void b32_get_slot_pair(const float *g1, const float *g2, int G, int c, size_t count, double *dst, cudaStream_t s) {
    k32_get_slot_pair<double><<<grid_flat(count), 256, 0, s>>>(g1, g2, G, c, count, dst);
}
void b32_get_slot_pair_f(const float *g1, const float *g2, int G, int c, size_t count, float *dst, cudaStream_t s) {
    k32_get_slot_pair<float><<<grid_flat(count), 256, 0, s>>>(g1, g2, G, c, count, dst);
}
template <typename S>
void b32_pack_group(const SlotSrc<S> &src, float *grpf, int G, size_t count, int stride, int off, cudaStream_t s) {
    if (G == 4) k32_pack_group<4, S><<<grid_flat(count), 256, 0, s>>>(src, grpf, count, stride, off);
    else k32_pack_group<2, S><<<grid_flat(count), 256, 0, s>>>(src, grpf, count, stride, off);
}
template <typename S>
void b32_unpack_group(const float *grpf, int G, size_t count, const SlotDst<S> &dst, int stride, int off,
                      cudaStream_t s) {
    if (G == 4) k32_unpack_group<4, S><<<grid_flat(count), 256, 0, s>>>(grpf, count, dst, stride, off);
    else k32_unpack_group<2, S><<<grid_flat(count), 256, 0, s>>>(grpf, count, dst, stride, off);
}
template void b32_pack_group<float>(const SlotSrc<float> &, float *, int, size_t, int, int, cudaStream_t);
template void b32_pack_group<double>(const SlotSrc<double> &, float *, int, size_t, int, int, cudaStream_t);
template void b32_unpack_group<float>(const float *, int, size_t, const SlotDst<float> &, int, int, cudaStream_t);
template void b32_unpack_group<double>(const float *, int, size_t, const SlotDst<double> &, int, int, cudaStream_t);

// multi-instance launch wrappers: ix_* hold the per-instance unit offsets of each stage
void bm32_vflux(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vflux<<<grid_nodes(u), kTB, 0, s>>>(I, ix);
}
void bm32_vfactors(const Inst32 *I, const MultiIdx &ix, cudaStream_t s) {
    const int u = ix.start[ix.n];
    if (u) k32m_vfactors<<<grid_nodes(u), kTB, 0, s>>>(I, ix);
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

}  // namespace fesom
