// fesom_internal.h -- device-side data structures shared by the host library
// and the kernels of the GB300 tracer-transport step.
//
// Layout in HBM: every 3-D field keeps the reference's Fortran layout
// a(level, entity): column-contiguous, stride nl-1 (layer fields) or nl
// (interface fields) per entity; all tracers of a batch share one allocation
// with a fixed per-tracer stride.  Topology is 0-based int32; gather lists are
// CSR arrays in ascending edge (element) order so that every node sum adds its
// terms in the order of the reference's serial edge scatter.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace fesom {

constexpr double kREarth = 6367500.0;  // src/oce_modules.F90:29
constexpr double kABEpsilon = 0.1;     // src/oce_modules.F90:105
constexpr double kFluxEps = 1e-16;     // src/oce_adv_tra_fct.F90:99 (double under -fdefault-real-8)
constexpr double kBigNumber = 1e3;     // src/oce_adv_tra_fct.F90:100

struct DTopo {
    int N2, E2, T2, nl, L1;
    const int *e_n1, *e_n2;   // edges(1:2, e)
    const int *e_t1, *e_t2;   // edge_tri(1:2, e), -1 = none
    const int *e_up, *e_dn;   // edge_up_dn_tri(1:2, e), -1 = none
    const int *e_lo, *e_hi;   // level range [nu12, nl12] of the edge scatters (1-based)
    const int *t_n;           // 3 * T2 element nodes
    const int *t_nlev, *t_ulev;
    const int *n_nlev, *n_ulev, *n_nlevmin, *n_ulevmax, *n_nbl;
    const int *ne_ptr, *ne_idx;    // node -> edge, idx >= 0: node is edges(1,e); ~e: node is edges(2,e)
    const int *nie_ptr, *nie_idx;  // node -> element, ascending element order
    int n_wide;                    // nodes of more than 8 edges (FP32 form: their own launch)
    const int *wide_nodes;
};

template <typename R>
struct DGeom {
    const R *elem_area, *elem_cos, *gs;  // gs: 6 per element
    const R *ecd, *edxy;                 // 4 / 2 per edge
    const R *area, *areasvol;            // nl per node
    const R *hnode, *hnode_new;          // nl-1 per node
    const R *helem;                      // nl-1 per element
    const R *Z3, *zbar3;                 // nl-1 / nl per node
    const R *zbar_n_bot;                 // per node
};

template <typename R>
struct DForcing {
    const R *uv;              // 2*(nl-1) per element
    const R *w, *wi, *we;     // nl per node
    const R *Kv;              // nl per node
    const R *bc;              // ntr per node (may be null)
    int wsplit;               // dynamics%use_wsplit: w = w_e + w_i, w_i advected implicitly
};

// Per-tracer scheme on the device (fesom_tra_cfg without the id).
struct DCfg {
    int hor, ver, lim, ab;
    double ph, pv;
    int ivd, pad;
};

template <typename R>
struct DTracers {
    int ntr;
    size_t sN;    // stride of a layer field per tracer: (nl-1) * N2
    size_t sNI;   // stride of an interface field per tracer: nl * N2
    size_t sE;    // stride of an edge field: (nl-1) * E2
    size_t sT;    // stride of tr_xy: 2 * (nl-1) * T2
    R *T, *Told, *TAB;   // Told holds (ab-1) interleaved previous levels
    R *trxy;
    R *FLO, *ADh;        // low-order / antidiffusive edge fluxes
    R *LO, *ADv;         // low-order solution / antidiffusive vertical flux
    R *bmax, *bmin;      // FCT bound increments, then R+ / R- in place
    R *dttf_h, *dttf_v;  // advective increments (drop-in outputs)
    const DCfg *cfg;
    unsigned *status;
    const R *Ki;         // horizontal diffusivity (nl-1 per node), null: no horizontal diffusion
    R *HD;               // horizontal diffusion flux per edge-layer (diff_part_hor_redi's c)
    R *VX;               // explicit vertical diffusion increment per node-layer
    // Redi = .true.: tapered neutral slopes slope_tapered(3, nl-1, nod2D) (null: Redi off) and
    // the increments of diff_ver_part_redi_expl per node-layer
    const R *slope;
    R *RV;
};

// FP32 batched form (kernels_fp32_batched.cu): one step's view of the tracer state.
//
// Tracer groups: the tracers of the form sit in groups of G (4, or 2 for small tracer
// counts) "slots" of one scheme, side by side in every entry: a field of a group is an
// array of G-float entries in the reference's a(level, entity) order, entry
// (g, entity, level) at ((g * count + entity) * levels + level - 1) * G floats.  A lane's
// 16-byte (8-byte) load of one entry brings the values of all G tracers, so every
// address, predicate and gather serves G tracers.  Slots a group does not fill hold zeros
// and compute zeros.  T / O1 / O2 are the current and previous time levels (rotated
// each step, no copy); the step writes the new values into Tnew (the oldest level).
constexpr int kMaxSlots = 64;   // tracer slots of one launch group (per-slot parameters)
constexpr int kMaxGroups = 32;  // tracer groups of one launch group (G >= 2)
struct B32View {
    int ng, ab, G;          // tracer groups of the launch, Adams-Bashforth order, slots per group
    size_t sN, sNI, sE;     // entries per group: layer (nl-1)*N2, interface nl*N2, edge (nl-1)*E2
    const float *T, *O1, *O2;
    float *Tnew;
    float *LO;              // low-order (upwind) solution
    float *ADv;             // vertical flux high order minus low order (the antidiffusive flux)
    float *ADh;             // the same for edges, in the direction edges(1,e) -> edges(2,e)
    float *Rp, *Rm;         // FCT ratios R+ and R-
    float *Bp, *Bm;         // FCT bounds of the advected value (builds with the clamp only)
    unsigned *status;
    // bit g: group g of the launch uses the FCT limiter / takes the implicit vertical
    // diffusion / gets horizontal or explicit vertical diffusion (k32_diff) / the PPM vertical
    // scheme (k32_vppm) / the implicit diffusion with the w_i terms of the split velocity
    unsigned long long fct, ivd, diff, ppm, wimpl;
    signed char hor[kMaxGroups], ver[kMaxGroups];  // per group, in the kernel parameters
    float ph[kMaxSlots], pv[kMaxSlots];            // per slot (slot = g * G + c)
    const float *Ki;        // horizontal diffusivity, nl-1 per node; null: none
    float *HD;              // horizontal diffusion flux per edge-layer (group layout)
    const float *Kv;        // vertical diffusivity (explicit part), nl per node
    const float *fsurf;     // surface flux per group entry (g, node), G floats each; null: none
    size_t sF;              // entries per group of fsurf (nodes)
    // Redi = .true.: tapered neutral slopes, 3 per node-layer (slope_tapered(3, nl-1, nod2D));
    // null: Redi off
    const float *slope;
};
// Node degree bound of the FP32 form (the node's edge list is staged per warp)
constexpr int kMaxDeg = 16;
// Per-edge MUSCL/MFCT reconstruction data of the FP32 form, precomputed at init:
// un / dn = nodes of the up (of edges(1,e)) and down (of edges(2,e)) triangle, the edge
// node first (un.x = edges(1,e), dn.x = edges(2,e)), with un.w = gzmin | gzmax << 16
// (levels where the triangle gradients apply, 0 if none); wu / wd = weights so that
// sum_k wu_k T(un_k) = edge_dxdy(1)*a*gx + edge_dxdy(2)*r_earth*gy of the triangle
// gradient (oce_adv_tra_hor.F90:446-461), wu.w = a (r_earth * mean elem_cos)
struct MusclW {
    const int4 *un, *dn;
    const float4 *wu, *wd;
    // edge-layers outside their triangles' shared range (and every layer of an edge
    // without an up or down triangle) take the area-weighted node means of the element
    // gradients (oce_muscl_adv.F90:388-405, 441-521): per item (edge e, level nz) the
    // projected mean gradient at edges(1,e) is sum_j w_j (T(node_j) - T(edges(1,e)))
    // over pairs [ptr, ptr + n1), at edges(2,e) over [ptr + n1, next ptr)
    int n_items;
    const int *it_e, *it_nz, *it_ptr, *it_n1;
    const int2 *pairs;  // (node, weight as float bits)
};
// FP32 copies of the FP64 factorisation of each column's vertical-diffusion matrix
struct VFactors {
    float *a, *c, *inv, *cp;
};
// once per process, before the first FP32 step (not inside a stream capture): the shared-memory
// limits of the node kernels that stage their gathers
cudaError_t b32_prepare();
// whether the build clamps advected values into their stored FCT bounds (FESOM_FCT_CLAMP); the
// bound arrays exist only then
bool b32_fct_clamp();
void b32_vflux(const DTopo &, const DGeom<float> &, const DForcing<float> &, float *VF, cudaStream_t);
void b32_vfactors(const DTopo &, const DGeom<float> &, const DForcing<float> &, double dt, const VFactors &,
                  cudaStream_t);
// launch shape of the node/edge stages (the autotuner's choices): blocks of 8 warps, at most
// `blocks_per_sm` x 152 blocks (grid-stride loops over the units; 0: one warp per unit), and
// for lo_ad, bounds and update the kernel variant
struct LaunchShape {
    int blocks_per_sm = 0;
    bool staged = false;  // node stages: gathers staged in shared memory (cp.async) instead of registers
    bool vsep = false;    // the update stage: the implicit vertical diffusion as its own kernel
};
void b32_lo_ad(const DTopo &, const DGeom<float> &, const DForcing<float> &, const B32View &, const float *VF,
               double dt, const LaunchShape &, cudaStream_t);
void b32_ho(const DTopo &, const DGeom<float> &, const B32View &, const MusclW &, const float *VF,
            const LaunchShape &, cudaStream_t);
void b32_bounds(const DTopo &, const DGeom<float> &, const B32View &, double dt, const LaunchShape &, cudaStream_t);
// vf: the factors of the implicit vertical diffusion, run as each node's epilogue for the groups in
// ivd & ~wimpl (null: the diffusion is left to b32_vdiff)
void b32_update(const DTopo &, const DGeom<float> &, const B32View &, double dt, const LaunchShape &,
                const VFactors *vf, cudaStream_t);
void b32_vdiff(const DTopo &, const DForcing<float> &, const B32View &, const VFactors &, cudaStream_t);
void b32_vppm(const DTopo &, const DGeom<float> &, const DForcing<float> &, const B32View &, double dt, cudaStream_t);
void b32_lo_impl(const DTopo &, const DGeom<float> &, const DForcing<float> &, const B32View &, double dt,
                 double *scratch, cudaStream_t);
void b32_vdiff_w(const DTopo &, const DGeom<float> &, const DForcing<float> &, const B32View &, double dt,
                 double *scratch, cudaStream_t);
void b32_hdiff(const DTopo &, const DGeom<float> &, const B32View &, cudaStream_t);
// Redi: K33 (nl per node) = Kv + Kd s^2 of the implicit solve (FP64 arithmetic, FP32 result)
void b32_k33(const DTopo &, const DGeom<float> &, const float *Kv, const float *Ki, const float *slope, float *K33,
             cudaStream_t);
void b32_diff(const DTopo &, const DGeom<float> &, const B32View &, double dt, cudaStream_t);
// FP64 content sum_nodes sum_levels T hnode_new areasvol of every slot of the ng groups at T
// (out[slot]); partials: nblk * ng * G doubles
void b32_content(const DTopo &, const DGeom<float> &, const float *T, int ng, int G, double *partials, int nblk,
                 double *out, cudaStream_t);
// layout conversions of the FP32 form: one tracer's column-major array (FP64 or FP32, host
// values staged on the device) into / out of slot c of a group field of `count` entries
void b32_put_slot(const double *src, float *grp, int G, int c, size_t count, cudaStream_t);
void b32_put_slot_f(const float *src, float *grp, int G, int c, size_t count, cudaStream_t);
void b32_get_slot(const float *grp, int G, int c, size_t count, double *dst, cudaStream_t);
void b32_get_slot_f(const float *grp, int G, int c, size_t count, float *dst, cudaStream_t);
// the same for AB3's interleaved valuesold(2, level, node): into / out of two group fields
void b32_put_slot_pair(const double *src, float *g1, float *g2, int G, int c, size_t count, cudaStream_t);
void b32_put_slot_pair_f(const float *src, float *g1, float *g2, int G, int c, size_t count, cudaStream_t);
void b32_get_slot_pair(const float *g1, const float *g2, int G, int c, size_t count, double *dst, cudaStream_t);
void b32_get_slot_pair_f(const float *g1, const float *g2, int G, int c, size_t count, float *dst, cudaStream_t);
// a whole group at once: G staged column-major arrays (FP64 or FP32; p[c] of slot c, null:
// zeros) into / out of one group field, full G-float entries; element i of slot c is
// p[c][i * stride + off]
template <typename S>
struct SlotSrc {
    const S *p[4];
};
template <typename S>
struct SlotDst {
    S *p[4];
};
template <typename S>
void b32_pack_group(const SlotSrc<S> &src, float *grp, int G, size_t count, int stride, int off, cudaStream_t);
template <typename S>
void b32_unpack_group(const float *grp, int G, size_t count, const SlotDst<S> &dst, int stride, int off, cudaStream_t);

// Multi-instance batch of the FP32 form: one descriptor per instance (device memory) and,
// per stage, the offsets of each instance's units in the launch
struct Inst32 {
    DTopo tp;
    DGeom<float> g;
    DForcing<float> f;
    B32View B;
    MusclW mw;
    float *VF;
    VFactors vf;
    float dt;
    double dtd;
    double *scratch;  // the instance's column scratch (split vertical velocity)
};
constexpr int kMaxInst = 64;
struct MultiIdx {
    int n;
    int start[kMaxInst + 1];
};
void bm32_vflux(const Inst32 *, const MultiIdx &, cudaStream_t);
void bm32_vfactors(const Inst32 *, const MultiIdx &, cudaStream_t);
void bm32_lo_ad(const Inst32 *, const MultiIdx &nodes, bool wide, bool ws, cudaStream_t);
void bm32_vppm(const Inst32 *, const MultiIdx &nodes, cudaStream_t);
void bm32_lo_impl(const Inst32 *, const MultiIdx &nodes, cudaStream_t);
void bm32_vdiff_w(const Inst32 *, const MultiIdx &nodes, cudaStream_t);
void bm32_ho(const Inst32 *, const MultiIdx &edges, const MultiIdx &items, cudaStream_t);
void bm32_bounds(const Inst32 *, const MultiIdx &, bool wide, cudaStream_t);
void bm32_update(const Inst32 *, const MultiIdx &, bool wide, cudaStream_t);
void bm32_hdiff(const Inst32 *, const MultiIdx &edges, cudaStream_t);
void bm32_diff(const Inst32 *, const MultiIdx &nodes, bool wide, cudaStream_t);

// tail of the tracer loop (kernels_tail.cu): one tracer's decay, relaxation and clamp
struct TailArgs {
    int decay;            // multiply the whole field by decay_f
    double decay_f;
    int relax;            // 0 none, 1 relax_to_clim (r2c, clim), 2 relax_zonal_temp (clim = Tclim, ztem)
    int repeat;           // applications of relax_zonal_temp (once per tracer of the loop)
    const double *r2c, *clim, *ztem;
    double dt, lat0, dy, tau_inv;
    int nbins;
    int clamp;            // 0 none, 1 salinity to [3, 45], 2 age tracer >= 0
};
void launch_tracer_tail(const DTopo &, const double *coord_y, double *v, const TailArgs &, cudaStream_t);

// launch wrappers (kernels_fp64.cu / kernels_fp32.cu)
template <typename R>
struct Launch {
    static void ab(const DTopo &, DTracers<R> &, int ab_order, cudaStream_t);
    static void trxy(const DTopo &, const DGeom<R> &, DTracers<R> &, cudaStream_t);
    // tracer_gradient_z of T into trz (nl per node)
    static void trz(const DTopo &, const DGeom<R> &, const R *T, R *trz, cudaStream_t);
    static void edge_flux(const DTopo &, const DGeom<R> &, const DForcing<R> &, DTracers<R> &, int fct, cudaStream_t);
    static void node_lo(const DTopo &, const DGeom<R> &, const DForcing<R> &, DTracers<R> &, double dt, int fct,
                        cudaStream_t);
    static void bounds(const DTopo &, const DGeom<R> &, DTracers<R> &, cudaStream_t);
    static void rpm(const DTopo &, const DGeom<R> &, DTracers<R> &, double dt, cudaStream_t);
    // mode 0: write dttf_h/dttf_v only; mode 1: del_ttf sum + T* update into T
    static void update(const DTopo &, const DGeom<R> &, DTracers<R> &, double dt, int fct, int mode, cudaStream_t);
    static void vdiff(const DTopo &, const DGeom<R> &, const DForcing<R> &, DTracers<R> &, double dt,
                      double *scratch, cudaStream_t);
    // adv_tra_vert_impl by w_i on the LO values of the FCT tracers (split vertical velocity)
    static void lo_impl(const DTopo &, const DGeom<R> &, const DForcing<R> &, DTracers<R> &, double dt,
                        double *scratch, cudaStream_t);
    static void content(const DTopo &, const DGeom<R> &, const DTracers<R> &, double *partials, int nblk,
                        double *out, cudaStream_t);
    // diff_part_hor_redi: edge fluxes into tr.HD; hdiff_gather adds them to del (ascending edges)
    static void hdiff(const DTopo &, const DGeom<R> &, DTracers<R> &, cudaStream_t);
    static void hdiff_gather(const DTopo &, const DGeom<R> &, DTracers<R> &, double dt, R *del, cudaStream_t);
    // diff_ver_part_expl_ale: increments of the tracers without implicit vertical diffusion (or of
    // every tracer with all != 0) into out (add == 0) or added to out (add != 0)
    static void vexpl(const DTopo &, const DGeom<R> &, const DForcing<R> &, DTracers<R> &, double dt, R *out,
                      int all, int add, cudaStream_t);
    // Redi: diff_ver_part_redi_expl increments of the group (from tr.trxy) into tr.RV (add == 0)
    // or added to it (add != 0)
    static void redi_v(const DTopo &, const DGeom<R> &, DTracers<R> &, double dt, int add, cudaStream_t);
    // Redi: K33 (nl per node) = Kv + Kd s^2 of the implicit solve, tracer-independent
    static void k33(const DTopo &, const DGeom<R> &, const R *Kv, const R *Ki, const R *slope, R *K33, cudaStream_t);
};

}  // namespace fesom
