// capi.cu -- context management and the C ABI (include/fesom_gpu.h).
//
// The context owns every device allocation: topology and geometry copied at
// fesom_gpu_init, forcing buffers, the tracer state and the per-stage work
// arrays (sized once; no allocation per step).  All work goes to one stream.
// The device-resident step is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fesom_gpu.h"
#include "fesom_internal.h"
#include "mesh_prep.h"

using namespace fesom;

struct fesom_gpu_ctx {
    int prec = FESOM_PREC_FP64;
    int max_tr = 1;
    HostTopo ht;
    int N2 = 0, E2 = 0, T2 = 0, nl = 0, L1 = 0, ibase = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<void *> allocs;
    DTopo tp{};
    DGeom<double> g64{};
    DGeom<float> g32{};
    // forcing (context precision)
    void *uv = nullptr, *w = nullptr, *wi = nullptr, *we = nullptr, *Kv = nullptr, *bc = nullptr;
    double *stage = nullptr;   // FP64 staging chunk for conversions
    size_t stage_n = 0;
    // tracer state
    int ntr = 0;
    int group = 0;             // tracers per launch (work arrays are sized for one group)
    int group_cap = 0;         // tracers the work arrays can hold
    int ab_max = 2;
    std::vector<fesom_tra_cfg> cfgs;
    DCfg *d_cfg = nullptr;
    void *T = nullptr, *Told = nullptr;
    void *TAB = nullptr, *trxy = nullptr, *FLO = nullptr, *ADh = nullptr, *LO = nullptr, *ADv = nullptr;
    void *bmax = nullptr, *bmin = nullptr, *dttf_h = nullptr, *dttf_v = nullptr;
    double *scratch = nullptr, *partials = nullptr, *content_out = nullptr;
    int content_blocks = 0;
    unsigned *status = nullptr;
    bool forcing_ready = false;
    bool state_ready = false;
    int wsplit = 0;            // dynamics%use_wsplit (fesom_gpu_set_wsplit)
    // FP32 form: tracers per launch of the node stages (lo_ad, ho, bounds, update), rounded up
    // to whole tracer groups; 0 = the whole launch group in one launch
    // (fesom_gpu_set_stage_tracers)
    int stage_tr[4] = {0, 0, 0, 0};
    // tracer groups of fesom_gpu_step_host_f32, in order (fesom_gpu_set_host_groups);
    // empty: the automatic ramp of host_groups()
    std::vector<int> host_groups;
    cudaGraphExec_t gexec = nullptr;
    double g_dt = 0.0;
    // FP32 batched form: tracers in groups of gw slots of one scheme (B32View), rotating
    // time-level buffers and the work arrays of one launch group
    int gw = 4;                          // slots per tracer group
    int gw_req = 0;                      // width asked for by fesom_gpu_set_tracer_width (0: automatic)
    int ngr = 0;                         // tracer groups
    std::vector<int> slot_g, slot_c;     // tracer t -> its group and slot in the group
    std::vector<int> gfirst;             // a tracer of each group (the group's scheme)
    std::vector<int> slot_tr;            // tracer of each slot (ngr * gw, -1: empty)
    float *Bf[3] = {nullptr, nullptr, nullptr};
    int rot = 0;
    float *VF = nullptr;
    VFactors vfac{};
    float *LO32 = nullptr, *ADv32 = nullptr, *ADh32 = nullptr;
    float *HD32 = nullptr;  // horizontal diffusion flux per edge-layer of a launch group
    float *Rp32 = nullptr, *Rm32 = nullptr, *Bp32 = nullptr, *Bm32 = nullptr;
    float *pack_in = nullptr, *pack_out = nullptr;  // staging of the host-array step (FP32 columns)
    size_t pack_n = 0;                   // floats each staging buffer holds
    // lo_ad, ho, bounds, update (the autotuner's choice); lo_ad stages its gathers in shared
    // memory by default, bounds and update keep them in registers
    LaunchShape shape[4] = {{0, true}, {0, false}, {0, false}, {0, false}};
    MusclW mw{};
    cudaGraphExec_t gexec32[3] = {nullptr, nullptr, nullptr};
    double g32_dt[3] = {0.0, 0.0, 0.0};
    // second stream: the tracer-independent vertical-diffusion factors run beside the
    // advection stages and join before the update
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host-array step with overlapped transfers: copy-in and copy-out streams, an event per
    // tracer group for "resident" and "computed"
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t ev_forcing = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_done;
    // tail of the tracer loop: node y coordinates (relax_zonal_temp) and work arrays
    void *Ki = nullptr;        // horizontal diffusivity (context precision), null: none
    // Redi (fesom_gpu_set_redi): tapered neutral slopes (3 per node-layer) and the K33 of the
    // implicit solve (nl per node), context precision; active while Ki is set too
    void *slope = nullptr, *K33 = nullptr;
    double *redi_tmp = nullptr;   // FP64 scratch of the routine-level Redi entry points
    size_t redi_tmp_n = 0;
    double *coord_y = nullptr;
    double *tail_v = nullptr, *tail_r2c = nullptr, *tail_T = nullptr, *tail_S = nullptr, *tail_z = nullptr;
    int tail_nbins = 0;
};

namespace {

size_t rsize(const fesom_gpu_ctx *c) { return c->prec == FESOM_PREC_FP32 ? sizeof(float) : sizeof(double); }

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                        \
            return FESOM_ERR_CUDA;                                                                \
        }                                                                                         \
    } while (0)

int dalloc(fesom_gpu_ctx *ctx, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
        *p = nullptr;
        return FESOM_ERR_NOMEM;
    }
    ctx->allocs.push_back(*p);
    return FESOM_OK;
}

void dfree(fesom_gpu_ctx *ctx, void *&p) {
    if (!p) return;
    cudaFree(p);
    ctx->allocs.erase(std::remove(ctx->allocs.begin(), ctx->allocs.end(), p), ctx->allocs.end());
    p = nullptr;
}

int upload_int(fesom_gpu_ctx *ctx, const int **dst, const std::vector<int> &v) {
    void *p;
    int rc = dalloc(ctx, &p, v.size() * sizeof(int));
    if (rc) return rc;
    CK(cudaMemcpy(p, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    *dst = (const int *)p;
    return FESOM_OK;
}

__global__ void k_d2f(const double *in, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}
__global__ void k_f2d(const float *in, double *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// host FP64 -> device array of the context precision (chunked through the stage buffer)
int put(fesom_gpu_ctx *ctx, void *dst, const double *src, size_t n) {
    if (!src) return FESOM_OK;
    if (ctx->prec == FESOM_PREC_FP64) {
        CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
        return FESOM_OK;
    }
    for (size_t off = 0; off < n; off += ctx->stage_n) {
        size_t m = std::min(ctx->stage_n, n - off);
        CK(cudaMemcpyAsync(ctx->stage, src + off, m * sizeof(double), cudaMemcpyDefault, ctx->stream));
        k_d2f<<<(int)std::min<size_t>((m + 255) / 256, 152 * 32), 256, 0, ctx->stream>>>(ctx->stage, (float *)dst + off, m);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}

// device array of the context precision -> host FP64
int get(fesom_gpu_ctx *ctx, double *dst, const void *src, size_t n) {
    if (!dst) return FESOM_OK;
    if (ctx->prec == FESOM_PREC_FP64) {
        CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
        return FESOM_OK;
    }
    for (size_t off = 0; off < n; off += ctx->stage_n) {
        size_t m = std::min(ctx->stage_n, n - off);
        k_f2d<<<(int)std::min<size_t>((m + 255) / 256, 152 * 32), 256, 0, ctx->stream>>>((const float *)src + off, ctx->stage, m);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst + off, ctx->stage, m * sizeof(double), cudaMemcpyDefault, ctx->stream));
    }
    return FESOM_OK;
}

static int nblk(size_t m) { return (int)std::min<size_t>((m + 255) / 256, 152 * 32); }

// One tracer's column-major array (host or device; FP64 or FP32) into / out of its slot of a
// group field of the FP32 form, through the stage buffer (chunks of stage_n doubles or
// 2 stage_n floats).  `count` entries; pair: AB3's interleaved valuesold(2, level, node) into
// / out of the group fields g1 (k = 1) and g2 (k = 2).
int put_slot(fesom_gpu_ctx *ctx, float *grpf, int c, const double *src, size_t count) {
    if (!src) return FESOM_OK;
    for (size_t off = 0; off < count; off += ctx->stage_n) {
        const size_t m = std::min(ctx->stage_n, count - off);
        CK(cudaMemcpyAsync(ctx->stage, src + off, m * sizeof(double), cudaMemcpyDefault, ctx->stream));
        b32_put_slot(ctx->stage, grpf + off * ctx->gw, ctx->gw, c, m, ctx->stream);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}
int put_slot_f(fesom_gpu_ctx *ctx, float *grpf, int c, const float *src, size_t count) {
    if (!src) return FESOM_OK;
    float *st = (float *)ctx->stage;
    const size_t ch = 2 * ctx->stage_n;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        CK(cudaMemcpyAsync(st, src + off, m * sizeof(float), cudaMemcpyDefault, ctx->stream));
        b32_put_slot_f(st, grpf + off * ctx->gw, ctx->gw, c, m, ctx->stream);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}
int get_slot(fesom_gpu_ctx *ctx, double *dst, const float *grpf, int c, size_t count) {
    if (!dst) return FESOM_OK;
    for (size_t off = 0; off < count; off += ctx->stage_n) {
        const size_t m = std::min(ctx->stage_n, count - off);
        b32_get_slot(grpf + off * ctx->gw, ctx->gw, c, m, ctx->stage, ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst + off, ctx->stage, m * sizeof(double), cudaMemcpyDefault, ctx->stream));
    }
    return FESOM_OK;
}
int get_slot_f(fesom_gpu_ctx *ctx, float *dst, const float *grpf, int c, size_t count) {
    if (!dst) return FESOM_OK;
    float *st = (float *)ctx->stage;
    const size_t ch = 2 * ctx->stage_n;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        b32_get_slot_f(grpf + off * ctx->gw, ctx->gw, c, m, st, ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst + off, st, m * sizeof(float), cudaMemcpyDefault, ctx->stream));
    }
    return FESOM_OK;
}
int put_slot_pair(fesom_gpu_ctx *ctx, float *g1, float *g2, int c, const double *src, size_t count) {
    if (!src) return FESOM_OK;
    const size_t ch = ctx->stage_n / 2;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        CK(cudaMemcpyAsync(ctx->stage, src + 2 * off, 2 * m * sizeof(double), cudaMemcpyDefault, ctx->stream));
        b32_put_slot_pair(ctx->stage, g1 + off * ctx->gw, g2 + off * ctx->gw, ctx->gw, c, m, ctx->stream);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}
int put_slot_pair_f(fesom_gpu_ctx *ctx, float *g1, float *g2, int c, const float *src, size_t count) {
    if (!src) return FESOM_OK;
    float *st = (float *)ctx->stage;
    const size_t ch = ctx->stage_n;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        CK(cudaMemcpyAsync(st, src + 2 * off, 2 * m * sizeof(float), cudaMemcpyDefault, ctx->stream));
        b32_put_slot_pair_f(st, g1 + off * ctx->gw, g2 + off * ctx->gw, ctx->gw, c, m, ctx->stream);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}
int get_slot_pair(fesom_gpu_ctx *ctx, double *dst, const float *g1, const float *g2, int c, size_t count) {
    if (!dst) return FESOM_OK;
    const size_t ch = ctx->stage_n / 2;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        b32_get_slot_pair(g1 + off * ctx->gw, g2 + off * ctx->gw, ctx->gw, c, m, ctx->stage, ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst + 2 * off, ctx->stage, 2 * m * sizeof(double), cudaMemcpyDefault, ctx->stream));
    }
    return FESOM_OK;
}
int get_slot_pair_f(fesom_gpu_ctx *ctx, float *dst, const float *g1, const float *g2, int c, size_t count) {
    if (!dst) return FESOM_OK;
    float *st = (float *)ctx->stage;
    const size_t ch = ctx->stage_n;
    for (size_t off = 0; off < count; off += ch) {
        const size_t m = std::min(ch, count - off);
        b32_get_slot_pair_f(g1 + off * ctx->gw, g2 + off * ctx->gw, ctx->gw, c, m, st, ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst + 2 * off, st, 2 * m * sizeof(float), cudaMemcpyDefault, ctx->stream));
    }
    return FESOM_OK;
}

// geometry upload in the context precision
template <typename R>
int upload_geom(fesom_gpu_ctx *ctx, const R **dst, const double *src, size_t n) {
    void *p;
    int rc = dalloc(ctx, &p, n * sizeof(R));
    if (rc) return rc;
    rc = put(ctx, p, src, n);
    if (rc) return rc;
    *dst = (const R *)p;
    return FESOM_OK;
}

template <typename R>
int init_geom(fesom_gpu_ctx *ctx, const fesom_mesh_desc *d, DGeom<R> &g) {
    const size_t N2 = ctx->N2, E2 = ctx->E2, T2 = ctx->T2, nl = ctx->nl, L1 = ctx->L1;
    int rc = 0;
    if ((rc = upload_geom<R>(ctx, &g.elem_area, d->elem_area, T2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.elem_cos, d->elem_cos, T2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.gs, d->gradient_sca, 6 * T2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.ecd, d->edge_cross_dxdy, 4 * E2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.edxy, d->edge_dxdy, 2 * E2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.area, d->area, nl * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.areasvol, d->areasvol, nl * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.hnode, d->hnode, L1 * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.hnode_new, d->hnode_new, L1 * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.helem, d->helem, L1 * T2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.Z3, d->Z_3d_n, L1 * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.zbar3, d->zbar_3d_n, nl * N2))) return rc;
    if ((rc = upload_geom<R>(ctx, &g.zbar_n_bot, d->zbar_n_bot, N2))) return rc;
    return FESOM_OK;
}

// Per-edge reconstruction data of the FP32 form (see MusclW): the triangle gradient
// projected on the edge, edge_dxdy(1)*a*gx + edge_dxdy(2)*r_earth*gy, as weights of the
// triangle's three node values (gradient_sca, src/oce_mesh.F90:2644-2666), in FP64.
int init_muscl_weights(fesom_gpu_ctx *ctx, const fesom_mesh_desc *d) {
    const HostTopo &h = ctx->ht;
    const int E2 = ctx->E2;
    for (int n = 0; n < ctx->N2; n++)
        if (h.ne_ptr[n + 1] - h.ne_ptr[n] > kMaxDeg) {
            ctx->err = "the FP32 form handles nodes with at most 16 edges";
            return FESOM_ERR_MESH;
        }
    std::vector<int4> un(E2), dn(E2);
    std::vector<float4> wu(E2), wd(E2);
    std::vector<int> it_e, it_nz, it_ptr(1, 0), it_n1, wn;
    std::vector<double> ww;
    std::vector<int2> pairs;
    int rc;
    for (int e = 0; e < E2; e++) {
        const int n1 = h.e_n1[e], n2 = h.e_n2[e], el1 = h.e_t1[e], el2 = h.e_t2[e];
        double a = kREarth * d->elem_cos[el1];
        if (el2 >= 0) a = 0.5 * (a + kREarth * d->elem_cos[el2]);
        const double ex = d->edge_dxdy[2 * (size_t)e], ey = d->edge_dxdy[2 * (size_t)e + 1];
        const int up = h.e_up[e], dw = h.e_dn[e];
        int gzmin = 1, gzmax = 0;
        if (up >= 0 && dw >= 0) {
            gzmin = std::max(h.n_ulevmax[n1], h.n_ulevmax[n2]);
            gzmax = std::min(h.n_nlevmin[n1], h.n_nlevmin[n2]);
        }
        // the triangle's nodes from the edge node on (prepare_mesh checked that the triangle holds it)
        auto tri = [&](int el, int node, int4 &nn, float4 &ww) {
            if (el < 0) {
                nn = make_int4(node, node, node, 0);
                ww = make_float4(0.f, 0.f, 0.f, (float)a);
                return;
            }
            const double *gs = d->gradient_sca + 6 * (size_t)el;
            const int *tn = &h.t_n[3 * (size_t)el];
            const int p = tn[0] == node ? 0 : (tn[1] == node ? 1 : 2);
            int q[3];
            float w[3];
            for (int k = 0; k < 3; k++) {
                const int r = (p + k) % 3;
                q[k] = tn[r];
                w[k] = (float)(ex * a * gs[r] + ey * kREarth * gs[r + 3]);
            }
            nn = make_int4(q[0], q[1], q[2], 0);
            ww = make_float4(w[0], w[1], w[2], (float)a);
        };
        tri(up, n1, un[e], wu[e]);
        tri(dw, n2, dn[e], wd[e]);
        un[e].w = gzmin | (gzmax << 16);
        // edge-layers outside [gzmin, gzmax): the projected node-mean gradient at each end
        // node as weights of its neighbours' values (difference form: the weights of an
        // element sum to zero, so the end node's own weight drops out)
        for (int nz = h.e_lo[e]; nz <= h.e_hi[e]; nz++) {
            if (nz >= gzmin && nz <= gzmax - 1) continue;
            it_e.push_back(e);
            it_nz.push_back(nz);
            for (int side = 0; side < 2; side++) {
                const int node = side == 0 ? n1 : n2;
                wn.clear();
                ww.clear();
                double tvol = 0.0;
                for (int k = h.nie_ptr[node]; k < h.nie_ptr[node + 1]; k++) {
                    const int el = h.nie_idx[k];
                    if (h.t_nlev[el] - 1 < nz || nz < h.t_ulev[el]) continue;
                    const double ea = d->elem_area[el];
                    const double *gs = d->gradient_sca + 6 * (size_t)el;
                    tvol += ea;
                    for (int q = 0; q < 3; q++) {
                        const int vtx = h.t_n[3 * (size_t)el + q];
                        const double wq = ea * (ex * a * gs[q] + ey * kREarth * gs[q + 3]);
                        size_t j = 0;
                        while (j < wn.size() && wn[j] != vtx) j++;
                        if (j == wn.size()) { wn.push_back(vtx); ww.push_back(0.0); }
                        ww[j] += wq;
                    }
                }
                int cnt = 0;
                for (size_t j = 0; j < wn.size(); j++) {
                    if (wn[j] == node || tvol <= 0.0) continue;
                    const float wf = (float)(ww[j] / tvol);
                    int wb;
                    std::memcpy(&wb, &wf, sizeof(int));
                    pairs.push_back(make_int2(wn[j], wb));
                    cnt++;
                }
                if (side == 0) it_n1.push_back(cnt);
            }
            it_ptr.push_back((int)pairs.size());
        }
    }
    MusclW &mw = ctx->mw;
    mw.n_items = (int)it_e.size();
    if (mw.n_items) {
        const int *q;
        if ((rc = upload_int(ctx, &q, it_e))) return rc;
        mw.it_e = q;
        if ((rc = upload_int(ctx, &q, it_nz))) return rc;
        mw.it_nz = q;
        if ((rc = upload_int(ctx, &q, it_ptr))) return rc;
        mw.it_ptr = q;
        if ((rc = upload_int(ctx, &q, it_n1))) return rc;
        mw.it_n1 = q;
        void *pp;
        if ((rc = dalloc(ctx, &pp, sizeof(int2) * std::max<size_t>(1, pairs.size())))) return rc;
        if (!pairs.empty()) CK(cudaMemcpy(pp, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice));
        mw.pairs = (const int2 *)pp;
    }
    void *p;
    if ((rc = dalloc(ctx, &p, sizeof(int4) * E2))) return rc;
    CK(cudaMemcpy(p, un.data(), sizeof(int4) * E2, cudaMemcpyHostToDevice));
    ctx->mw.un = (const int4 *)p;
    if ((rc = dalloc(ctx, &p, sizeof(int4) * E2))) return rc;
    CK(cudaMemcpy(p, dn.data(), sizeof(int4) * E2, cudaMemcpyHostToDevice));
    ctx->mw.dn = (const int4 *)p;
    if ((rc = dalloc(ctx, &p, sizeof(float4) * E2))) return rc;
    CK(cudaMemcpy(p, wu.data(), sizeof(float4) * E2, cudaMemcpyHostToDevice));
    ctx->mw.wu = (const float4 *)p;
    if ((rc = dalloc(ctx, &p, sizeof(float4) * E2))) return rc;
    CK(cudaMemcpy(p, wd.data(), sizeof(float4) * E2, cudaMemcpyHostToDevice));
    ctx->mw.wd = (const float4 *)p;
    return FESOM_OK;
}

int check_cfg(fesom_gpu_ctx *ctx, const fesom_tra_cfg *c) {
    if (!c) { ctx->err = "null tracer configuration"; return FESOM_ERR_ARG; }
    if (c->adv_hor < 0 || c->adv_hor > 2) { ctx->err = "unknown horizontal advection scheme"; return FESOM_ERR_SCHEME; }
    if (c->adv_ver < 0 || c->adv_ver > 3) { ctx->err = "unknown vertical advection scheme"; return FESOM_ERR_SCHEME; }
    if (c->adv_lim != 0 && c->adv_lim != 1) { ctx->err = "unknown limiter"; return FESOM_ERR_SCHEME; }
    if (c->ab_order != 2 && c->ab_order != 3) {
        ctx->err = "Adams-Bashforth tracer order must be 2 or 3";
        return FESOM_ERR_ARG;
    }
    return FESOM_OK;
}

DCfg to_dcfg(const fesom_tra_cfg &c) {
    DCfg d{};
    d.hor = c.adv_hor;
    d.ver = c.adv_ver;
    d.lim = c.adv_lim;
    d.ab = c.ab_order;
    d.ph = c.adv_ph;
    d.pv = c.adv_pv;
    d.ivd = c.i_vert_diff;
    return d;
}

// Allocate tracer state for ntr tracers (values/valuesold) and work arrays for
// one group of tracers; the group size is the largest that fits in 85% of the
// free device memory (at least 1).
int alloc_state(fesom_gpu_ctx *ctx, int ntr, int ab_max) {
    const size_t rs = rsize(ctx);
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    const size_t sE = (size_t)ctx->L1 * ctx->E2, sT = 2 * (size_t)ctx->L1 * ctx->T2;
    if (ctx->state_ready && ctx->ntr >= ntr && ctx->ab_max >= ab_max) return FESOM_OK;
    void *bufs[] = {ctx->T, ctx->Told, ctx->TAB, ctx->trxy, ctx->FLO, ctx->ADh, ctx->LO, ctx->ADv,
                    ctx->bmax, ctx->bmin, ctx->dttf_h, ctx->dttf_v, ctx->d_cfg, ctx->bc};
    for (void *b : bufs) { void *p = b; dfree(ctx, p); }
    ctx->T = ctx->Told = ctx->TAB = ctx->trxy = ctx->FLO = ctx->ADh = ctx->LO = ctx->ADv = nullptr;
    ctx->bmax = ctx->bmin = ctx->dttf_h = ctx->dttf_v = ctx->bc = nullptr;
    ctx->d_cfg = nullptr;
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    int rc;
    if ((rc = dalloc(ctx, &ctx->T, rs * sN * ntr))) return rc;
    if ((rc = dalloc(ctx, &ctx->Told, rs * sN * ntr * (ab_max - 1)))) return rc;
    CK(cudaMemset(ctx->Told, 0, rs * sN * ntr * (ab_max - 1)));
    if ((rc = dalloc(ctx, &ctx->bc, rs * (size_t)ctx->N2 * ntr))) return rc;
    CK(cudaMemset(ctx->bc, 0, rs * (size_t)ctx->N2 * ntr));
    if ((rc = dalloc(ctx, (void **)&ctx->d_cfg, sizeof(DCfg) * ntr))) return rc;
    const size_t per_tracer = rs * (5 * sN + sNI + sT + 2 * sE);
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    int g = (int)std::min<size_t>((size_t)ntr, std::max<size_t>(1, (size_t)(0.85 * fr) / per_tracer));
    ctx->group = g;
    ctx->group_cap = g;
    if ((rc = dalloc(ctx, &ctx->TAB, rs * sN * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->trxy, rs * sT * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->FLO, rs * sE * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->ADh, rs * sE * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->LO, rs * sN * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->ADv, rs * sNI * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->bmax, rs * sN * g))) return rc;
    if ((rc = dalloc(ctx, &ctx->bmin, rs * sN * g))) return rc;
    // the advective increments are outputs of the single-tracer drop-in only; in a step
    // dttf_v holds the explicit vertical diffusion increments of every tracer of a group
    if ((rc = dalloc(ctx, &ctx->dttf_h, rs * sN))) return rc;
    if ((rc = dalloc(ctx, &ctx->dttf_v, rs * sN * g))) return rc;
    ctx->ntr = ntr;
    ctx->ab_max = ab_max;
    ctx->state_ready = true;
    return FESOM_OK;
}

template <typename R>
DTracers<R> group_view(fesom_gpu_ctx *ctx, int t0, int nt) {
    DTracers<R> v{};
    v.ntr = nt;
    v.sN = (size_t)ctx->L1 * ctx->N2;
    v.sNI = (size_t)ctx->nl * ctx->N2;
    v.sE = (size_t)ctx->L1 * ctx->E2;
    v.sT = 2 * (size_t)ctx->L1 * ctx->T2;
    v.T = (R *)ctx->T + t0 * v.sN;
    v.Told = (R *)ctx->Told + t0 * v.sN * (ctx->ab_max - 1);
    v.TAB = (R *)ctx->TAB;
    v.trxy = (R *)ctx->trxy;
    v.FLO = (R *)ctx->FLO;
    v.ADh = (R *)ctx->ADh;
    v.LO = (R *)ctx->LO;
    v.ADv = (R *)ctx->ADv;
    v.bmax = (R *)ctx->bmax;
    v.bmin = (R *)ctx->bmin;
    v.dttf_h = (R *)ctx->dttf_h;
    v.dttf_v = (R *)ctx->dttf_v;
    v.cfg = ctx->d_cfg + t0;
    v.status = ctx->status;
    // diff_tracers_ale: the edge diffusion fluxes reuse FLO (dead after the LO stage), the
    // explicit vertical increments reuse dttf_v (unused by the step)
    v.Ki = (const R *)ctx->Ki;
    v.HD = ctx->Ki ? (R *)ctx->FLO : nullptr;
    v.VX = (R *)ctx->dttf_v;
    return v;
}

template <typename R>
DForcing<R> forcing_view(fesom_gpu_ctx *ctx, int t0) {
    DForcing<R> f{};
    f.uv = (const R *)ctx->uv;
    f.w = (const R *)ctx->w;
    f.wi = (const R *)ctx->wi;
    f.we = (const R *)ctx->we;
    f.Kv = (const R *)ctx->Kv;
    f.bc = ctx->bc ? (const R *)ctx->bc + (size_t)t0 * ctx->N2 : nullptr;
    f.wsplit = ctx->wsplit;
    return f;
}

template <typename R>
const DGeom<R> &geom(fesom_gpu_ctx *ctx);
template <>
const DGeom<double> &geom<double>(fesom_gpu_ctx *ctx) { return ctx->g64; }

// One tracer step for tracers [0, ntr): per group init_tracers_AB, gradients,
// edge fluxes, LO + vertical fluxes, FCT bounds, R+/R-, limited update with
// T*, implicit vertical diffusion.  Stream-ordered, capturable.
// ---- FP32 batched form ---------------------------------------------------------
// time level k (0 = current values, 1 = previous, 2 = the one before) of the rotation
float *level32(fesom_gpu_ctx *ctx, int k) {
    if (ctx->ab_max == 2) return ctx->Bf[k == 0 ? ctx->rot : ctx->rot ^ 1];
    const int r = ctx->rot;
    return ctx->Bf[k == 0 ? r : (k == 1 ? (r + 2) % 3 : (r + 1) % 3)];
}
void rotate32(fesom_gpu_ctx *ctx) { ctx->rot = ctx->ab_max == 2 ? ctx->rot ^ 1 : (ctx->rot + 1) % 3; }

void free_graphs32(fesom_gpu_ctx *ctx) {
    for (auto &g : ctx->gexec32)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// Tracer groups of the FP32 form: tracers of one scheme (limiter, horizontal and vertical
// scheme, implicit vertical diffusion) share a group of G slots, filled in tracer order.
bool same_scheme(const fesom_tra_cfg &a, const fesom_tra_cfg &b) {
    return a.adv_hor == b.adv_hor && a.adv_ver == b.adv_ver && a.adv_lim == b.adv_lim &&
           a.i_vert_diff == b.i_vert_diff;
}
// groups of width G for the tracer schemes cf; slot (group, place) of each tracer
int place_tracers(const std::vector<fesom_tra_cfg> &cf, int G, std::vector<int> *sg, std::vector<int> *sc,
                  std::vector<int> *first) {
    std::vector<int> fill, gf;
    if (sg) sg->assign(cf.size(), 0);
    if (sc) sc->assign(cf.size(), 0);
    for (size_t t = 0; t < cf.size(); t++) {
        int g = -1;
        for (size_t k = 0; k < gf.size() && g < 0; k++)
            if (fill[k] < G && same_scheme(cf[gf[k]], cf[t])) g = (int)k;
        if (g < 0) {
            g = (int)gf.size();
            gf.push_back((int)t);
            fill.push_back(0);
        }
        if (sg) (*sg)[t] = g;
        if (sc) (*sc)[t] = fill[g];
        fill[g]++;
    }
    if (first) *first = gf;
    return (int)gf.size();
}
// the group width: as asked, else the one with the fewest slots (4 on a tie)
void assign_groups(fesom_gpu_ctx *ctx, const std::vector<fesom_tra_cfg> &cf) {
    int G = ctx->gw_req;
    if (G != 2 && G != 4) G = 2 * place_tracers(cf, 2, nullptr, nullptr, nullptr) < 4 * place_tracers(cf, 4, nullptr, nullptr, nullptr) ? 2 : 4;
    ctx->gw = G;
    ctx->ngr = place_tracers(cf, G, &ctx->slot_g, &ctx->slot_c, &ctx->gfirst);
    ctx->slot_tr.assign((size_t)ctx->ngr * G, -1);
    for (size_t t = 0; t < cf.size(); t++) ctx->slot_tr[(size_t)ctx->slot_g[t] * G + ctx->slot_c[t]] = (int)t;
}

int alloc_state32(fesom_gpu_ctx *ctx, int ab) {
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2, sE = (size_t)ctx->L1 * ctx->E2;
    const int G = ctx->gw, ngr = ctx->ngr;
    void *old[] = {ctx->Bf[0], ctx->Bf[1], ctx->Bf[2], ctx->VF, ctx->vfac.a, ctx->vfac.c, ctx->vfac.inv, ctx->vfac.cp,
                   ctx->LO32, ctx->ADv32, ctx->ADh32, ctx->Rp32, ctx->Rm32, ctx->Bp32, ctx->Bm32, ctx->d_cfg, ctx->bc,
                   ctx->HD32, ctx->partials, ctx->content_out, ctx->pack_in, ctx->pack_out};
    for (void *b : old) { void *p = b; dfree(ctx, p); }
    ctx->Bf[0] = ctx->Bf[1] = ctx->Bf[2] = nullptr;
    ctx->VF = ctx->LO32 = ctx->ADv32 = ctx->ADh32 = ctx->HD32 = nullptr;
    ctx->Rp32 = ctx->Rm32 = ctx->Bp32 = ctx->Bm32 = nullptr;
    ctx->pack_in = ctx->pack_out = nullptr;
    ctx->pack_n = 0;
    ctx->partials = ctx->content_out = nullptr;
    ctx->vfac = VFactors{};
    ctx->d_cfg = nullptr;
    ctx->bc = nullptr;
    free_graphs32(ctx);
    int rc;
    const size_t lev = 4 * sN * G * (size_t)ngr;  // bytes of one time level of every group
    for (int k = 0; k < ab; k++)
        if ((rc = dalloc(ctx, (void **)&ctx->Bf[k], lev))) return rc;
    for (int k = 0; k < ab; k++) CK(cudaMemset(ctx->Bf[k], 0, lev));
    if ((rc = dalloc(ctx, &ctx->bc, 4 * (size_t)ctx->N2 * G * ngr))) return rc;
    CK(cudaMemset(ctx->bc, 0, 4 * (size_t)ctx->N2 * G * ngr));
    if ((rc = dalloc(ctx, (void **)&ctx->d_cfg, sizeof(DCfg) * std::max<size_t>(1, ctx->cfgs.size())))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->partials, sizeof(double) * (size_t)ctx->content_blocks * ngr * G))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->content_out, sizeof(double) * (size_t)ngr * G))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->VF, 4 * sE))) return rc;
    float **fac[] = {&ctx->vfac.a, &ctx->vfac.c, &ctx->vfac.inv, &ctx->vfac.cp};
    for (float **f : fac)
        if ((rc = dalloc(ctx, (void **)f, 4 * sN))) return rc;
    // LO, R+, R-, (the two bounds,) ADv, ADh (+ the horizontal diffusion fluxes) per group
    const bool clamp = b32_fct_clamp();
    const size_t per_group = 4 * (size_t)G * ((clamp ? 5 : 3) * sN + sNI + sE + (ctx->Ki ? sE : 0));
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    // at most kMaxSlots slots and kMaxGroups groups per launch (per-slot kernel parameters)
    const int gmax = std::min(kMaxGroups, kMaxSlots / G);
    const int g = (int)std::min<size_t>(std::min<size_t>((size_t)ngr, (size_t)gmax),
                                        std::max<size_t>(1, (size_t)(0.85 * fr) / per_group));
    ctx->group = ctx->group_cap = g;
    const size_t wg = 4 * (size_t)G * g;
    if ((rc = dalloc(ctx, (void **)&ctx->LO32, wg * sN))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->ADv32, wg * sNI))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->ADh32, wg * sE))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->Rp32, wg * sN))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->Rm32, wg * sN))) return rc;
    if (clamp && (rc = dalloc(ctx, (void **)&ctx->Bp32, wg * sN))) return rc;
    if (clamp && (rc = dalloc(ctx, (void **)&ctx->Bm32, wg * sN))) return rc;
    if (ctx->Ki && (rc = dalloc(ctx, (void **)&ctx->HD32, wg * sE))) return rc;
    // created here, not on first use: a first step may run inside a stream capture
    CK(b32_prepare());
    if (!ctx->side) {
        CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
        CK(cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->ev_forcing, cudaEventDisableTiming));
    }
    ctx->rot = 0;
    ctx->ab_max = ab;
    ctx->state_ready = true;
    return FESOM_OK;
}

// groups [g0, g0 + ng) of the tracer state; the work arrays hold the launch group from 0
B32View view32(fesom_gpu_ctx *ctx, int g0, int ng) {
    const int G = ctx->gw;
    B32View v{};
    v.ng = ng;
    v.ab = ctx->ab_max;
    v.G = G;
    v.sN = (size_t)ctx->L1 * ctx->N2;
    v.sNI = (size_t)ctx->nl * ctx->N2;
    v.sE = (size_t)ctx->L1 * ctx->E2;
    const size_t go = (size_t)g0 * v.sN * G;
    v.T = level32(ctx, 0) + go;
    v.O1 = level32(ctx, 1) + go;
    v.O2 = ctx->ab_max == 3 ? level32(ctx, 2) + go : nullptr;
    v.Tnew = level32(ctx, ctx->ab_max - 1) + go;
    v.LO = ctx->LO32;
    v.ADv = ctx->ADv32;
    v.ADh = ctx->ADh32;
    v.Rp = ctx->Rp32;
    v.Rm = ctx->Rm32;
    v.Bp = ctx->Bp32;
    v.Bm = ctx->Bm32;
    v.status = ctx->status;
    v.fct = v.ivd = v.diff = v.ppm = v.wimpl = 0;
    v.Ki = (const float *)ctx->Ki;
    v.HD = ctx->Ki ? ctx->HD32 : nullptr;
    v.Kv = (const float *)ctx->Kv;
    v.sF = ctx->N2;
    v.fsurf = ctx->bc ? (const float *)ctx->bc + (size_t)g0 * ctx->N2 * G : nullptr;
    for (int g = 0; g < ng; g++) {
        const fesom_tra_cfg &c = ctx->cfgs[ctx->gfirst[g0 + g]];
        if (c.adv_lim == FESOM_ADV_LIM_FCT) v.fct |= 1ull << g;
        if (c.i_vert_diff) v.ivd |= 1ull << g;
        if (ctx->Ki || !c.i_vert_diff) v.diff |= 1ull << g;
        if (c.adv_ver == FESOM_ADV_VER_PPM) v.ppm |= 1ull << g;
        if (ctx->wsplit && c.i_vert_diff && c.adv_lim != FESOM_ADV_LIM_FCT) v.wimpl |= 1ull << g;
        v.hor[g] = (signed char)c.adv_hor;
        v.ver[g] = (signed char)c.adv_ver;
        for (int k = 0; k < G; k++) {
            const int t = ctx->slot_tr[(size_t)(g0 + g) * G + k];
            v.ph[g * G + k] = t >= 0 ? (float)ctx->cfgs[t].adv_ph : 0.f;
            v.pv[g * G + k] = t >= 0 ? (float)ctx->cfgs[t].adv_pv : 0.f;
        }
    }
    return v;
}

// groups [s0, s0 + ns) of a launch group
B32View sub32(const B32View &B, int s0, int ns) {
    B32View v = B;
    const size_t G = B.G;
    v.ng = ns;
    v.T += s0 * B.sN * G;
    v.O1 += s0 * B.sN * G;
    if (v.O2) v.O2 += s0 * B.sN * G;
    v.Tnew += s0 * B.sN * G;
    v.LO += s0 * B.sN * G;
    v.ADv += s0 * B.sNI * G;
    v.ADh += s0 * B.sE * G;
    v.Rp += s0 * B.sN * G;
    v.Rm += s0 * B.sN * G;
    v.Bp += s0 * B.sN * G;
    v.Bm += s0 * B.sN * G;
    v.fct = B.fct >> s0;
    v.ivd = B.ivd >> s0;
    v.diff = B.diff >> s0;
    v.ppm = B.ppm >> s0;
    v.wimpl = B.wimpl >> s0;
    if (v.HD) v.HD += s0 * B.sE * G;
    if (v.fsurf) v.fsurf += s0 * B.sF * G;
    for (int g = 0; g < ns; g++) {
        v.hor[g] = B.hor[s0 + g];
        v.ver[g] = B.ver[s0 + g];
    }
    for (int k = 0; k < ns * B.G; k++) {
        v.ph[k] = B.ph[s0 * B.G + k];
        v.pv[k] = B.pv[s0 * B.G + k];
    }
    return v;
}

// groups per launch of node stage k of a launch group of ng groups (stage_tr in tracers)
inline int stage_group(const fesom_gpu_ctx *ctx, int k, int ng) {
    const int t = ctx->stage_tr[k];
    const int g = t > 0 ? (t + ctx->gw - 1) / ctx->gw : ng;
    return g < ng ? g : ng;
}

struct StageTimer {
    cudaEvent_t ev[2 * FESOM_NUM_STAGES * 64];
    int stage[FESOM_NUM_STAGES * 64];
    int n = 0;
};

bool redi_on(const fesom_gpu_ctx *ctx) { return ctx->slope && ctx->Ki; }

template <typename R>
int enqueue_step(fesom_gpu_ctx *ctx, double dt, StageTimer *tm = nullptr) {
    const DGeom<R> &g = geom<R>(ctx);
#define STAGE(id, call)                                                                  \
    do {                                                                                 \
        if (tm && tm->n < FESOM_NUM_STAGES * 64) {                                       \
            cudaEventRecord(tm->ev[2 * tm->n], ctx->stream);                             \
            call;                                                                        \
            cudaEventRecord(tm->ev[2 * tm->n + 1], ctx->stream);                         \
            tm->stage[tm->n++] = id;                                                     \
        } else {                                                                         \
            call;                                                                        \
        }                                                                                \
    } while (0)
    const bool redi = redi_on(ctx);
    if (redi) {
        bool vd = false;
        for (int t = 0; t < ctx->ntr; t++) vd |= ctx->cfgs[t].i_vert_diff != 0;
        if (vd)
            STAGE(7, Launch<R>::k33(ctx->tp, g, (const R *)ctx->Kv, (const R *)ctx->Ki, (const R *)ctx->slope,
                                    (R *)ctx->K33, ctx->stream));
    }
    for (int t0 = 0; t0 < ctx->ntr; t0 += ctx->group) {
        const int nt = std::min(ctx->group, ctx->ntr - t0);
        DTracers<R> tr = group_view<R>(ctx, t0, nt);
        DForcing<R> f = forcing_view<R>(ctx, t0);
        // Redi: the slopes; the increments of diff_ver_part_redi_expl in TAB (dead after the LO stage)
        tr.slope = redi ? (const R *)ctx->slope : nullptr;
        tr.RV = redi ? (R *)ctx->TAB : nullptr;
        bool any_fct = false, any_ho = false, any_vd = false, any_ex = false;
        int ab = 2;
        for (int t = t0; t < t0 + nt; t++) {
            any_fct |= ctx->cfgs[t].adv_lim == FESOM_ADV_LIM_FCT;
            any_ho |= ctx->cfgs[t].adv_hor != FESOM_ADV_HOR_UPW1;
            any_vd |= ctx->cfgs[t].i_vert_diff != 0;
            any_ex |= ctx->cfgs[t].i_vert_diff == 0;
            ab = std::max(ab, (int)ctx->cfgs[t].ab_order);
        }
        // all tracers of a group share the valuesold depth of the context
        STAGE(0, Launch<R>::ab(ctx->tp, tr, ctx->ab_max, ctx->stream));
        if (any_ho || ctx->Ki) STAGE(1, Launch<R>::trxy(ctx->tp, g, tr, ctx->stream));
        STAGE(2, Launch<R>::edge_flux(ctx->tp, g, f, tr, any_fct, ctx->stream));
        STAGE(3, Launch<R>::node_lo(ctx->tp, g, f, tr, dt, any_fct, ctx->stream));
        // split vertical velocity: w_i advects the LO values implicitly (oce_adv_tra_driver.F90:323-334)
        if (ctx->wsplit && any_fct) STAGE(3, Launch<R>::lo_impl(ctx->tp, g, f, tr, dt, ctx->scratch, ctx->stream));
        // diff_tracers_ale: horizontal diffusion fluxes, explicit vertical increments (both from
        // the values before the update)
        if (ctx->Ki) STAGE(2, Launch<R>::hdiff(ctx->tp, g, tr, ctx->stream));
        if (any_ex) STAGE(7, Launch<R>::vexpl(ctx->tp, g, f, tr, dt, tr.VX, 0, 0, ctx->stream));
        if (redi) STAGE(7, Launch<R>::redi_v(ctx->tp, g, tr, dt, 0, ctx->stream));
        if (any_fct) {
            STAGE(4, Launch<R>::bounds(ctx->tp, g, tr, ctx->stream));
            STAGE(5, Launch<R>::rpm(ctx->tp, g, tr, dt, ctx->stream));
        }
        STAGE(6, Launch<R>::update(ctx->tp, g, tr, dt, any_fct, 1, ctx->stream));
        if (any_vd) {
            // Redi: the implicit solve diffuses with K33 = Kv + Kd s^2
            DForcing<R> fv = f;
            if (redi) fv.Kv = (const R *)ctx->K33;
            STAGE(7, Launch<R>::vdiff(ctx->tp, g, fv, tr, dt, ctx->scratch, ctx->stream));
        }
    }
    CK(cudaGetLastError());
    return FESOM_OK;
}

// the tracer-independent stages of a step: edge volume fluxes, then the vertical-diffusion
// factors (outside profiled steps on the side stream, joined before the first diffusion)
int enqueue_shared32(fesom_gpu_ctx *ctx, double dt, StageTimer *tm, bool &fork) {
    const DGeom<float> &g = ctx->g32;
    DForcing<float> f = forcing_view<float>(ctx, 0);
    bool any_vd = false;
    for (int t = 0; t < ctx->ntr; t++) any_vd |= ctx->cfgs[t].i_vert_diff != 0;
    STAGE(8, b32_vflux(ctx->tp, g, f, ctx->VF, ctx->stream));
    if (redi_on(ctx) && any_vd) {
        // Redi: the factors of the implicit solve use K33 = Kv + Kd s^2
        STAGE(9, b32_k33(ctx->tp, g, (const float *)ctx->Kv, (const float *)ctx->Ki, (const float *)ctx->slope,
                         (float *)ctx->K33, ctx->stream));
        f.Kv = (const float *)ctx->K33;
    }
    fork = any_vd && !tm;
    if (fork) {
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
        b32_vfactors(ctx->tp, g, f, dt, ctx->vfac, ctx->side);
        CK(cudaEventRecord(ctx->ev_join, ctx->side));
    } else if (any_vd) {
        STAGE(9, b32_vfactors(ctx->tp, g, f, dt, ctx->vfac, ctx->stream));
    }
    return FESOM_OK;
}

// the stages of groups [g0, g0 + ng); `joined` records that the stream already waited for
// the factors of the side stream
int enqueue_group32(fesom_gpu_ctx *ctx, double dt, int g0, int ng, StageTimer *tm, bool fork, bool &joined) {
    const DGeom<float> &g = ctx->g32;
    B32View B = view32(ctx, g0, ng);
    DForcing<float> fg = forcing_view<float>(ctx, 0);
    const bool any_fct = B.fct != 0;
    if (redi_on(ctx)) B.slope = (const float *)ctx->slope;
    // the implicit solve with the w_i terms diffuses with K33 under Redi
    DForcing<float> fk = fg;
    if (redi_on(ctx)) fk.Kv = (const float *)ctx->K33;
    {
        const int sg = stage_group(ctx, 0, ng);
        for (int s0 = 0; s0 < ng; s0 += sg)
            STAGE(10, b32_lo_ad(ctx->tp, g, fg, sub32(B, s0, std::min(sg, ng - s0)), ctx->VF, dt, ctx->shape[0],
                                ctx->stream));
    }
    if (B.ppm) STAGE(10, b32_vppm(ctx->tp, g, fg, B, dt, ctx->stream));
    // split vertical velocity: w_i advects the LO values implicitly (oce_adv_tra_driver.F90:323-334)
    if (ctx->wsplit && any_fct) STAGE(10, b32_lo_impl(ctx->tp, g, fg, B, dt, ctx->scratch, ctx->stream));
    {
        const int sg = stage_group(ctx, 1, ng);
        for (int s0 = 0; s0 < ng; s0 += sg)
            STAGE(2, b32_ho(ctx->tp, g, sub32(B, s0, std::min(sg, ng - s0)), ctx->mw, ctx->VF, ctx->shape[1],
                            ctx->stream));
    }
    // diff_tracers_ale from the values before the update; the increment waits in Tnew (the
    // oldest level, read by lo_ad and ho only) for the update to add it after the limiter
    if (B.Ki) STAGE(2, b32_hdiff(ctx->tp, g, B, ctx->stream));
    if (B.diff) STAGE(7, b32_diff(ctx->tp, g, B, dt, ctx->stream));
    if (any_fct) {
        const int bg = stage_group(ctx, 2, ng);
        for (int s0 = 0; s0 < ng; s0 += bg)
            STAGE(4, b32_bounds(ctx->tp, g, sub32(B, s0, std::min(bg, ng - s0)), dt, ctx->shape[2], ctx->stream));
    }
    // the implicit vertical diffusion: the epilogue of each node of the update (default), or its
    // own launch after it
    const bool vd = (B.ivd & ~B.wimpl) != 0, vfuse = vd && !ctx->shape[3].vsep;
    if (vd && fork && !joined) {
        CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
        joined = true;
    }
    {
        const int sg = stage_group(ctx, 3, ng);
        for (int s0 = 0; s0 < ng; s0 += sg)
            STAGE(6, b32_update(ctx->tp, g, sub32(B, s0, std::min(sg, ng - s0)), dt, ctx->shape[3],
                                vfuse ? &ctx->vfac : nullptr, ctx->stream));
    }
    if (vd && !vfuse) STAGE(7, b32_vdiff(ctx->tp, fg, B, ctx->vfac, ctx->stream));
    if (B.wimpl) STAGE(7, b32_vdiff_w(ctx->tp, g, fk, B, dt, ctx->scratch, ctx->stream));
    return FESOM_OK;
}

int enqueue_step32(fesom_gpu_ctx *ctx, double dt, StageTimer *tm = nullptr) {
    bool fork = false, joined = false;
    int rc = enqueue_shared32(ctx, dt, tm, fork);
    if (rc) return rc;
    for (int g0 = 0; g0 < ctx->ngr; g0 += ctx->group)
        if ((rc = enqueue_group32(ctx, dt, g0, std::min(ctx->group, ctx->ngr - g0), tm, fork, joined))) return rc;
    // a side-stream branch must rejoin the stream (a captured graph requires it)
    if (fork && !joined) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    CK(cudaGetLastError());
    return FESOM_OK;
}
#undef STAGE

int launches_per_step(fesom_gpu_ctx *ctx) {
    int n = 0;
    if (ctx->prec == FESOM_PREC_FP32) {
        bool any_vd = false;
        for (int t = 0; t < ctx->ntr; t++) any_vd |= ctx->cfgs[t].i_vert_diff != 0;
        n = 1 + (any_vd ? 1 : 0) + ((any_vd && redi_on(ctx)) ? 1 : 0);
        for (int g0 = 0; g0 < ctx->ngr; g0 += ctx->group) {
            const int ng = std::min(ctx->group, ctx->ngr - g0);
            const B32View B = view32(ctx, g0, ng);
            // lo_ad, update (+ bounds), launched again for the wide nodes; ho (+ its node-mean
            // edge-layers); vdiff
            const int wide = ctx->tp.n_wide ? 2 : 1;
            auto passes = [&](int k) { return (ng + stage_group(ctx, k, ng) - 1) / stage_group(ctx, k, ng); };
            n += wide * (passes(0) + passes(3) + (B.fct ? passes(2) : 0) + (B.diff ? 1 : 0)) +
                 passes(1) * (ctx->mw.n_items ? 2 : 1) + (((B.ivd & ~B.wimpl) && ctx->shape[3].vsep) ? 1 : 0) +
                 (ctx->Ki ? 1 : 0) +
                 (B.ppm ? 1 : 0) + ((ctx->wsplit && B.fct) ? 1 : 0) + (B.wimpl ? 1 : 0);
        }
        return n;
    }
    if (redi_on(ctx)) {
        bool vd = false;
        for (int t = 0; t < ctx->ntr; t++) vd |= ctx->cfgs[t].i_vert_diff != 0;
        n += vd ? 1 : 0;
    }
    for (int t0 = 0; t0 < ctx->ntr; t0 += ctx->group) {
        const int nt = std::min(ctx->group, ctx->ntr - t0);
        bool any_fct = false, any_ho = false, any_vd = false;
        for (int t = t0; t < t0 + nt; t++) {
            any_fct |= ctx->cfgs[t].adv_lim == FESOM_ADV_LIM_FCT;
            any_ho |= ctx->cfgs[t].adv_hor != FESOM_ADV_HOR_UPW1;
            any_vd |= ctx->cfgs[t].i_vert_diff != 0;
        }
        bool any_ex = false;
        for (int t = t0; t < t0 + nt; t++) any_ex |= ctx->cfgs[t].i_vert_diff == 0;
        n += 4 + ((any_ho || ctx->Ki) ? 1 : 0) + (any_fct ? 2 : 0) + (any_vd ? 1 : 0) + (ctx->Ki ? 1 : 0) +
             (any_ex ? 1 : 0) + ((ctx->wsplit && any_fct) ? 1 : 0) + (redi_on(ctx) ? 1 : 0);
    }
    return n;
}

int enqueue_step_any(fesom_gpu_ctx *ctx, double dt) {
    return ctx->prec == FESOM_PREC_FP32 ? enqueue_step32(ctx, dt) : enqueue_step<double>(ctx, dt);
}

int wait_stream(fesom_gpu_ctx *ctx, int timeout_ms) {
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, ctx->stream));
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t q = cudaEventQuery(ev);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) {
            cudaEventDestroy(ev);
            ctx->err = std::string("stream error: ") + cudaGetErrorString(q);
            return FESOM_ERR_CUDA;
        }
        auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms >= 0 && ms > timeout_ms) {
            cudaEventDestroy(ev);
            ctx->err = "device work did not finish within the time limit";
            return FESOM_ERR_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(ms < 10 ? 20 : 500));
    }
    cudaEventDestroy(ev);
    return FESOM_OK;
}

int need_fp64(fesom_gpu_ctx *ctx) {
    if (ctx->prec != FESOM_PREC_FP64) {
        ctx->err = "the per-routine drop-ins run in FESOM_PREC_FP64 contexts";
        return FESOM_ERR_STATE;
    }
    return FESOM_OK;
}

int ensure_one(fesom_gpu_ctx *ctx, const fesom_tra_cfg *cfg) {
    int rc = check_cfg(ctx, cfg);
    if (rc) return rc;
    if (!ctx->state_ready || ctx->ab_max < cfg->ab_order) {
        rc = alloc_state(ctx, std::max(1, ctx->ntr), std::max(ctx->ab_max, (int)cfg->ab_order));
        if (rc) return rc;
        if (ctx->cfgs.size() < (size_t)ctx->ntr) ctx->cfgs.resize(ctx->ntr, *cfg);
    }
    DCfg d = to_dcfg(*cfg);
    CK(cudaMemcpyAsync(ctx->d_cfg, &d, sizeof(DCfg), cudaMemcpyDefault, ctx->stream));
    return FESOM_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
namespace {
// the pipelined host-array step of the FP32 form (defined with the host-array entry points)
template <typename S>
int step_host(fesom_gpu_ctx *ctx, double dt, const S *uv, const S *w, const S *wi, const S *we, const S *Kv,
              const S *bc_surf, const S *const *values_in, const S *const *valuesold_in, S *const *values_out,
              S *const *valuesold_out);
}  // namespace

extern "C" {

int fesom_gpu_abi_version(void) { return FESOM_GPU_ABI_VERSION; }

int fesom_gpu_host_alloc(size_t bytes, void **ptr) {
    if (!ptr || bytes == 0) return FESOM_ERR_ARG;
    *ptr = nullptr;
    if (cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) != cudaSuccess) {
        *ptr = nullptr;
        return FESOM_ERR_NOMEM;
    }
    return FESOM_OK;
}

int fesom_gpu_host_free(void *ptr) {
    if (!ptr) return FESOM_OK;
    return cudaFreeHost(ptr) == cudaSuccess ? FESOM_OK : FESOM_ERR_CUDA;
}

const char *fesom_gpu_last_error(const fesom_gpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fesom_gpu_init(const fesom_mesh_desc *mesh, int32_t precision, int32_t max_tracers, fesom_gpu_ctx **out) {
    if (!mesh || !out) return FESOM_ERR_ARG;
    *out = nullptr;
    if (precision != FESOM_PREC_FP64 && precision != FESOM_PREC_FP32) return FESOM_ERR_ARG;
    fesom_gpu_ctx *ctx = new fesom_gpu_ctx();
    ctx->prec = precision;
    ctx->max_tr = std::max(1, (int)max_tracers);
    std::string perr;
    if (!prepare_mesh(*mesh, ctx->ht, perr)) {
        ctx->err = perr;
        *out = ctx;  // the caller can read the message, then finalize
        return FESOM_ERR_MESH;
    }
    if (precision == FESOM_PREC_FP32 && mesh->nl - 1 > 128) {
        ctx->err = "the FP32 form handles columns of up to 128 layers";
        *out = ctx;
        return FESOM_ERR_MESH;
    }
    // the FP32 kernels index a tracer's columns and edge layers with 32-bit offsets
    if (precision == FESOM_PREC_FP32 &&
        std::max((size_t)mesh->nl * (size_t)mesh->nod2D, (size_t)mesh->nl * (size_t)mesh->edge2D) >= ((size_t)1 << 31)) {
        ctx->err = "the FP32 form handles meshes with nl * max(nod2D, edge2D) below 2^31";
        *out = ctx;
        return FESOM_ERR_MESH;
    }
    ctx->N2 = mesh->nod2D;
    ctx->E2 = mesh->edge2D;
    ctx->T2 = mesh->elem2D;
    ctx->nl = mesh->nl;
    ctx->L1 = mesh->nl - 1;
    ctx->ibase = mesh->index_base;
    *out = ctx;
    int rc;
    const HostTopo &h = ctx->ht;
    DTopo &tp = ctx->tp;
    tp.N2 = ctx->N2; tp.E2 = ctx->E2; tp.T2 = ctx->T2; tp.nl = ctx->nl; tp.L1 = ctx->L1;
    if ((rc = upload_int(ctx, &tp.e_n1, h.e_n1)) || (rc = upload_int(ctx, &tp.e_n2, h.e_n2)) ||
        (rc = upload_int(ctx, &tp.e_t1, h.e_t1)) || (rc = upload_int(ctx, &tp.e_t2, h.e_t2)) ||
        (rc = upload_int(ctx, &tp.e_up, h.e_up)) || (rc = upload_int(ctx, &tp.e_dn, h.e_dn)) ||
        (rc = upload_int(ctx, &tp.e_lo, h.e_lo)) || (rc = upload_int(ctx, &tp.e_hi, h.e_hi)) ||
        (rc = upload_int(ctx, &tp.t_n, h.t_n)) || (rc = upload_int(ctx, &tp.t_nlev, h.t_nlev)) ||
        (rc = upload_int(ctx, &tp.t_ulev, h.t_ulev)) || (rc = upload_int(ctx, &tp.n_nlev, h.n_nlev)) ||
        (rc = upload_int(ctx, &tp.n_ulev, h.n_ulev)) || (rc = upload_int(ctx, &tp.n_nlevmin, h.n_nlevmin)) ||
        (rc = upload_int(ctx, &tp.n_ulevmax, h.n_ulevmax)) || (rc = upload_int(ctx, &tp.n_nbl, h.n_nbl)) ||
        (rc = upload_int(ctx, &tp.ne_ptr, h.ne_ptr)) || (rc = upload_int(ctx, &tp.ne_idx, h.ne_idx)) ||
        (rc = upload_int(ctx, &tp.nie_ptr, h.nie_ptr)) || (rc = upload_int(ctx, &tp.nie_idx, h.nie_idx)))
        return rc;
    // nodes of more than 8 edges: the FP32 node kernels give them a launch of their own
    {
        std::vector<int> wide;
        for (int n = 0; n < ctx->N2; n++)
            if (h.ne_ptr[n + 1] - h.ne_ptr[n] > 8) wide.push_back(n);
        tp.n_wide = (int)wide.size();
        tp.wide_nodes = nullptr;
        if (!wide.empty() && (rc = upload_int(ctx, &tp.wide_nodes, wide))) return rc;
    }
    ctx->stage_n = std::min<size_t>((size_t)16 << 20, std::max<size_t>(2 * (size_t)ctx->L1 * ctx->T2, (size_t)ctx->nl * ctx->N2));
    if ((rc = dalloc(ctx, (void **)&ctx->stage, ctx->stage_n * sizeof(double)))) return rc;
    if (precision == FESOM_PREC_FP32) rc = init_geom<float>(ctx, mesh, ctx->g32);
    else rc = init_geom<double>(ctx, mesh, ctx->g64);
    if (rc) return rc;
    if (precision == FESOM_PREC_FP32 && (rc = init_muscl_weights(ctx, mesh))) return rc;
    {
        std::vector<double> y(ctx->N2);
        for (int n = 0; n < ctx->N2; n++) y[n] = mesh->coord_nod2D[2 * (size_t)n + 1];
        if ((rc = dalloc(ctx, (void **)&ctx->coord_y, sizeof(double) * ctx->N2))) return rc;
        CK(cudaMemcpy(ctx->coord_y, y.data(), sizeof(double) * ctx->N2, cudaMemcpyHostToDevice));
    }
    const size_t rs = rsize(ctx);
    if ((rc = dalloc(ctx, &ctx->uv, rs * 2 * (size_t)ctx->L1 * ctx->T2))) return rc;
    if ((rc = dalloc(ctx, &ctx->w, rs * (size_t)ctx->nl * ctx->N2))) return rc;
    if ((rc = dalloc(ctx, &ctx->wi, rs * (size_t)ctx->nl * ctx->N2))) return rc;
    if ((rc = dalloc(ctx, &ctx->we, rs * (size_t)ctx->nl * ctx->N2))) return rc;
    if ((rc = dalloc(ctx, &ctx->Kv, rs * (size_t)ctx->nl * ctx->N2))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->scratch, sizeof(double) * 3 * (size_t)(ctx->L1 + 1) * ctx->N2))) return rc;
    ctx->content_blocks = 152 * 4;
    if ((rc = dalloc(ctx, (void **)&ctx->partials, sizeof(double) * (size_t)ctx->content_blocks * ctx->max_tr))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->content_out, sizeof(double) * ctx->max_tr))) return rc;
    if ((rc = dalloc(ctx, (void **)&ctx->status, sizeof(unsigned)))) return rc;
    CK(cudaMemset(ctx->status, 0, sizeof(unsigned)));
    CK(cudaDeviceSynchronize());
    return FESOM_OK;
}

int fesom_gpu_mesh_check(const fesom_mesh_desc *mesh, int32_t *nbl, int32_t *updn, char *errbuf, int32_t errlen) {
    if (!mesh) return FESOM_ERR_ARG;
    HostTopo h;
    std::string perr;
    if (!prepare_mesh(*mesh, h, perr)) {
        if (errbuf && errlen > 0) {
            std::strncpy(errbuf, perr.c_str(), (size_t)errlen - 1);
            errbuf[errlen - 1] = 0;
        }
        return FESOM_ERR_MESH;
    }
    const int b = mesh->index_base;
    if (nbl) std::memcpy(nbl, h.n_nbl.data(), sizeof(int) * h.N2);
    if (updn)
        for (int e = 0; e < h.E2; e++) {
            updn[2 * e] = h.e_up[e] < 0 ? b - 1 : h.e_up[e] + b;
            updn[2 * e + 1] = h.e_dn[e] < 0 ? b - 1 : h.e_dn[e] + b;
        }
    return FESOM_OK;
}

int fesom_gpu_finalize(fesom_gpu_ctx *ctx) {
    if (!ctx) return FESOM_OK;
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    free_graphs32(ctx);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->ev_forcing) cudaEventDestroy(ctx->ev_forcing);
    for (cudaEvent_t e : ctx->ev_in) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ev_done) cudaEventDestroy(e);
    if (ctx->h2d) cudaStreamDestroy(ctx->h2d);
    if (ctx->d2h) cudaStreamDestroy(ctx->d2h);
    for (void *p : ctx->allocs) cudaFree(p);
    delete ctx;
    return FESOM_OK;
}

int fesom_gpu_set_stream(fesom_gpu_ctx *ctx, void *stream) {
    if (!ctx) return FESOM_ERR_ARG;
    ctx->stream = (cudaStream_t)stream;
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    free_graphs32(ctx);
    return FESOM_OK;
}

int fesom_gpu_get_muscl_init(fesom_gpu_ctx *ctx, int32_t *nbl, int32_t *updn) {
    if (!ctx) return FESOM_ERR_ARG;
    if (nbl) std::memcpy(nbl, ctx->ht.n_nbl.data(), sizeof(int) * ctx->N2);
    if (updn)
        for (int e = 0; e < ctx->E2; e++) {
            updn[2 * e] = ctx->ht.e_up[e] < 0 ? ctx->ibase - 1 : ctx->ht.e_up[e] + ctx->ibase;
            updn[2 * e + 1] = ctx->ht.e_dn[e] < 0 ? ctx->ibase - 1 : ctx->ht.e_dn[e] + ctx->ibase;
        }
    return FESOM_OK;
}

int fesom_gpu_status(fesom_gpu_ctx *ctx, uint32_t *status, int32_t timeout_ms) {
    if (!ctx || !status) return FESOM_ERR_ARG;
    int rc = wait_stream(ctx, timeout_ms);
    if (rc) return rc;
    unsigned s = 0;
    CK(cudaMemcpy(&s, ctx->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
    CK(cudaMemset(ctx->status, 0, sizeof(unsigned)));
    *status = s;
    return FESOM_OK;
}

int fesom_gpu_update_thickness(fesom_gpu_ctx *ctx, const double *hnode, const double *hnode_new, const double *helem,
                               const double *Z_3d_n, const double *zbar_3d_n) {
    if (!ctx) return FESOM_ERR_ARG;
    const size_t N2 = ctx->N2, T2 = ctx->T2, L1 = ctx->L1, nl = ctx->nl;
    int rc;
    if (ctx->prec == FESOM_PREC_FP32) {
        DGeom<float> &g = ctx->g32;
        if ((rc = put(ctx, (void *)g.hnode, hnode, L1 * N2)) || (rc = put(ctx, (void *)g.hnode_new, hnode_new, L1 * N2)) ||
            (rc = put(ctx, (void *)g.helem, helem, L1 * T2)) || (rc = put(ctx, (void *)g.Z3, Z_3d_n, L1 * N2)) ||
            (rc = put(ctx, (void *)g.zbar3, zbar_3d_n, nl * N2)))
            return rc;
    } else {
        DGeom<double> &g = ctx->g64;
        if ((rc = put(ctx, (void *)g.hnode, hnode, L1 * N2)) || (rc = put(ctx, (void *)g.hnode_new, hnode_new, L1 * N2)) ||
            (rc = put(ctx, (void *)g.helem, helem, L1 * T2)) || (rc = put(ctx, (void *)g.Z3, Z_3d_n, L1 * N2)) ||
            (rc = put(ctx, (void *)g.zbar3, zbar_3d_n, nl * N2)))
            return rc;
    }
    return wait_stream(ctx, -1);
}

// ---- per-routine drop-ins ----------------------------------------------------
int fesom_gpu_init_tracers_ab(fesom_gpu_ctx *ctx, const fesom_tra_cfg *cfg, const double *values, double *valuesAB,
                              double *valuesold) {
    if (!ctx || !values || !valuesAB || !valuesold) return FESOM_ERR_ARG;
    int rc;
    if ((rc = need_fp64(ctx)) || (rc = ensure_one(ctx, cfg))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    const int ab = cfg->ab_order;
    if ((rc = put(ctx, ctx->T, values, sN))) return rc;
    if (ab == ctx->ab_max) {
        if ((rc = put(ctx, ctx->Told, valuesold, sN * (ab - 1)))) return rc;
    } else {
        ctx->err = "valuesold depth differs from the context's Adams-Bashforth order";
        return FESOM_ERR_STATE;
    }
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    Launch<double>::ab(ctx->tp, tr, ab, ctx->stream);
    Launch<double>::trxy(ctx->tp, ctx->g64, tr, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, valuesAB, ctx->TAB, sN))) return rc;
    if ((rc = get(ctx, valuesold, ctx->Told, sN * (ab - 1)))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_tracer_gradient_z(fesom_gpu_ctx *ctx, const double *values, double *tr_z) {
    if (!ctx || !values || !tr_z) return FESOM_ERR_ARG;
    int rc;
    if ((rc = need_fp64(ctx))) return rc;
    if (!ctx->state_ready) {  // the work arrays of one tracer
        fesom_tra_cfg c{};
        c.ab_order = 2;
        if ((rc = ensure_one(ctx, &c))) return rc;
    }
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    // tr_z travels both ways: the interfaces outside a column keep the caller's values
    if ((rc = put(ctx, ctx->T, values, sN)) || (rc = put(ctx, ctx->ADv, tr_z, sNI))) return rc;
    Launch<double>::trz(ctx->tp, ctx->g64, (const double *)ctx->T, (double *)ctx->ADv, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, tr_z, ctx->ADv, sNI))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_adv_tra(fesom_gpu_ctx *ctx, double dt, const double *vel, const double *w, const double *wi,
                      const double *we, const fesom_tra_cfg *cfg, const double *ttf, const double *ttfAB,
                      double *dttf_h, double *dttf_v) {
    if (!ctx || !vel || !w || !we || !ttf || !ttfAB || !dttf_h || !dttf_v) return FESOM_ERR_ARG;
    if (ctx->wsplit && !wi) {
        ctx->err = "the split vertical velocity needs w_i";
        return FESOM_ERR_ARG;
    }
    int rc;
    if ((rc = need_fp64(ctx)) || (rc = ensure_one(ctx, cfg))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    if ((rc = put(ctx, ctx->uv, vel, 2 * (size_t)ctx->L1 * ctx->T2))) return rc;
    if ((rc = put(ctx, ctx->w, w, sNI))) return rc;
    if ((rc = put(ctx, ctx->wi, wi, sNI))) return rc;
    if ((rc = put(ctx, ctx->we, we, sNI))) return rc;
    if ((rc = put(ctx, ctx->T, ttf, sN))) return rc;
    if ((rc = put(ctx, ctx->TAB, ttfAB, sN))) return rc;
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    DForcing<double> f = forcing_view<double>(ctx, 0);
    const int fct = cfg->adv_lim == FESOM_ADV_LIM_FCT;
    if (cfg->adv_hor != FESOM_ADV_HOR_UPW1) Launch<double>::trxy(ctx->tp, ctx->g64, tr, ctx->stream);
    Launch<double>::edge_flux(ctx->tp, ctx->g64, f, tr, fct, ctx->stream);
    Launch<double>::node_lo(ctx->tp, ctx->g64, f, tr, dt, fct, ctx->stream);
    if (fct && ctx->wsplit) Launch<double>::lo_impl(ctx->tp, ctx->g64, f, tr, dt, ctx->scratch, ctx->stream);
    if (fct) {
        Launch<double>::bounds(ctx->tp, ctx->g64, tr, ctx->stream);
        Launch<double>::rpm(ctx->tp, ctx->g64, tr, dt, ctx->stream);
    }
    Launch<double>::update(ctx->tp, ctx->g64, tr, dt, fct, 0, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, dttf_h, ctx->dttf_h, sN))) return rc;
    if ((rc = get(ctx, dttf_v, ctx->dttf_v, sN))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_vdiff_impl(fesom_gpu_ctx *ctx, double dt, const fesom_tra_cfg *cfg, const double *Kv,
                         const double *bc_surf, double *values) {
    return fesom_gpu_vdiff_impl_wi(ctx, dt, cfg, Kv, bc_surf, nullptr, values);
}

int fesom_gpu_vdiff_impl_wi(fesom_gpu_ctx *ctx, double dt, const fesom_tra_cfg *cfg, const double *Kv,
                            const double *bc_surf, const double *wi, double *values) {
    if (!ctx || !Kv || !values) return FESOM_ERR_ARG;
    int rc;
    if ((rc = need_fp64(ctx)) || (rc = ensure_one(ctx, cfg))) return rc;
    if (wi && (rc = put(ctx, ctx->wi, wi, (size_t)ctx->nl * ctx->N2))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    if ((rc = put(ctx, ctx->Kv, Kv, sNI))) return rc;
    if (bc_surf) {
        if ((rc = put(ctx, ctx->bc, bc_surf, ctx->N2))) return rc;
    } else {
        CK(cudaMemsetAsync(ctx->bc, 0, sizeof(double) * ctx->N2, ctx->stream));
    }
    if ((rc = put(ctx, ctx->T, values, sN))) return rc;
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    DForcing<double> f = forcing_view<double>(ctx, 0);
    f.wsplit = wi != nullptr;  // do_wimpl: w_i given and no limiter (the kernel checks the limiter)
    fesom_tra_cfg c = *cfg;
    c.i_vert_diff = 1;
    DCfg d = to_dcfg(c);
    CK(cudaMemcpyAsync(ctx->d_cfg, &d, sizeof(DCfg), cudaMemcpyDefault, ctx->stream));
    Launch<double>::vdiff(ctx->tp, ctx->g64, f, tr, dt, ctx->scratch, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, values, ctx->T, sN))) return rc;
    return wait_stream(ctx, -1);
}

// ---- device-resident stepping ---------------------------------------------------
int fesom_gpu_state_setup(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs) {
    if (!ctx || ntr < 1 || !cfgs) return FESOM_ERR_ARG;
    if (ntr > ctx->max_tr) { ctx->err = "ntr exceeds max_tracers given to fesom_gpu_init"; return FESOM_ERR_ARG; }
    int ab_max = 2, rc;
    for (int t = 0; t < ntr; t++) {
        if ((rc = check_cfg(ctx, &cfgs[t]))) return rc;
        ab_max = std::max(ab_max, (int)cfgs[t].ab_order);
    }
    for (int t = 0; t < ntr; t++)
        if (cfgs[t].ab_order != ab_max) {
            ctx->err = "all tracers of a batch must use the same Adams-Bashforth order";
            return FESOM_ERR_ARG;
        }
    if (ctx->prec == FESOM_PREC_FP32) {
        // the tracer groups follow the schemes: a new set of schemes may place tracers anew
        std::vector<fesom_tra_cfg> cf(cfgs, cfgs + ntr);
        const std::vector<int> keep_g = ctx->slot_g, keep_c = ctx->slot_c;
        const int keep_w = ctx->gw, keep_n = ctx->ngr;
        assign_groups(ctx, cf);
        const bool same = ctx->state_ready && ctx->ntr == ntr && ctx->ab_max == ab_max && keep_g == ctx->slot_g &&
                          keep_c == ctx->slot_c && keep_w == ctx->gw && keep_n == ctx->ngr;
        ctx->cfgs = cf;
        if (!same) {
            ctx->host_groups.clear();
            if ((rc = alloc_state32(ctx, ab_max))) return rc;
        }
        free_graphs32(ctx);
    } else if ((rc = alloc_state(ctx, ntr, ab_max))) {
        return rc;
    }
    if (ctx->ntr != ntr) ctx->host_groups.clear();
    ctx->ntr = ntr;
    ctx->cfgs.assign(cfgs, cfgs + ntr);
    std::vector<DCfg> d(ntr);
    for (int t = 0; t < ntr; t++) d[t] = to_dcfg(cfgs[t]);
    CK(cudaMemcpy(ctx->d_cfg, d.data(), sizeof(DCfg) * ntr, cudaMemcpyHostToDevice));
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    return FESOM_OK;
}

int fesom_gpu_forcing_upload(fesom_gpu_ctx *ctx, const double *uv, const double *w, const double *wi,
                             const double *we, const double *Kv, const double *bc_surf) {
    if (!ctx || !uv || !w || !we || !Kv) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    const size_t sNI = (size_t)ctx->nl * ctx->N2;
    int rc;
    if ((rc = put(ctx, ctx->uv, uv, 2 * (size_t)ctx->L1 * ctx->T2)) || (rc = put(ctx, ctx->w, w, sNI)) ||
        (rc = put(ctx, ctx->we, we, sNI)) || (rc = put(ctx, ctx->Kv, Kv, sNI)))
        return rc;
    if (wi && (rc = put(ctx, ctx->wi, wi, sNI))) return rc;
    if (ctx->prec == FESOM_PREC_FP32) {
        // the surface flux of tracer t goes to its slot of the group layout
        CK(cudaMemsetAsync(ctx->bc, 0, 4 * (size_t)ctx->N2 * ctx->gw * ctx->ngr, ctx->stream));
        for (int t = 0; bc_surf && t < ctx->ntr; t++)
            if ((rc = put_slot(ctx, (float *)ctx->bc + (size_t)ctx->slot_g[t] * ctx->N2 * ctx->gw, ctx->slot_c[t],
                               bc_surf + (size_t)t * ctx->N2, ctx->N2)))
                return rc;
    } else if (bc_surf) {
        if ((rc = put(ctx, ctx->bc, bc_surf, (size_t)ctx->N2 * ctx->ntr))) return rc;
    } else {
        CK(cudaMemsetAsync(ctx->bc, 0, rsize(ctx) * (size_t)ctx->N2 * ctx->ntr, ctx->stream));
    }
    ctx->forcing_ready = true;
    return FESOM_OK;
}

int fesom_gpu_forcing_upload_f32(fesom_gpu_ctx *ctx, const float *uv, const float *w, const float *wi, const float *we,
                                 const float *Kv, const float *bc_surf) {
    if (!ctx || !uv || !w || !we || !Kv) return FESOM_ERR_ARG;
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "FP32 buffers need a FESOM_PREC_FP32 context"; return FESOM_ERR_STATE; }
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    const size_t sNI = (size_t)ctx->nl * ctx->N2;
    CK(cudaMemcpyAsync(ctx->uv, uv, 4 * 2 * (size_t)ctx->L1 * ctx->T2, cudaMemcpyDefault, ctx->stream));
    CK(cudaMemcpyAsync(ctx->w, w, 4 * sNI, cudaMemcpyDefault, ctx->stream));
    CK(cudaMemcpyAsync(ctx->we, we, 4 * sNI, cudaMemcpyDefault, ctx->stream));
    CK(cudaMemcpyAsync(ctx->Kv, Kv, 4 * sNI, cudaMemcpyDefault, ctx->stream));
    if (wi) CK(cudaMemcpyAsync(ctx->wi, wi, 4 * sNI, cudaMemcpyDefault, ctx->stream));
    CK(cudaMemsetAsync(ctx->bc, 0, 4 * (size_t)ctx->N2 * ctx->gw * ctx->ngr, ctx->stream));
    for (int t = 0; bc_surf && t < ctx->ntr; t++) {
        const int rc = put_slot_f(ctx, (float *)ctx->bc + (size_t)ctx->slot_g[t] * ctx->N2 * ctx->gw, ctx->slot_c[t],
                                  bc_surf + (size_t)t * ctx->N2, ctx->N2);
        if (rc) return rc;
    }
    ctx->forcing_ready = true;
    return FESOM_OK;
}

static int tracer_check(fesom_gpu_ctx *ctx, int32_t tr) {
    if (!ctx) return FESOM_ERR_ARG;
    if (!ctx->state_ready || tr < 0 || tr >= ctx->ntr) {
        ctx->err = "tracer index outside the state set up by fesom_gpu_state_setup";
        return FESOM_ERR_STATE;
    }
    return FESOM_OK;
}

int fesom_gpu_tracer_upload(fesom_gpu_ctx *ctx, int32_t tr, const double *values, const double *valuesold) {
    int rc = tracer_check(ctx, tr);
    if (rc) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, rs = rsize(ctx);
    if (ctx->prec == FESOM_PREC_FP32) {
        const size_t go = (size_t)ctx->slot_g[tr] * sN * ctx->gw;
        const int c = ctx->slot_c[tr];
        if ((rc = put_slot(ctx, level32(ctx, 0) + go, c, values, sN))) return rc;
        if (!valuesold) return FESOM_OK;
        if (ctx->ab_max == 2) return put_slot(ctx, level32(ctx, 1) + go, c, valuesold, sN);
        return put_slot_pair(ctx, level32(ctx, 1) + go, level32(ctx, 2) + go, c, valuesold, sN);
    }
    if ((rc = put(ctx, (char *)ctx->T + rs * sN * tr, values, sN))) return rc;
    return put(ctx, (char *)ctx->Told + rs * sN * (ctx->ab_max - 1) * tr, valuesold, sN * (ctx->ab_max - 1));
}

int fesom_gpu_tracer_download(fesom_gpu_ctx *ctx, int32_t tr, double *values, double *valuesold) {
    int rc = tracer_check(ctx, tr);
    if (rc) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, rs = rsize(ctx);
    if (ctx->prec == FESOM_PREC_FP32) {
        const size_t go = (size_t)ctx->slot_g[tr] * sN * ctx->gw;
        const int c = ctx->slot_c[tr];
        if ((rc = get_slot(ctx, values, level32(ctx, 0) + go, c, sN))) return rc;
        if (valuesold) {
            if (ctx->ab_max == 2) rc = get_slot(ctx, valuesold, level32(ctx, 1) + go, c, sN);
            else rc = get_slot_pair(ctx, valuesold, level32(ctx, 1) + go, level32(ctx, 2) + go, c, sN);
            if (rc) return rc;
        }
        return wait_stream(ctx, -1);
    }
    if ((rc = get(ctx, values, (char *)ctx->T + rs * sN * tr, sN))) return rc;
    if ((rc = get(ctx, valuesold, (char *)ctx->Told + rs * sN * (ctx->ab_max - 1) * tr, sN * (ctx->ab_max - 1))))
        return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_tracer_upload_f32(fesom_gpu_ctx *ctx, int32_t tr, const float *values, const float *valuesold) {
    int rc = tracer_check(ctx, tr);
    if (rc) return rc;
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "FP32 buffers need a FESOM_PREC_FP32 context"; return FESOM_ERR_STATE; }
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    const size_t go = (size_t)ctx->slot_g[tr] * sN * ctx->gw;
    const int c = ctx->slot_c[tr];
    if ((rc = put_slot_f(ctx, level32(ctx, 0) + go, c, values, sN))) return rc;
    if (valuesold) {
        if (ctx->ab_max == 2) return put_slot_f(ctx, level32(ctx, 1) + go, c, valuesold, sN);
        return put_slot_pair_f(ctx, level32(ctx, 1) + go, level32(ctx, 2) + go, c, valuesold, sN);
    }
    return FESOM_OK;
}

int fesom_gpu_tracer_download_f32(fesom_gpu_ctx *ctx, int32_t tr, float *values, float *valuesold) {
    int rc = tracer_check(ctx, tr);
    if (rc) return rc;
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "FP32 buffers need a FESOM_PREC_FP32 context"; return FESOM_ERR_STATE; }
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    const size_t go = (size_t)ctx->slot_g[tr] * sN * ctx->gw;
    const int c = ctx->slot_c[tr];
    if ((rc = get_slot_f(ctx, values, level32(ctx, 0) + go, c, sN))) return rc;
    if (valuesold) {
        if (ctx->ab_max == 2) return get_slot_f(ctx, valuesold, level32(ctx, 1) + go, c, sN);
        return get_slot_pair_f(ctx, valuesold, level32(ctx, 1) + go, level32(ctx, 2) + go, c, sN);
    }
    return FESOM_OK;
}

// capture one step (stream-ordered launches) into an executable graph
static int capture_graph(fesom_gpu_ctx *ctx, double dt, cudaGraphExec_t *out) {
    cudaStream_t cap = ctx->stream;
    bool own = false;
    if (!cap) {  // the legacy stream cannot be captured: capture on a private stream
        CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        own = true;
    }
    cudaStream_t keep = ctx->stream;
    ctx->stream = cap;
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int rc = FESOM_OK;
    if (e == cudaSuccess) {
        rc = enqueue_step_any(ctx, dt);
        e = cudaStreamEndCapture(cap, &graph);
    }
    ctx->stream = keep;
    if (own) cudaStreamDestroy(cap);
    if (rc) return rc;
    if (e != cudaSuccess) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(e); return FESOM_ERR_CUDA; }
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e); return FESOM_ERR_CUDA; }
    return FESOM_OK;
}

int fesom_gpu_run_steps(fesom_gpu_ctx *ctx, double dt, int32_t nsteps, int32_t use_graph) {
    if (!ctx || nsteps < 0) return FESOM_ERR_ARG;
    if (!ctx->state_ready || !ctx->forcing_ready) {
        ctx->err = "state and forcing must be set up before stepping";
        return FESOM_ERR_STATE;
    }
    int rc;
    if (ctx->prec == FESOM_PREC_FP32) {
        for (int s = 0; s < nsteps; s++) {
            if (!use_graph) {
                if ((rc = enqueue_step32(ctx, dt))) return rc;
            } else {
                const int r = ctx->rot;
                if (!ctx->gexec32[r] || ctx->g32_dt[r] != dt) {
                    if (ctx->gexec32[r]) { cudaGraphExecDestroy(ctx->gexec32[r]); ctx->gexec32[r] = nullptr; }
                    if ((rc = capture_graph(ctx, dt, &ctx->gexec32[r]))) return rc;
                    ctx->g32_dt[r] = dt;
                }
                CK(cudaGraphLaunch(ctx->gexec32[r], ctx->stream));
            }
            rotate32(ctx);
        }
        return FESOM_OK;
    }
    if (!use_graph) {
        for (int s = 0; s < nsteps; s++)
            if ((rc = enqueue_step_any(ctx, dt))) return rc;
        return FESOM_OK;
    }
    if (!ctx->gexec || ctx->g_dt != dt) {
        if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
        if ((rc = capture_graph(ctx, dt, &ctx->gexec))) return rc;
        ctx->g_dt = dt;
    }
    for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
    return FESOM_OK;
}

int fesom_gpu_tracer_step(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs, double dt, const double *uv,
                          const double *w, const double *wi, const double *we, const double *Kv, const double *bc_surf,
                          double *const *values, double *const *valuesold) {
    if (!ctx || !values || !valuesold) return FESOM_ERR_ARG;
    int rc;
    bool same = ctx->state_ready && ctx->ntr == ntr && (int)ctx->cfgs.size() == ntr;
    for (int t = 0; same && t < ntr; t++) same = std::memcmp(&ctx->cfgs[t], &cfgs[t], sizeof(fesom_tra_cfg)) == 0;
    if (!same && (rc = fesom_gpu_state_setup(ctx, ntr, cfgs))) return rc;
    if (ctx->prec == FESOM_PREC_FP32) {
        if (!uv || !w || !we || !Kv) return FESOM_ERR_ARG;
        // the FP64 host arrays go through the pipelined host-array step (converted on the device)
        std::vector<const double *> vin(values, values + ntr), oin(valuesold, valuesold + ntr);
        return step_host<double>(ctx, dt, uv, w, wi, we, Kv, bc_surf, vin.data(), oin.data(), values, valuesold);
    }
    if ((rc = fesom_gpu_forcing_upload(ctx, uv, w, wi, we, Kv, bc_surf))) return rc;
    for (int t = 0; t < ntr; t++)
        if ((rc = fesom_gpu_tracer_upload(ctx, t, values[t], valuesold[t]))) return rc;
    if ((rc = fesom_gpu_run_steps(ctx, dt, 1, 0))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, rs = rsize(ctx);
    for (int t = 0; t < ntr; t++) {
        if ((rc = get(ctx, values[t], (char *)ctx->T + rs * sN * t, sN))) return rc;
        if ((rc = get(ctx, valuesold[t], (char *)ctx->Told + rs * sN * (ctx->ab_max - 1) * t, sN * (ctx->ab_max - 1))))
            return rc;
    }
    rc = wait_stream(ctx, -1);
    if (rc) return rc;
    unsigned s = 0;
    CK(cudaMemcpy(&s, ctx->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (s & FESOM_STATUS_NAN) {
        CK(cudaMemset(ctx->status, 0, sizeof(unsigned)));
        ctx->err = "non-finite tracer value produced";
        return FESOM_ERR_NUMERIC;
    }
    return FESOM_OK;
}

int fesom_gpu_set_tracers_per_launch(fesom_gpu_ctx *ctx, int32_t n) {
    if (!ctx || n < 0) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    // the FP32 form launches whole tracer groups: n tracers round up to groups
    const int m = ctx->prec == FESOM_PREC_FP32 ? (n + ctx->gw - 1) / ctx->gw : n;
    ctx->group = m == 0 ? ctx->group_cap : std::min(m, ctx->group_cap);
    ctx->host_groups.clear();
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    free_graphs32(ctx);
    return FESOM_OK;
}

int fesom_gpu_debug_fetch(fesom_gpu_ctx *ctx, const char *name, int32_t tr, double *out, size_t count) {
    if (!ctx || !name || !out) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "no tracer state"; return FESOM_ERR_STATE; }
    if (ctx->prec != FESOM_PREC_FP64) { ctx->err = "work arrays are exposed for FP64 contexts"; return FESOM_ERR_STATE; }
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    const size_t sE = (size_t)ctx->L1 * ctx->E2, sT = 2 * (size_t)ctx->L1 * ctx->T2;
    const std::string n(name);
    const void *src = nullptr;
    size_t len = 0;
    const bool work = !(n == "T" || n == "Told");
    if (work && tr >= ctx->group) { ctx->err = "work arrays hold one launch group"; return FESOM_ERR_ARG; }
    const size_t rs = rsize(ctx);
    if (n == "T") { src = (char *)ctx->T + rs * sN * tr; len = sN; }
    else if (n == "Told") { src = (char *)ctx->Told + rs * sN * (ctx->ab_max - 1) * tr; len = sN * (ctx->ab_max - 1); }
    else if (n == "TAB") { src = (char *)ctx->TAB + rs * sN * tr; len = sN; }
    else if (n == "trxy") { src = (char *)ctx->trxy + rs * sT * tr; len = sT; }
    else if (n == "FLO") { src = (char *)ctx->FLO + rs * sE * tr; len = sE; }
    else if (n == "ADh") { src = (char *)ctx->ADh + rs * sE * tr; len = sE; }
    else if (n == "LO") { src = (char *)ctx->LO + rs * sN * tr; len = sN; }
    else if (n == "ADv") { src = (char *)ctx->ADv + rs * sNI * tr; len = sNI; }
    else if (n == "bmax") { src = (char *)ctx->bmax + rs * sN * tr; len = sN; }
    else if (n == "bmin") { src = (char *)ctx->bmin + rs * sN * tr; len = sN; }
    else if (n == "dttf_h" && tr == 0) { src = ctx->dttf_h; len = sN; }
    else if (n == "dttf_v" && tr == 0) { src = ctx->dttf_v; len = sN; }
    else { ctx->err = "unknown work array " + n; return FESOM_ERR_ARG; }
    if (count < len) { ctx->err = "output buffer too small"; return FESOM_ERR_ARG; }
    int rc = get(ctx, out, src, len);
    if (rc) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_launches_per_step(fesom_gpu_ctx *ctx, int32_t *launches) {
    if (!ctx || !launches) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "no tracer state"; return FESOM_ERR_STATE; }
    *launches = launches_per_step(ctx);
    return FESOM_OK;
}

int fesom_gpu_profile_step(fesom_gpu_ctx *ctx, double dt, float *stage_ms, int32_t *launches) {
    if (!ctx || !stage_ms || !launches) return FESOM_ERR_ARG;
    if (!ctx->state_ready || !ctx->forcing_ready) {
        ctx->err = "state and forcing must be set up before stepping";
        return FESOM_ERR_STATE;
    }
    StageTimer *tm = new StageTimer();
    const int nev = 2 * FESOM_NUM_STAGES * 64;
    for (int i = 0; i < nev; i++) cudaEventCreate(&tm->ev[i]);
    int rc = ctx->prec == FESOM_PREC_FP32 ? enqueue_step32(ctx, dt, tm) : enqueue_step<double>(ctx, dt, tm);
    if (!rc && ctx->prec == FESOM_PREC_FP32) rotate32(ctx);
    if (!rc) rc = wait_stream(ctx, -1);
    for (int i = 0; i < FESOM_NUM_STAGES; i++) { stage_ms[i] = 0.f; launches[i] = 0; }
    if (!rc)
        for (int k = 0; k < tm->n; k++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, tm->ev[2 * k], tm->ev[2 * k + 1]);
            stage_ms[tm->stage[k]] += ms;
            launches[tm->stage[k]] += 1;
        }
    for (int i = 0; i < nev; i++) cudaEventDestroy(tm->ev[i]);
    delete tm;
    return rc;
}

int fesom_gpu_tracer_content(fesom_gpu_ctx *ctx, double *content) {
    if (!ctx || !content) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "no tracer state"; return FESOM_ERR_STATE; }
    if (ctx->prec == FESOM_PREC_FP32) {
        b32_content(ctx->tp, ctx->g32, level32(ctx, 0), ctx->ngr, ctx->gw, ctx->partials, ctx->content_blocks,
                    ctx->content_out, ctx->stream);
        CK(cudaGetLastError());
        std::vector<double> slots((size_t)ctx->ngr * ctx->gw);
        CK(cudaMemcpyAsync(slots.data(), ctx->content_out, sizeof(double) * slots.size(), cudaMemcpyDefault,
                           ctx->stream));
        int rc = wait_stream(ctx, -1);
        if (rc) return rc;
        for (int t = 0; t < ctx->ntr; t++) content[t] = slots[(size_t)ctx->slot_g[t] * ctx->gw + ctx->slot_c[t]];
        return FESOM_OK;
    } else {
        DTracers<double> tr = group_view<double>(ctx, 0, ctx->ntr);
        Launch<double>::content(ctx->tp, ctx->g64, tr, ctx->partials, ctx->content_blocks, ctx->content_out, ctx->stream);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(content, ctx->content_out, sizeof(double) * ctx->ntr, cudaMemcpyDefault, ctx->stream));
    return wait_stream(ctx, -1);
}

int fesom_gpu_set_launch_shape(fesom_gpu_ctx *ctx, int32_t stage, int32_t blocks_per_sm) {
    if (!ctx || stage < 0 || stage > 3 || blocks_per_sm < 0 || blocks_per_sm > 64) return FESOM_ERR_ARG;
    ctx->shape[stage].blocks_per_sm = blocks_per_sm;
    free_graphs32(ctx);
    return FESOM_OK;
}

int fesom_gpu_set_stage_variant(fesom_gpu_ctx *ctx, int32_t stage, int32_t variant) {
    if (!ctx || stage < 0 || stage > 3 || variant < 0 || variant > (stage == 3 ? 3 : 1)) return FESOM_ERR_ARG;
    ctx->shape[stage].staged = (variant & 1) != 0;
    ctx->shape[stage].vsep = (variant & 2) != 0;
    free_graphs32(ctx);
    return FESOM_OK;
}

int fesom_gpu_set_stage_tracers(fesom_gpu_ctx *ctx, int32_t stage, int32_t tracers) {
    if (!ctx || stage < 0 || stage > 3 || tracers < 0) return FESOM_ERR_ARG;
    ctx->stage_tr[stage] = tracers;
    free_graphs32(ctx);
    return FESOM_OK;
}

// ---- autotuning of the FP32 form's launch settings (results do not change) -----------------
namespace {
struct TuneSetting {
    int stage_tr[4];
    LaunchShape shape[4];
    bool operator==(const TuneSetting &o) const {
        for (int k = 0; k < 4; k++)
            if (stage_tr[k] != o.stage_tr[k] || shape[k].blocks_per_sm != o.shape[k].blocks_per_sm ||
                shape[k].staged != o.shape[k].staged || shape[k].vsep != o.shape[k].vsep)
                return false;
        return true;
    }
};

TuneSetting get_setting(const fesom_gpu_ctx *ctx) {
    TuneSetting t;
    for (int k = 0; k < 4; k++) {
        t.stage_tr[k] = ctx->stage_tr[k];
        t.shape[k] = ctx->shape[k];
    }
    return t;
}

void put_setting(fesom_gpu_ctx *ctx, const TuneSetting &t) {
    for (int k = 0; k < 4; k++) {
        ctx->stage_tr[k] = t.stage_tr[k];
        ctx->shape[k] = t.shape[k];
    }
    free_graphs32(ctx);
}

// one untimed step (cold caches, first launches), then `steps` steps between two events on the
// context's stream, launched directly (no graph: a candidate would otherwise pay the captures)
int time_setting(fesom_gpu_ctx *ctx, double dt, int steps, cudaEvent_t e0, cudaEvent_t e1, float *ms) {
    int rc;
    if ((rc = fesom_gpu_run_steps(ctx, dt, 1, 0))) return rc;
    CK(cudaEventRecord(e0, ctx->stream));
    if ((rc = fesom_gpu_run_steps(ctx, dt, steps, 0))) return rc;
    CK(cudaEventRecord(e1, ctx->stream));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(ms, e0, e1));
    *ms /= (float)steps;
    return FESOM_OK;
}
}  // namespace

int fesom_gpu_autotune(fesom_gpu_ctx *ctx, double dt, int32_t steps, fesom_tune_result *res) {
    if (!ctx || steps < 1 || !res) return FESOM_ERR_ARG;
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "the autotuner tunes the FP32 form"; return FESOM_ERR_STATE; }
    if (!ctx->state_ready || !ctx->forcing_ready) {
        ctx->err = "state and forcing must be set up before tuning";
        return FESOM_ERR_STATE;
    }
    int rc;
    // the time levels and their rotation are put back afterwards: tuning leaves the state as it was
    const int nlev = ctx->ab_max;
    const size_t lev = 4 * (size_t)ctx->L1 * ctx->N2 * ctx->gw * (size_t)ctx->ngr;
    void *backup = nullptr;
    if ((rc = dalloc(ctx, &backup, lev * nlev))) return rc;
    for (int k = 0; k < nlev; k++)
        CK(cudaMemcpyAsync((char *)backup + lev * k, ctx->Bf[k], lev, cudaMemcpyDeviceToDevice, ctx->stream));
    const int rot0 = ctx->rot;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const TuneSetting start = get_setting(ctx);
    TuneSetting def{};
    def.shape[0].staged = true;  // the library defaults: lo_ad staged, the rest in registers
    int ncand = 0;
    float def_ms = 0.f, best_ms = 0.f;
    put_setting(ctx, def);
    rc = time_setting(ctx, dt, steps, e0, e1, &def_ms);
    TuneSetting best = def;
    best_ms = def_ms;
    ncand = 1;
    if (!rc && !(start == def)) {
        float ms = 0.f;
        put_setting(ctx, start);
        if (!(rc = time_setting(ctx, dt, steps, e0, e1, &ms)) && ms < best_ms) { best = start; best_ms = ms; }
        ncand++;
    }
    // coordinate descent over the stages: kernel variant, blocks per SM, tracers per launch; a
    // candidate replaces the best when it is faster by more than 1 % (timing noise)
    const int ntr_slots = ctx->ngr * ctx->gw;
    const int bps[] = {0, 2, 4};
    for (int k = 0; k < 4 && !rc; k++) {
        // the update: also with the vertical diffusion as its own launch
        const int nvar = k == 3 ? 4 : 2;
        const int ntrs = (k >= 2 && ntr_slots > 8) ? 2 : 1;
        for (int v = 0; v < nvar && !rc; v++)
            for (int b : bps)
                for (int q = 0; q < ntrs && !rc; q++) {
                    TuneSetting c = best;
                    c.shape[k].staged = (v & 1) != 0;
                    c.shape[k].vsep = (v & 2) != 0;
                    c.shape[k].blocks_per_sm = b;
                    c.stage_tr[k] = q ? 8 : 0;
                    if (c == best) continue;
                    float ms = 0.f;
                    put_setting(ctx, c);
                    if ((rc = time_setting(ctx, dt, steps, e0, e1, &ms))) break;
                    ncand++;
                    if (ms < 0.99f * best_ms) { best = c; best_ms = ms; }
                }
    }
    put_setting(ctx, rc ? start : best);
    for (int k = 0; k < nlev; k++)
        cudaMemcpyAsync(ctx->Bf[k], (char *)backup + lev * k, lev, cudaMemcpyDeviceToDevice, ctx->stream);
    ctx->rot = rot0;
    cudaStreamSynchronize(ctx->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dfree(ctx, backup);
    if (rc) return rc;
    res->default_ms = def_ms;
    res->tuned_ms = best_ms;
    res->candidates = ncand;
    for (int k = 0; k < 4; k++) {
        res->stage_tracers[k] = best.stage_tr[k];
        res->blocks_per_sm[k] = best.shape[k].blocks_per_sm;
        res->variant[k] = (best.shape[k].staged ? 1 : 0) | (best.shape[k].vsep ? 2 : 0);
    }
    return FESOM_OK;
}

int fesom_gpu_set_wsplit(fesom_gpu_ctx *ctx, int32_t on) {
    if (!ctx) return FESOM_ERR_ARG;
    ctx->wsplit = on ? 1 : 0;
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    free_graphs32(ctx);
    return FESOM_OK;
}

int fesom_gpu_set_hdiff(fesom_gpu_ctx *ctx, const double *Ki) {
    if (!ctx) return FESOM_ERR_ARG;
    if (!Ki) {
        if (ctx->Ki) { void *p = ctx->Ki; dfree(ctx, p); ctx->Ki = nullptr; }
        if (ctx->HD32) { void *p = ctx->HD32; dfree(ctx, p); ctx->HD32 = nullptr; }
    } else {
        int rc;
        const size_t sN = (size_t)ctx->L1 * ctx->N2;
        if (!ctx->Ki && (rc = dalloc(ctx, &ctx->Ki, rsize(ctx) * sN))) return rc;
        if ((rc = put(ctx, ctx->Ki, Ki, sN))) return rc;
        // the FP32 form keeps the edge fluxes of a launch group apart from the advective ones
        if (ctx->prec == FESOM_PREC_FP32 && ctx->state_ready && !ctx->HD32 &&
            (rc = dalloc(ctx, (void **)&ctx->HD32, 4 * (size_t)ctx->L1 * ctx->E2 * ctx->gw * ctx->group_cap)))
            return rc;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    free_graphs32(ctx);
    return FESOM_OK;
}

// FP64 scratch of at least n doubles for the routine-level Redi entry points
int redi_scratch(fesom_gpu_ctx *ctx, size_t n) {
    if (ctx->redi_tmp_n >= n) return FESOM_OK;
    if (ctx->redi_tmp) { void *p = ctx->redi_tmp; dfree(ctx, p); ctx->redi_tmp = nullptr; ctx->redi_tmp_n = 0; }
    int rc = dalloc(ctx, (void **)&ctx->redi_tmp, sizeof(double) * n);
    if (rc) return rc;
    ctx->redi_tmp_n = n;
    return FESOM_OK;
}

int fesom_gpu_set_redi(fesom_gpu_ctx *ctx, const double *slope) {
    if (!ctx) return FESOM_ERR_ARG;
    const bool was = ctx->slope != nullptr;
    if (!slope) {
        if (ctx->slope) { void *p = ctx->slope; dfree(ctx, p); ctx->slope = nullptr; }
        if (ctx->K33) { void *p = ctx->K33; dfree(ctx, p); ctx->K33 = nullptr; }
    } else {
        if (!ctx->Ki) {
            ctx->err = "Redi needs the horizontal diffusivity Ki (fesom_gpu_set_hdiff)";
            return FESOM_ERR_STATE;
        }
        int rc;
        const size_t sN = (size_t)ctx->L1 * ctx->N2;
        if (!ctx->slope && (rc = dalloc(ctx, &ctx->slope, rsize(ctx) * 3 * sN))) return rc;
        if (!ctx->K33 && (rc = dalloc(ctx, &ctx->K33, rsize(ctx) * (size_t)ctx->nl * ctx->N2))) return rc;
        if ((rc = put(ctx, ctx->slope, slope, 3 * sN))) return rc;
        // the caller may reuse its array when the call returns
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (was != (slope != nullptr)) {
        if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
        free_graphs32(ctx);
    }
    return FESOM_OK;
}

int fesom_gpu_diff_hor(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *values, double *del_ttf) {
    return fesom_gpu_diff_hor_redi(ctx, dt, Ki, nullptr, values, del_ttf);
}

int fesom_gpu_diff_hor_redi(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *slope, const double *values,
                            double *del_ttf) {
    if (!ctx || !Ki || !values || !del_ttf) return FESOM_ERR_ARG;
    fesom_tra_cfg cfg{};
    cfg.adv_hor = FESOM_ADV_HOR_MUSCL;
    cfg.ab_order = 2;
    int rc = need_fp64(ctx);
    if (rc || (rc = ensure_one(ctx, &cfg))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    if (!ctx->tail_v && (rc = dalloc(ctx, (void **)&ctx->tail_v, sizeof(double) * sN))) return rc;
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    tr.Ki = ctx->tail_v;
    tr.HD = (double *)ctx->FLO;
    if ((rc = put(ctx, ctx->tail_v, Ki, sN)) || (rc = put(ctx, tr.T, values, sN)) ||
        (rc = put(ctx, tr.dttf_h, del_ttf, sN)))
        return rc;
    if (slope) {
        if ((rc = redi_scratch(ctx, 3 * sN))) return rc;
        if ((rc = put(ctx, ctx->redi_tmp, slope, 3 * sN))) return rc;
        tr.slope = ctx->redi_tmp;
    }
    Launch<double>::trxy(ctx->tp, ctx->g64, tr, ctx->stream);
    Launch<double>::hdiff(ctx->tp, ctx->g64, tr, ctx->stream);
    Launch<double>::hdiff_gather(ctx->tp, ctx->g64, tr, dt, tr.dttf_h, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, del_ttf, tr.dttf_h, sN))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_diff_ver_redi_expl(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *slope,
                                 const double *values, double *del_ttf) {
    if (!ctx || !Ki || !slope || !values || !del_ttf) return FESOM_ERR_ARG;
    fesom_tra_cfg cfg{};
    cfg.adv_hor = FESOM_ADV_HOR_MUSCL;
    cfg.ab_order = 2;
    int rc = need_fp64(ctx);
    if (rc || (rc = ensure_one(ctx, &cfg))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    if ((rc = redi_scratch(ctx, 4 * sN))) return rc;
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    tr.Ki = ctx->redi_tmp + 3 * sN;
    tr.slope = ctx->redi_tmp;
    tr.RV = tr.dttf_h;
    if ((rc = put(ctx, ctx->redi_tmp, slope, 3 * sN)) || (rc = put(ctx, ctx->redi_tmp + 3 * sN, Ki, sN)) ||
        (rc = put(ctx, tr.T, values, sN)) || (rc = put(ctx, tr.dttf_h, del_ttf, sN)))
        return rc;
    Launch<double>::trxy(ctx->tp, ctx->g64, tr, ctx->stream);
    Launch<double>::redi_v(ctx->tp, ctx->g64, tr, dt, 1, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, del_ttf, tr.dttf_h, sN))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_redi_k33(fesom_gpu_ctx *ctx, const double *Kv, const double *Ki, const double *slope, double *K33) {
    if (!ctx || !Kv || !Ki || !slope || !K33) return FESOM_ERR_ARG;
    int rc = need_fp64(ctx);
    if (rc) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    if ((rc = redi_scratch(ctx, 4 * sN + 2 * sNI))) return rc;
    double *d_s = ctx->redi_tmp, *d_ki = d_s + 3 * sN, *d_kv = d_ki + sN, *d_k = d_kv + sNI;
    if ((rc = put(ctx, d_s, slope, 3 * sN)) || (rc = put(ctx, d_ki, Ki, sN)) || (rc = put(ctx, d_kv, Kv, sNI)))
        return rc;
    Launch<double>::k33(ctx->tp, ctx->g64, d_kv, d_ki, d_s, d_k, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, K33, d_k, sNI))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_diff_ver_expl(fesom_gpu_ctx *ctx, double dt, const double *Kv, const double *flux_surf,
                            const double *values, double *del_ttf) {
    if (!ctx || !Kv || !values || !del_ttf) return FESOM_ERR_ARG;
    fesom_tra_cfg cfg{};
    cfg.ab_order = 2;
    int rc = need_fp64(ctx);
    if (rc || (rc = ensure_one(ctx, &cfg))) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    DTracers<double> tr = group_view<double>(ctx, 0, 1);
    if ((rc = put(ctx, ctx->Kv, Kv, (size_t)ctx->nl * ctx->N2)) || (rc = put(ctx, tr.T, values, sN)) ||
        (rc = put(ctx, tr.dttf_h, del_ttf, sN)))
        return rc;
    if (flux_surf) CK(cudaMemcpyAsync(ctx->bc, flux_surf, sizeof(double) * ctx->N2, cudaMemcpyDefault, ctx->stream));
    else CK(cudaMemsetAsync(ctx->bc, 0, sizeof(double) * ctx->N2, ctx->stream));
    DForcing<double> f = forcing_view<double>(ctx, 0);
    Launch<double>::vexpl(ctx->tp, ctx->g64, f, tr, dt, tr.dttf_h, 1, 1, ctx->stream);
    CK(cudaGetLastError());
    if ((rc = get(ctx, del_ttf, tr.dttf_h, sN))) return rc;
    return wait_stream(ctx, -1);
}

int fesom_gpu_tracer_tail(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs, double dt,
                          const fesom_tail_cfg *tc, const double *relax2clim, const double *Tclim, const double *Sclim,
                          const double *ztem, double *const *values) {
    if (!ctx || !cfgs || !tc || !values || ntr < 1) return FESOM_ERR_ARG;
    int rc = need_fp64(ctx);
    if (rc) return rc;
    const bool clim = tc->clim_relax > 1.0e-8 && !tc->zonal_relax;
    if (clim && (!relax2clim || !Tclim || !Sclim)) {
        ctx->err = "relax_to_clim needs relax2clim, Tclim and Sclim";
        return FESOM_ERR_ARG;
    }
    if (tc->zonal_relax && (!Tclim || !ztem || tc->nbins < 1 || !(tc->dy > 0.0))) {
        ctx->err = "relax_zonal_temp needs Tclim, ztem, nbins >= 1 and dy > 0";
        return FESOM_ERR_ARG;
    }
    const size_t sN = (size_t)ctx->L1 * ctx->N2;
    if (!ctx->tail_v) {
        if ((rc = dalloc(ctx, (void **)&ctx->tail_v, sizeof(double) * sN)) ||
            (rc = dalloc(ctx, (void **)&ctx->tail_r2c, sizeof(double) * ctx->N2)) ||
            (rc = dalloc(ctx, (void **)&ctx->tail_T, sizeof(double) * sN)) ||
            (rc = dalloc(ctx, (void **)&ctx->tail_S, sizeof(double) * sN)))
            return rc;
    }
    if (tc->zonal_relax && ctx->tail_nbins < tc->nbins) {
        if (ctx->tail_z) { void *p = ctx->tail_z; dfree(ctx, p); ctx->tail_z = nullptr; }
        if ((rc = dalloc(ctx, (void **)&ctx->tail_z, sizeof(double) * (size_t)tc->nbins * ctx->L1))) return rc;
        ctx->tail_nbins = tc->nbins;
    }
    if (clim) {
        CK(cudaMemcpyAsync(ctx->tail_r2c, relax2clim, sizeof(double) * ctx->N2, cudaMemcpyDefault, ctx->stream));
        CK(cudaMemcpyAsync(ctx->tail_S, Sclim, sizeof(double) * sN, cudaMemcpyDefault, ctx->stream));
    }
    if (clim || tc->zonal_relax) CK(cudaMemcpyAsync(ctx->tail_T, Tclim, sizeof(double) * sN, cudaMemcpyDefault, ctx->stream));
    if (tc->zonal_relax)
        CK(cudaMemcpyAsync(ctx->tail_z, ztem, sizeof(double) * (size_t)tc->nbins * ctx->L1, cudaMemcpyDefault,
                           ctx->stream));
    // decay constants of 14C and 39Ar (src/mod_transit.F90:49-50), factors formed on the host
    const double k14 = 3.8561e-12, k39 = 8.1708e-11;
    for (int t = 0; t < ntr; t++) {
        TailArgs a{};
        a.decay = cfgs[t].id == 14 || cfgs[t].id == 39;
        a.decay_f = a.decay ? std::exp(-(cfgs[t].id == 14 ? k14 : k39) * dt) : 1.0;
        a.dt = dt;
        if (tc->zonal_relax) {
            // relax_zonal_temp of tracer 1 runs at every iteration of the tracer loop
            if (t == 0) {
                a.relax = 2;
                a.repeat = ntr;
                a.clim = ctx->tail_T;
                a.ztem = ctx->tail_z;
                a.lat0 = tc->lat0;
                a.dy = tc->dy;
                a.tau_inv = tc->tau_inv;
                a.nbins = tc->nbins;
            }
        } else if (clim && (cfgs[t].id == 1 || cfgs[t].id == 2)) {
            a.relax = 1;
            a.r2c = ctx->tail_r2c;
            a.clim = cfgs[t].id == 1 ? ctx->tail_T : ctx->tail_S;
        }
        a.clamp = t == tc->salt_index ? 1 : (t == tc->age_index ? 2 : 0);
        if (!a.decay && !a.relax && !a.clamp) continue;
        CK(cudaMemcpyAsync(ctx->tail_v, values[t], sizeof(double) * sN, cudaMemcpyDefault, ctx->stream));
        launch_tracer_tail(ctx->tp, ctx->coord_y, ctx->tail_v, a, ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(values[t], ctx->tail_v, sizeof(double) * sN, cudaMemcpyDefault, ctx->stream));
    }
    return wait_stream(ctx, -1);
}

}  // extern "C"

// Pipeline stages of the host-array step, in tracer groups: the first stage's upload and the
// last stage's download are the parts of the step no compute hides, so both are small;
// between them the stages double up to the launch group.  With L groups per launch the first
// stage holds max(1, L/6) groups and so does the last (24 tracers in 6 groups of 4: stages of
// 1, 2, 2 and 1 groups, 211 ms per step against 218 ms for 2, 2, 2 and 234 ms for six of 1).
static std::vector<int> host_groups(const fesom_gpu_ctx *ctx) {
    if (!ctx->host_groups.empty()) return ctx->host_groups;
    const int L = std::max(1, ctx->group), s0 = std::max(1, L / 6);
    std::vector<int> out;
    for (int rem = ctx->ngr, s = s0; rem > 0; s = std::min(L, 2 * s)) {
        const int x = std::min(std::min(s, rem), L);
        out.push_back(x);
        rem -= x;
    }
    if (out.size() > 1 && out.back() > s0) {
        const int last = out.back();
        out.back() = last - s0;
        out.push_back(s0);
    }
    return out;
}

namespace {

// forcing of the host-array step on the copy-in stream, FP32 or FP64 host arrays
int put_on(fesom_gpu_ctx *ctx, cudaStream_t st, float *dst, const float *src, size_t n) {
    CK(cudaMemcpyAsync(dst, src, 4 * n, cudaMemcpyDefault, st));
    return FESOM_OK;
}
int put_on(fesom_gpu_ctx *ctx, cudaStream_t st, float *dst, const double *src, size_t n) {
    for (size_t off = 0; off < n; off += ctx->stage_n) {
        const size_t m = std::min(ctx->stage_n, n - off);
        CK(cudaMemcpyAsync(ctx->stage, src + off, m * sizeof(double), cudaMemcpyDefault, st));
        k_d2f<<<nblk(m), 256, 0, st>>>(ctx->stage, dst + off, m);
        CK(cudaGetLastError());
    }
    return FESOM_OK;
}

// One FP32 step from and to host arrays of type S (FP32 or FP64), the transfers overlapped
// with the compute: the stages of host_groups() go in on the copy-in stream into a ring of two
// staging buffers, are packed into the group layout and stepped on the context stream as soon
// as they are resident, and are unpacked into a ring of two output buffers and copied out on
// the copy-out stream as soon as they are computed.
template <typename S>
int step_host(fesom_gpu_ctx *ctx, double dt, const S *uv, const S *w, const S *wi, const S *we, const S *Kv,
              const S *bc_surf, const S *const *values_in, const S *const *valuesold_in, S *const *values_out,
              S *const *valuesold_out) {
    int rc;
    const int G = ctx->gw, ab = ctx->ab_max, lv = ab - 1;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, sNI = (size_t)ctx->nl * ctx->N2;
    std::vector<int> gs(1, 0);
    for (int x : host_groups(ctx)) gs.push_back(gs.back() + x);
    if (gs.back() != ctx->ngr || (int)gs.size() < 2) {
        ctx->err = "the host groups must hold every tracer group once";
        return FESOM_ERR_ARG;
    }
    const int ns = (int)gs.size() - 1;
    // staging per slot of the two rings: the largest stage's tracers, values and previous levels
    size_t need = 0;
    for (int k = 0; k < ns; k++) need = std::max(need, (size_t)(gs[k + 1] - gs[k]) * G * (1 + lv) * sN * sizeof(S));
    need = std::max(need, sizeof(S) * (size_t)ctx->N2 * ctx->ntr);  // the surface fluxes pass through slot 0
    if (ctx->pack_n < need) {
        for (float **b : {&ctx->pack_in, &ctx->pack_out}) {
            void *p = *b;
            dfree(ctx, p);
            *b = nullptr;
        }
        ctx->pack_n = 0;
        if ((rc = dalloc(ctx, (void **)&ctx->pack_in, 2 * need)) || (rc = dalloc(ctx, (void **)&ctx->pack_out, 2 * need)))
            return rc;
        ctx->pack_n = need;
    }
    while ((int)ctx->ev_in.size() < 2 * ns) {
        cudaEvent_t a, b;
        CK(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
        ctx->ev_in.push_back(a);
        ctx->ev_done.push_back(b);
    }
    // ev_in[k]: stage k resident in its staging slot; ev_in[ns + k]: stage k packed (its
    // staging slot free); ev_done[k]: stage k computed and unpacked; ev_done[ns + k]: copied out
    cudaEvent_t *ev_res = ctx->ev_in.data(), *ev_pack = ctx->ev_in.data() + ns;
    cudaEvent_t *ev_comp = ctx->ev_done.data(), *ev_out = ctx->ev_done.data() + ns;
    // the previous step's kernels are done with the buffers the copies fill
    CK(cudaEventRecord(ctx->ev_forcing, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->h2d, ctx->ev_forcing, 0));
    if ((rc = put_on(ctx, ctx->h2d, (float *)ctx->uv, uv, 2 * (size_t)ctx->L1 * ctx->T2)) ||
        (rc = put_on(ctx, ctx->h2d, (float *)ctx->w, w, sNI)) || (rc = put_on(ctx, ctx->h2d, (float *)ctx->we, we, sNI)) ||
        (rc = put_on(ctx, ctx->h2d, (float *)ctx->Kv, Kv, sNI)))
        return rc;
    if (wi && (rc = put_on(ctx, ctx->h2d, (float *)ctx->wi, wi, sNI))) return rc;
    CK(cudaMemsetAsync(ctx->bc, 0, 4 * (size_t)ctx->N2 * G * ctx->ngr, ctx->h2d));
    if (bc_surf) {
        // per tracer into its slot, through the first staging slot (free at this point)
        S *st = (S *)ctx->pack_in;
        CK(cudaMemcpyAsync(st, bc_surf, sizeof(S) * (size_t)ctx->N2 * ctx->ntr, cudaMemcpyDefault, ctx->h2d));
        for (int g = 0; g < ctx->ngr; g++) {
            SlotSrc<S> src{};
            for (int c = 0; c < G; c++) {
                const int t = ctx->slot_tr[(size_t)g * G + c];
                src.p[c] = t >= 0 ? st + (size_t)t * ctx->N2 : nullptr;
            }
            b32_pack_group<S>(src, (float *)ctx->bc + (size_t)g * ctx->N2 * G, G, ctx->N2, 1, 0, ctx->h2d);
        }
        CK(cudaGetLastError());
    }
    ctx->forcing_ready = true;
    CK(cudaEventRecord(ctx->ev_forcing, ctx->h2d));
    float *L0 = level32(ctx, 0), *L1b = level32(ctx, 1), *L2b = ab == 3 ? level32(ctx, 2) : nullptr;
    float *Lnew = level32(ctx, ab - 1);
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_forcing, 0));
    bool fork = false, joined = false;
    if ((rc = enqueue_shared32(ctx, dt, nullptr, fork))) return rc;
    const size_t per_tr = (1 + lv) * sN;  // staged elements per tracer: values, then valuesold
    for (int k = 0; k < ns; k++) {
        S *in = (S *)((char *)ctx->pack_in + (k & 1) * need);
        S *out = (S *)((char *)ctx->pack_out + (k & 1) * need);
        // copy in: stage k's tracers, once stage k-2 has left the slot
        if (k >= 2) CK(cudaStreamWaitEvent(ctx->h2d, ev_pack[k - 2], 0));
        int q = 0;
        for (int g = gs[k]; g < gs[k + 1]; g++)
            for (int c = 0; c < G; c++, q++) {
                const int t = ctx->slot_tr[(size_t)g * G + c];
                if (t < 0) continue;
                CK(cudaMemcpyAsync(in + q * per_tr, values_in[t], sizeof(S) * sN, cudaMemcpyDefault, ctx->h2d));
                CK(cudaMemcpyAsync(in + q * per_tr + sN, valuesold_in[t], sizeof(S) * sN * lv, cudaMemcpyDefault,
                                   ctx->h2d));
            }
        CK(cudaEventRecord(ev_res[k], ctx->h2d));
        // compute: pack into the time levels, the stages of the groups, unpack the results
        CK(cudaStreamWaitEvent(ctx->stream, ev_res[k], 0));
        q = 0;
        for (int g = gs[k]; g < gs[k + 1]; g++, q += G) {
            SlotSrc<S> v{}, o{};
            for (int c = 0; c < G; c++) {
                const bool has = ctx->slot_tr[(size_t)g * G + c] >= 0;
                v.p[c] = has ? in + (q + c) * per_tr : nullptr;
                o.p[c] = has ? in + (q + c) * per_tr + sN : nullptr;
            }
            const size_t go = (size_t)g * sN * G;
            b32_pack_group<S>(v, L0 + go, G, sN, 1, 0, ctx->stream);
            b32_pack_group<S>(o, L1b + go, G, sN, lv, 0, ctx->stream);
            if (ab == 3) b32_pack_group<S>(o, L2b + go, G, sN, 2, 1, ctx->stream);
        }
        CK(cudaGetLastError());
        CK(cudaEventRecord(ev_pack[k], ctx->stream));
        for (int g0 = gs[k]; g0 < gs[k + 1]; g0 += ctx->group)
            if ((rc = enqueue_group32(ctx, dt, g0, std::min(ctx->group, gs[k + 1] - g0), nullptr, fork, joined)))
                return rc;
        if (k >= 2) CK(cudaStreamWaitEvent(ctx->stream, ev_out[k - 2], 0));
        q = 0;
        for (int g = gs[k]; g < gs[k + 1]; g++, q += G) {
            SlotDst<S> v{}, o{};
            for (int c = 0; c < G; c++) {
                const bool has = ctx->slot_tr[(size_t)g * G + c] >= 0;
                v.p[c] = has ? out + (q + c) * per_tr : nullptr;
                o.p[c] = (has && valuesold_out) ? out + (q + c) * per_tr + sN : nullptr;
            }
            const size_t go = (size_t)g * sN * G;
            b32_unpack_group<S>(Lnew + go, G, sN, v, 1, 0, ctx->stream);
            if (valuesold_out) {
                // the new previous levels: the values the step started from (and, AB3, the level before)
                b32_unpack_group<S>(L0 + go, G, sN, o, lv, 0, ctx->stream);
                if (ab == 3) b32_unpack_group<S>(L1b + go, G, sN, o, 2, 1, ctx->stream);
            }
        }
        CK(cudaGetLastError());
        CK(cudaEventRecord(ev_comp[k], ctx->stream));
        // copy out
        CK(cudaStreamWaitEvent(ctx->d2h, ev_comp[k], 0));
        q = 0;
        for (int g = gs[k]; g < gs[k + 1]; g++)
            for (int c = 0; c < G; c++, q++) {
                const int t = ctx->slot_tr[(size_t)g * G + c];
                if (t < 0) continue;
                CK(cudaMemcpyAsync(values_out[t], out + q * per_tr, sizeof(S) * sN, cudaMemcpyDefault, ctx->d2h));
                if (valuesold_out)
                    CK(cudaMemcpyAsync(valuesold_out[t], out + q * per_tr + sN, sizeof(S) * sN * lv, cudaMemcpyDefault,
                                       ctx->d2h));
            }
        CK(cudaEventRecord(ev_out[k], ctx->d2h));
    }
    if (fork && !joined) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    rotate32(ctx);
    // the context's stream follows the copies out, so later calls see a quiet context
    CK(cudaEventRecord(ctx->ev_forcing, ctx->d2h));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_forcing, 0));
    if ((rc = wait_stream(ctx, -1))) return rc;
    unsigned st = 0;
    CK(cudaMemcpy(&st, ctx->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (st) {
        CK(cudaMemset(ctx->status, 0, sizeof(unsigned)));
        ctx->err = st & FESOM_STATUS_NAN ? "NaN in the tracer step" : "FCT limiter needed more than round-off clamping";
        return FESOM_ERR_NUMERIC;
    }
    return FESOM_OK;
}

}  // namespace

extern "C" {

int fesom_gpu_set_host_groups(fesom_gpu_ctx *ctx, int32_t n, const int32_t *sizes) {
    if (!ctx || n < 0 || (n > 0 && !sizes)) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "host groups belong to the FP32 form"; return FESOM_ERR_STATE; }
    std::vector<int> gs;
    int sum = 0;
    for (int i = 0; i < n; i++) {
        if (sizes[i] < 1 || sizes[i] > ctx->group) {
            ctx->err = "a host group holds 1 to groups-per-launch tracer groups";
            return FESOM_ERR_ARG;
        }
        gs.push_back(sizes[i]);
        sum += sizes[i];
    }
    if (n > 0 && sum != ctx->ngr) { ctx->err = "the host groups must hold every tracer group once"; return FESOM_ERR_ARG; }
    ctx->host_groups = gs;
    return FESOM_OK;
}

int fesom_gpu_tracer_groups(fesom_gpu_ctx *ctx, int32_t *groups, int32_t *width, int32_t *group_of,
                            int32_t *slot_of) {
    if (!ctx) return FESOM_ERR_ARG;
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "tracer groups belong to the FP32 form"; return FESOM_ERR_STATE; }
    if (groups) *groups = ctx->ngr;
    if (width) *width = ctx->gw;
    for (int t = 0; t < ctx->ntr; t++) {
        if (group_of) group_of[t] = ctx->slot_g[t];
        if (slot_of) slot_of[t] = ctx->slot_c[t];
    }
    return FESOM_OK;
}

int fesom_gpu_set_tracer_width(fesom_gpu_ctx *ctx, int32_t width) {
    if (!ctx || (width != 0 && width != 2 && width != 4)) return FESOM_ERR_ARG;
    ctx->gw_req = width;
    // the next fesom_gpu_state_setup places the tracers with it
    return FESOM_OK;
}

int fesom_gpu_step_host_f32(fesom_gpu_ctx *ctx, double dt, const float *uv, const float *w, const float *wi,
                            const float *we, const float *Kv, const float *bc_surf, const float *const *values_in,
                            const float *const *valuesold_in, float *const *values_out, float *const *valuesold_out) {
    if (!ctx || !uv || !w || !we || !Kv || !values_in || !valuesold_in || !values_out) return FESOM_ERR_ARG;
    if (ctx->prec != FESOM_PREC_FP32) { ctx->err = "FP32 buffers need a FESOM_PREC_FP32 context"; return FESOM_ERR_STATE; }
    if (!ctx->state_ready) { ctx->err = "call fesom_gpu_state_setup first"; return FESOM_ERR_STATE; }
    return step_host<float>(ctx, dt, uv, w, wi, we, Kv, bc_surf, values_in, valuesold_in, values_out, valuesold_out);
}

int fesom_gpu_tracer_device_ptr(fesom_gpu_ctx *ctx, int32_t tr, void **values, void **valuesold) {
    int rc = tracer_check(ctx, tr);
    if (rc) return rc;
    const size_t sN = (size_t)ctx->L1 * ctx->N2, rs = rsize(ctx);
    if (ctx->prec == FESOM_PREC_FP32) {
        ctx->err = "the FP32 form stores tracers in interleaved groups (fesom_gpu_tracer_groups): use the upload and "
                   "download calls";
        return FESOM_ERR_STATE;
    }
    if (values) *values = (char *)ctx->T + rs * sN * tr;
    if (valuesold) *valuesold = (char *)ctx->Told + rs * sN * (ctx->ab_max - 1) * tr;
    return FESOM_OK;
}

// ---------------------------------------------------------------------------
// multi-instance batch of the FP32 form (no counterpart in the reference, which runs
// one mesh per process)
// ---------------------------------------------------------------------------
}  // extern "C"

struct fesom_gpu_batch {
    std::vector<fesom_gpu_ctx *> inst;
    int ab = 2, phase = 0;
    cudaStream_t stream = nullptr;
    Inst32 *d_inst = nullptr;  // ab descriptor sets (one per rotation phase), inst.size() each
    double d_dt = -1.0;
    MultiIdx ix_e{}, ix_n{}, ix_w{}, ix_it{};
    int maxL1 = 0;
    bool any_vd = false, any_fct = false, any_hd = false, any_diff = false;
    bool any_ws = false, any_ppm = false, any_lo_impl = false, any_wimpl = false;
    cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
    double g_dt[3] = {0.0, 0.0, 0.0};
    std::string err;
};

namespace {

#define BCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return FESOM_ERR_CUDA;                                                                \
        }                                                                                         \
    } while (0)

void set_prefix(MultiIdx &ix, const std::vector<int> &count) {
    ix.n = (int)count.size();
    ix.start[0] = 0;
    for (int i = 0; i < ix.n; i++) ix.start[i + 1] = ix.start[i] + count[i];
}

// descriptors of every instance for each rotation phase, for time step dt
int batch_descriptors(fesom_gpu_batch *b, double dt) {
    const int n = (int)b->inst.size();
    std::vector<Inst32> h((size_t)n * b->ab);
    for (int p = 0; p < b->ab; p++)
        for (int i = 0; i < n; i++) {
            fesom_gpu_ctx *c = b->inst[i];
            const int keep = c->rot;
            for (int k = 0; k < p; k++) rotate32(c);
            Inst32 &d = h[(size_t)p * n + i];
            d.tp = c->tp;
            d.g = c->g32;
            d.f = forcing_view<float>(c, 0);
            d.B = view32(c, 0, c->ngr);
            d.mw = c->mw;
            d.VF = c->VF;
            d.vf = c->vfac;
            d.dt = (float)dt;
            d.dtd = dt;
            d.scratch = c->scratch;
            c->rot = keep;
        }
    BCK(cudaMemcpy(b->d_inst, h.data(), sizeof(Inst32) * h.size(), cudaMemcpyHostToDevice));
    b->d_dt = dt;
    return FESOM_OK;
}

void enqueue_batch_step(fesom_gpu_batch *b, cudaStream_t s) {
    const Inst32 *I = b->d_inst + (size_t)b->phase * b->inst.size();
    const bool wide = b->ix_w.start[b->ix_w.n] > 0;
    bm32_vflux(I, b->ix_e, s);
    if (b->any_vd) bm32_vfactors(I, b->ix_n, s);
    bm32_lo_ad(I, b->ix_n, false, b->any_ws, s);
    if (wide) bm32_lo_ad(I, b->ix_w, true, b->any_ws, s);
    if (b->any_ppm) bm32_vppm(I, b->ix_n, s);
    if (b->any_lo_impl) bm32_lo_impl(I, b->ix_n, s);
    bm32_ho(I, b->ix_e, b->ix_it, s);
    if (b->any_hd) bm32_hdiff(I, b->ix_e, s);
    if (b->any_diff) {
        bm32_diff(I, b->ix_n, false, s);
        if (wide) bm32_diff(I, b->ix_w, true, s);
    }
    if (b->any_fct) {
        bm32_bounds(I, b->ix_n, false, s);
        if (wide) bm32_bounds(I, b->ix_w, true, s);
    }
    // (the implicit vertical diffusion runs inside the update, per node)
    bm32_update(I, b->ix_n, false, s);
    if (wide) bm32_update(I, b->ix_w, true, s);
    if (b->any_wimpl) bm32_vdiff_w(I, b->ix_n, s);
}

}  // namespace

extern "C" {

int fesom_gpu_batch_create(fesom_gpu_ctx *const *ctxs, int32_t n, fesom_gpu_batch **out) {
    if (!out) return FESOM_ERR_ARG;
    *out = nullptr;
    fesom_gpu_batch *b = new fesom_gpu_batch();
    *out = b;
    if (!ctxs || n < 1 || n > kMaxInst) {
        b->err = "a batch holds 1 to 64 FP32 contexts";
        return FESOM_ERR_ARG;
    }
    std::vector<int> ce, cn, cw, cit;
    for (int i = 0; i < n; i++) {
        fesom_gpu_ctx *c = ctxs[i];
        if (!c || c->prec != FESOM_PREC_FP32) { b->err = "batch instances must be FP32 contexts"; return FESOM_ERR_ARG; }
        if (!c->state_ready || !c->forcing_ready) {
            b->err = "every batch instance needs its tracer state and forcing set up";
            return FESOM_ERR_STATE;
        }
        if (c->group != c->ngr) {
            b->err = "every batch instance must hold all its tracers in one launch group";
            return FESOM_ERR_STATE;
        }
        if (i > 0 && c->ab_max != b->ab) { b->err = "batch instances must share one Adams-Bashforth order"; return FESOM_ERR_ARG; }
        if (redi_on(c)) { b->err = "batch instances cannot use Redi (step Redi contexts on their own)"; return FESOM_ERR_STATE; }
        bool fct = false;
        for (int t = 0; t < c->ntr; t++) {
            b->any_ppm |= c->cfgs[t].adv_ver == FESOM_ADV_VER_PPM;
            b->any_wimpl |= c->wsplit && c->cfgs[t].i_vert_diff && c->cfgs[t].adv_lim != FESOM_ADV_LIM_FCT;
            fct |= c->cfgs[t].adv_lim == FESOM_ADV_LIM_FCT;
        }
        b->any_ws |= c->wsplit != 0;
        b->any_lo_impl |= c->wsplit && fct;
        b->ab = c->ab_max;
        for (int t = 0; t < c->ntr; t++) {
            b->any_vd |= c->cfgs[t].i_vert_diff != 0;
            b->any_fct |= c->cfgs[t].adv_lim == FESOM_ADV_LIM_FCT;
            b->any_diff |= c->cfgs[t].i_vert_diff == 0;
        }
        b->any_hd |= c->Ki != nullptr;
        b->any_diff |= c->Ki != nullptr;
        b->maxL1 = std::max(b->maxL1, c->L1);
        b->inst.push_back(c);
        ce.push_back(c->E2);
        cn.push_back(c->N2);
        cw.push_back(c->tp.n_wide);
        cit.push_back(c->mw.n_items);
    }
    set_prefix(b->ix_e, ce);
    set_prefix(b->ix_n, cn);
    set_prefix(b->ix_w, cw);
    set_prefix(b->ix_it, cit);
    BCK(cudaMalloc((void **)&b->d_inst, sizeof(Inst32) * (size_t)n * b->ab));
    return FESOM_OK;
}

int fesom_gpu_batch_set_stream(fesom_gpu_batch *b, void *stream) {
    if (!b) return FESOM_ERR_ARG;
    b->stream = (cudaStream_t)stream;
    for (auto &g : b->gexec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    return FESOM_OK;
}

int fesom_gpu_batch_run_steps(fesom_gpu_batch *b, double dt, int32_t nsteps, int32_t use_graph) {
    if (!b || nsteps < 0) return FESOM_ERR_ARG;
    int rc;
    if (b->d_dt != dt) {
        BCK(cudaStreamSynchronize(b->stream));
        if ((rc = batch_descriptors(b, dt))) return rc;
    }
    for (int s = 0; s < nsteps; s++) {
        if (!use_graph) {
            enqueue_batch_step(b, b->stream);
            BCK(cudaGetLastError());
        } else {
            const int p = b->phase;
            if (!b->gexec[p] || b->g_dt[p] != dt) {
                if (b->gexec[p]) { cudaGraphExecDestroy(b->gexec[p]); b->gexec[p] = nullptr; }
                cudaStream_t cap = b->stream;
                bool own = false;
                if (!cap) {  // the legacy stream cannot be captured: capture on a private stream
                    BCK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
                    own = true;
                }
                cudaGraph_t graph;
                cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    enqueue_batch_step(b, cap);
                    e = cudaStreamEndCapture(cap, &graph);
                }
                if (own) cudaStreamDestroy(cap);
                if (e != cudaSuccess) { b->err = std::string("graph capture: ") + cudaGetErrorString(e); return FESOM_ERR_CUDA; }
                e = cudaGraphInstantiate(&b->gexec[p], graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) { b->err = std::string("graph instantiate: ") + cudaGetErrorString(e); return FESOM_ERR_CUDA; }
                b->g_dt[p] = dt;
            }
            BCK(cudaGraphLaunch(b->gexec[p], b->stream));
        }
        b->phase = (b->phase + 1) % b->ab;
        for (fesom_gpu_ctx *c : b->inst) {
            rotate32(c);
            // a context's own graphs were captured for its own rotation: its next
            // single-context step picks the graph of the new rotation
        }
    }
    return FESOM_OK;
}

int fesom_gpu_batch_launches_per_step(fesom_gpu_batch *b, int32_t *launches) {
    if (!b || !launches) return FESOM_ERR_ARG;
    const bool wide = b->ix_w.start[b->ix_w.n] > 0;
    const int k = wide ? 2 : 1;
    // vflux, vfactors (the diffusion itself runs inside the update), lo_ad and update (+ bounds,
    // diff) per node range, ho (+ its node-mean items), the optional stages
    int n = 1 + (b->any_vd ? 1 : 0) + k * (2 + (b->any_fct ? 1 : 0) + (b->any_diff ? 1 : 0)) + 1 +
            (b->ix_it.start[b->ix_it.n] ? 1 : 0) + (b->any_hd ? 1 : 0) + (b->any_ppm ? 1 : 0) +
            (b->any_lo_impl ? 1 : 0) + (b->any_wimpl ? 1 : 0);
    *launches = n;
    return FESOM_OK;
}

const char *fesom_gpu_batch_last_error(const fesom_gpu_batch *b) { return b ? b->err.c_str() : "null batch"; }

int fesom_gpu_batch_destroy(fesom_gpu_batch *b) {
    if (!b) return FESOM_OK;
    for (auto &g : b->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (b->d_inst) cudaFree(b->d_inst);
    delete b;
    return FESOM_OK;
}

}  // extern "C"
