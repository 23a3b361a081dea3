/*
 * tracer_oracle.c -- FP64 CPU restatement of FESOM2's tracer-transport step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See tracer_oracle.h.
 *
 * Each routine restates the reference loop for loop, in the reference's
 * evaluation order (left to right, no contraction: build with
 * -ffp-contract=off), with 1-based level indices as in the Fortran.  With one
 * thread every edge scatter runs in ascending edge order, which is the
 * reference's serial (and OPENMP_REPRODUCIBLE) order.  With more threads the
 * loops are split the way the reference's !$OMP directives split them and the
 * scatters take a per-node lock (the reference's default OpenMP build).
 *
 * Literal constants follow the reference's GNU build, which promotes default
 * reals to 8 bytes (-fdefault-real-8, src/CMakeLists.txt:383-388): flux_eps is
 * the double 1e-16 and bignumber the double 1e3.
 */
#include "tracer_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void or_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int or_get_threads(void) { return g_threads; }

#define R_EARTH 6367500.0        /* src/oce_modules.F90:29 */
#define AB_EPSILON 0.1           /* src/oce_modules.F90:105 */

#define OMP_FOR _Pragma("omp parallel for schedule(static) if(g_threads > 1) num_threads(g_threads)")

/* ---- per-node locks for the OpenMP scatters ----------------------------- */
#ifdef _OPENMP
static omp_lock_t *g_locks = NULL;
static int g_nlocks = 0;
static void locks_ensure(int n) {
    if (g_nlocks >= n) return;
    if (g_locks) {
        for (int i = 0; i < g_nlocks; i++) omp_destroy_lock(&g_locks[i]);
        free(g_locks);
    }
    g_locks = (omp_lock_t *)malloc(sizeof(omp_lock_t) * (size_t)n);
    for (int i = 0; i < n; i++) omp_init_lock(&g_locks[i]);
    g_nlocks = n;
}
#define LOCK(n)   do { if (g_threads > 1) omp_set_lock(&g_locks[(n)]); } while (0)
#define UNLOCK(n) do { if (g_threads > 1) omp_unset_lock(&g_locks[(n)]); } while (0)
#else
static void locks_ensure(int n) { (void)n; }
#define LOCK(n)   do { } while (0)
#define UNLOCK(n) do { } while (0)
#endif

/* ---- accessors: Fortran a(level, entity), level 1-based, entity 0-based --- */
#define IX1(nz, n) ((size_t)(n) * (size_t)L1 + (size_t)((nz) - 1))
#define IXN(nz, n) ((size_t)(n) * (size_t)NL + (size_t)((nz) - 1))

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* ========================================================================== */
/* muscl_adv_init / find_up_downwind_triangles  (src/oce_muscl_adv.F90:32-352) */
/* ========================================================================== */
void or_muscl_adv_init(const or_mesh *m, or_work *w) {
    const int NL = m->nl;
    /* nboundary_lay (:92-155) */
    for (int n = 0; n < m->nod2D; n++) w->nboundary_lay[n] = NL - 1;
    for (int e = 0; e < m->edge2D; e++) {
        int n1 = m->edges[2 * e], n2 = m->edges[2 * e + 1];
        int t1 = m->edge_tri[2 * e], t2 = m->edge_tri[2 * e + 1];
        if (t1 < 0 || t2 < 0) {
            w->nboundary_lay[n1] = 0;
            w->nboundary_lay[n2] = 0;
        } else {
            int mv = (m->nlevels[t1] < m->nlevels[t2] ? m->nlevels[t1] : m->nlevels[t2]) - 1;
            if (mv < w->nboundary_lay[n1]) w->nboundary_lay[n1] = mv;
            if (mv < w->nboundary_lay[n2]) w->nboundary_lay[n2] = mv;
        }
    }
    /* find_up_downwind_triangles (:240-333) */
    const double cyc = m->cyclic_length;
    const double *X = m->coord_nod2D;
    for (int e = 0; e < m->edge2D; e++) {
        w->edge_up_dn_tri[2 * e] = -1;
        w->edge_up_dn_tri[2 * e + 1] = -1;
    }
    for (int e = 0; e < m->edge2D; e++) {
        int ed[2] = {m->edges[2 * e], m->edges[2 * e + 1]};
        double x[2];
        x[0] = X[2 * ed[1]] - X[2 * ed[0]];
        x[1] = X[2 * ed[1] + 1] - X[2 * ed[0] + 1];
        if (x[0] > cyc / 2.0) x[0] = x[0] - cyc;
        if (x[0] < -cyc / 2.0) x[0] = x[0] + cyc;
        for (int side = 0; side < 2; side++) {
            /* side 0: look upwind of node 1 (x = -x); side 1: of node 2 (x restored) */
            x[0] = -x[0];
            x[1] = -x[1];
            int node = ed[side];
            for (int k = m->nod_in_elem2D_ptr[node]; k < m->nod_in_elem2D_ptr[node + 1]; k++) {
                int elem = m->nod_in_elem2D[k];
                const int *en = &m->elem2D_nodes[3 * elem];
                int i0, i1, i2;
                if (en[0] == node) { i0 = 0; i1 = 1; i2 = 2; }
                else if (en[1] == node) { i0 = 1; i1 = 0; i2 = 2; }
                else { i0 = 2; i1 = 0; i2 = 1; }
                double b[2], c[2];
                b[0] = X[2 * en[i1]] - X[2 * en[i0]];
                b[1] = X[2 * en[i1] + 1] - X[2 * en[i0] + 1];
                c[0] = X[2 * en[i2]] - X[2 * en[i0]];
                c[1] = X[2 * en[i2] + 1] - X[2 * en[i0] + 1];
                if (b[0] > cyc / 2.0) b[0] = b[0] - cyc;
                if (b[0] < -cyc / 2.0) b[0] = b[0] + cyc;
                if (c[0] > cyc / 2.0) c[0] = c[0] - cyc;
                if (c[0] < -cyc / 2.0) c[0] = c[0] + cyc;
                double cr = 0.0; cr += c[0] * c[0]; cr += c[1] * c[1];
                double s = 0.0; s += b[0] * c[0]; s += b[1] * c[1];
                double bx = s / cr;
                double by = (-(b[0] * c[1]) + b[1] * c[0]) / cr;
                s = 0.0; s += x[0] * c[0]; s += x[1] * c[1];
                double xx = s / cr;
                double xy = (-(x[0] * c[1]) + x[1] * c[0]) / cr;
                double ab = atan2(by, bx);
                double ax = atan2(xy, xx);
                if ((ab > 0.0) && (ax > 0.0) && (ax < ab)) { w->edge_up_dn_tri[2 * e + side] = elem; continue; }
                if ((ab < 0.0) && (ax < 0.0) && (ax > ab)) { w->edge_up_dn_tri[2 * e + side] = elem; continue; }
                if ((ab == ax) || (ax == 0.0)) { w->edge_up_dn_tri[2 * e + side] = elem; continue; }
            }
        }
    }
    const int L1 = NL - 1;
    memset(w->edge_up_dn_grad, 0, sizeof(double) * 4 * (size_t)L1 * (size_t)m->edge2D);
}

/* ========================================================================== */
/* gradients (src/oce_tracer_mod.F90:147-232) and fill_up_dn_grad             */
/* ========================================================================== */
void or_tracer_gradient_elements(const or_mesh *m, const double *ttf, double *tr_xy) {
    const int L1 = m->nl - 1;
    OMP_FOR
    for (int elem = 0; elem < m->elem2D; elem++) {
        const int *en = &m->elem2D_nodes[3 * elem];
        const double *gs = &m->gradient_sca[6 * elem];
        for (int nz = m->ulevels[elem]; nz <= m->nlevels[elem] - 1; nz++) {
            double s = 0.0;
            s += gs[0] * ttf[IX1(nz, en[0])];
            s += gs[1] * ttf[IX1(nz, en[1])];
            s += gs[2] * ttf[IX1(nz, en[2])];
            tr_xy[2 * IX1(nz, elem)] = s;
            s = 0.0;
            s += gs[3] * ttf[IX1(nz, en[0])];
            s += gs[4] * ttf[IX1(nz, en[1])];
            s += gs[5] * ttf[IX1(nz, en[2])];
            tr_xy[2 * IX1(nz, elem) + 1] = s;
        }
    }
}

void or_tracer_gradient_z(const or_mesh *m, const double *ttf, double *tr_z) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        for (int nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            double dz = 0.5 * (m->hnode[IX1(nz - 1, n)] + m->hnode[IX1(nz, n)]);
            tr_z[IXN(nz, n)] = (ttf[IX1(nz - 1, n)] - ttf[IX1(nz, n)]) / dz;
        }
        tr_z[IXN(nzmin, n)] = 0.0;
        tr_z[IXN(nzmax, n)] = 0.0;
    }
}

/* area-weighted mean of tr_xy over the node's elements that are wet at nz */
static inline void node_mean_grad(const or_mesh *m, const double *tr_xy, int node, int nz, double *gx,
                                  double *gy) {
    const int L1 = m->nl - 1;
    double tvol = 0.0, tx = 0.0, ty = 0.0;
    for (int k = m->nod_in_elem2D_ptr[node]; k < m->nod_in_elem2D_ptr[node + 1]; k++) {
        int elem = m->nod_in_elem2D[k];
        if (m->nlevels[elem] - 1 < nz || nz < m->ulevels[elem]) continue;
        tvol = tvol + m->elem_area[elem];
        tx = tx + tr_xy[2 * IX1(nz, elem)] * m->elem_area[elem];
        ty = ty + tr_xy[2 * IX1(nz, elem) + 1] * m->elem_area[elem];
    }
    *gx = tx / tvol;
    *gy = ty / tvol;
}

void or_fill_up_dn_grad(const or_mesh *m, or_work *w) {
    const int L1 = m->nl - 1;
    double *G = w->edge_up_dn_grad;
#define GR(k, nz, e) G[4 * IX1(nz, e) + (k) - 1]
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        int ed[2] = {m->edges[2 * edge], m->edges[2 * edge + 1]};
        int up = w->edge_up_dn_tri[2 * edge], dn = w->edge_up_dn_tri[2 * edge + 1];
        double gx, gy;
        if (up >= 0 && dn >= 0) {
            int nzmin = m->ulevels_nod2D_max[ed[0]] > m->ulevels_nod2D_max[ed[1]] ? m->ulevels_nod2D_max[ed[0]]
                                                                                 : m->ulevels_nod2D_max[ed[1]];
            int nzmax = m->nlevels_nod2D_min[ed[0]] < m->nlevels_nod2D_min[ed[1]] ? m->nlevels_nod2D_min[ed[0]]
                                                                                 : m->nlevels_nod2D_min[ed[1]];
            for (int nz = m->ulevels_nod2D[ed[0]]; nz <= nzmin - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[0], nz, &gx, &gy);
                GR(1, nz, edge) = gx; GR(3, nz, edge) = gy;
            }
            for (int nz = m->ulevels_nod2D[ed[1]]; nz <= nzmin - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[1], nz, &gx, &gy);
                GR(2, nz, edge) = gx; GR(4, nz, edge) = gy;
            }
            for (int nz = nzmin; nz <= nzmax - 1; nz++) {
                GR(1, nz, edge) = w->tr_xy[2 * IX1(nz, up)];
                GR(2, nz, edge) = w->tr_xy[2 * IX1(nz, dn)];
                GR(3, nz, edge) = w->tr_xy[2 * IX1(nz, up) + 1];
                GR(4, nz, edge) = w->tr_xy[2 * IX1(nz, dn) + 1];
            }
            for (int nz = nzmax; nz <= m->nlevels_nod2D[ed[0]] - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[0], nz, &gx, &gy);
                GR(1, nz, edge) = gx; GR(3, nz, edge) = gy;
            }
            for (int nz = nzmax; nz <= m->nlevels_nod2D[ed[1]] - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[1], nz, &gx, &gy);
                GR(2, nz, edge) = gx; GR(4, nz, edge) = gy;
            }
        } else {
            for (int nz = m->ulevels_nod2D[ed[0]]; nz <= m->nlevels_nod2D[ed[0]] - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[0], nz, &gx, &gy);
                GR(1, nz, edge) = gx; GR(3, nz, edge) = gy;
            }
            for (int nz = m->ulevels_nod2D[ed[1]]; nz <= m->nlevels_nod2D[ed[1]] - 1; nz++) {
                node_mean_grad(m, w->tr_xy, ed[1], nz, &gx, &gy);
                GR(2, nz, edge) = gx; GR(4, nz, edge) = gy;
            }
        }
    }
#undef GR
}

/* ========================================================================== */
/* init_tracers_AB (src/oce_tracer_mod.F90:13-143)                             */
/* ========================================================================== */
void or_init_tracers_AB(const or_mesh *m, const or_tra_cfg *c, double *values, double *valuesAB,
                        double *valuesold, or_work *w) {
    const int L1 = m->nl - 1;
    const size_t N = (size_t)L1 * (size_t)m->nod2D;
    memset(w->del_ttf, 0, sizeof(double) * N);
    memset(w->del_ttf_advhoriz, 0, sizeof(double) * N);
    memset(w->del_ttf_advvert, 0, sizeof(double) * N);
    if (c->ab_order == 2) {
        const double ca = 0.5 + AB_EPSILON, cb = 1.5 + AB_EPSILON;
        OMP_FOR
        for (long i = 0; i < (long)N; i++) valuesAB[i] = -(ca * valuesold[i]) + cb * values[i];
        OMP_FOR
        for (long i = 0; i < (long)N; i++) valuesold[i] = values[i];
    } else {
        OMP_FOR
        for (long i = 0; i < (long)N; i++) {
            double v = 5.0 * valuesold[2 * i + 1] - 16.0 * valuesold[2 * i] + 23.0 * values[i];
            valuesAB[i] = v / 12.0;
        }
        OMP_FOR
        for (long i = 0; i < (long)N; i++) {
            valuesold[2 * i + 1] = valuesold[2 * i];
            valuesold[2 * i] = values[i];
        }
    }
    or_tracer_gradient_elements(m, values, w->tr_xy);
    or_tracer_gradient_z(m, values, w->tr_z);
    or_fill_up_dn_grad(m, w);
}

/* ========================================================================== */
/* horizontal fluxes (src/oce_adv_tra_hor.F90)                                 */
/* ========================================================================== */
typedef struct {
    int n1, n2, el1, el2, nl1, nu1, nl2, nu2;
    double dX1, dY1, dX2, dY2, a;
} edge_geo;

static inline void edge_setup(const or_mesh *m, int edge, edge_geo *g) {
    g->n1 = m->edges[2 * edge];
    g->n2 = m->edges[2 * edge + 1];
    g->el1 = m->edge_tri[2 * edge];
    g->el2 = m->edge_tri[2 * edge + 1];
    g->nl1 = m->nlevels[g->el1] - 1;
    g->nu1 = m->ulevels[g->el1];
    g->dX1 = m->edge_cross_dxdy[4 * edge + 0];
    g->dY1 = m->edge_cross_dxdy[4 * edge + 1];
    g->a = R_EARTH * m->elem_cos[g->el1];
    g->nl2 = 0;
    g->nu2 = 0;
    g->dX2 = 0.0;
    g->dY2 = 0.0;
    if (g->el2 >= 0) {
        g->dX2 = m->edge_cross_dxdy[4 * edge + 2];
        g->dY2 = m->edge_cross_dxdy[4 * edge + 3];
        g->nl2 = m->nlevels[g->el2] - 1;
        g->nu2 = m->ulevels[g->el2];
        g->a = 0.5 * (g->a + R_EARTH * m->elem_cos[g->el2]);
    }
}

#define VEL(c, nz, el) vel[2 * IX1(nz, el) + (c) - 1]

/* volume flux of segment 1, segment 2, both (oce_adv_tra_hor.F90:170,190,211-212) */
static inline double vflux1(const or_mesh *m, const double *vel, const edge_geo *g, int nz) {
    const int L1 = m->nl - 1;
    return (-(VEL(2, nz, g->el1) * g->dX1) + VEL(1, nz, g->el1) * g->dY1) * m->helem[IX1(nz, g->el1)];
}
static inline double vflux2(const or_mesh *m, const double *vel, const edge_geo *g, int nz) {
    const int L1 = m->nl - 1;
    return (VEL(2, nz, g->el2) * g->dX2 - VEL(1, nz, g->el2) * g->dY2) * m->helem[IX1(nz, g->el2)];
}
static inline double vflux12(const or_mesh *m, const double *vel, const edge_geo *g, int nz) {
    return vflux1(m, vel, g, nz) + vflux2(m, vel, g, nz);
}

void or_adv_tra_hor_upw1(const or_mesh *m, const double *vel, const double *ttf, double *flux, int init_zero) {
    const int L1 = m->nl - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)L1 * (size_t)m->edge2D);
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        edge_geo g;
        edge_setup(m, edge, &g);
        int nl12 = g.nl1 < g.nl2 ? g.nl1 : g.nl2;
        int nu12 = g.nu1 > g.nu2 ? g.nu1 : g.nu2;
#define UPW(vf)                                                                                          \
    flux[IX1(nz, edge)] = -(0.5 * (ttf[IX1(nz, g.n1)] * ((vf) + fabs(vf)) + ttf[IX1(nz, g.n2)] * ((vf) - fabs(vf)))) - \
                          flux[IX1(nz, edge)]
        for (int nz = g.nu1; nz <= nu12 - 1; nz++) { double vf = vflux1(m, vel, &g, nz); UPW(vf); }
        if (g.nu2 > 0)
            for (int nz = g.nu2; nz <= nu12 - 1; nz++) { double vf = vflux2(m, vel, &g, nz); UPW(vf); }
        for (int nz = nu12; nz <= nl12; nz++) { double vf = vflux12(m, vel, &g, nz); UPW(vf); }
        for (int nz = nl12 + 1; nz <= g.nl1; nz++) { double vf = vflux1(m, vel, &g, nz); UPW(vf); }
        for (int nz = nl12 + 1; nz <= g.nl2; nz++) { double vf = vflux2(m, vel, &g, nz); UPW(vf); }
#undef UPW
    }
}

/* MUSCL (use_clo = 1, :261-542) and MFCT (use_clo = 0, :546-834) */
static void hor_ho(const or_mesh *m, const double *vel, const double *ttf, double num_ord, double *flux,
                   const double *G, const int *nboundary_lay, int use_clo, int init_zero) {
    const int L1 = m->nl - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)L1 * (size_t)m->edge2D);
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        edge_geo g;
        edge_setup(m, edge, &g);
        int nl12 = g.nl1 < g.nl2 ? g.nl1 : g.nl2;
        int nu12 = g.nu1 > g.nu2 ? g.nu1 : g.nu2;
        const double ex = m->edge_dxdy[2 * edge], ey = m->edge_dxdy[2 * edge + 1];
#define HO(vf)                                                                                                 \
    do {                                                                                                       \
        double t1 = ttf[IX1(nz, g.n1)], t2 = ttf[IX1(nz, g.n2)];                                               \
        const double *gg = &G[4 * IX1(nz, edge)];                                                              \
        double Tmean2, Tmean1;                                                                                 \
        if (use_clo) {                                                                                         \
            double clo1 = (nboundary_lay[g.n1] - nz) >= 0 ? 1.0 : 0.0;                                         \
            double clo2 = (nboundary_lay[g.n2] - nz) >= 0 ? 1.0 : 0.0;                                         \
            Tmean2 = t2 - (2.0 * (t2 - t1) + ex * g.a * gg[1] + ey * R_EARTH * gg[3]) / 6.0 * clo2;           \
            Tmean1 = t1 + (2.0 * (t2 - t1) + ex * g.a * gg[0] + ey * R_EARTH * gg[2]) / 6.0 * clo1;           \
        } else {                                                                                               \
            Tmean2 = t2 - (2.0 * (t2 - t1) + ex * g.a * gg[1] + ey * R_EARTH * gg[3]) / 6.0;                  \
            Tmean1 = t1 + (2.0 * (t2 - t1) + ex * g.a * gg[0] + ey * R_EARTH * gg[2]) / 6.0;                  \
        }                                                                                                      \
        double cHO = ((vf) + fabs(vf)) * Tmean1 + ((vf) - fabs(vf)) * Tmean2;                                  \
        flux[IX1(nz, edge)] =                                                                                  \
            -(0.5 * (1.0 - num_ord) * cHO) - (vf) * num_ord * 0.5 * (Tmean1 + Tmean2) - flux[IX1(nz, edge)];   \
    } while (0)
        for (int nz = g.nu1; nz <= nu12 - 1; nz++) { double vf = vflux1(m, vel, &g, nz); HO(vf); }
        if (g.nu2 > 0)
            for (int nz = g.nu2; nz <= nu12 - 1; nz++) { double vf = vflux2(m, vel, &g, nz); HO(vf); }
        for (int nz = nu12; nz <= nl12; nz++) { double vf = vflux12(m, vel, &g, nz); HO(vf); }
        for (int nz = nl12 + 1; nz <= g.nl1; nz++) { double vf = vflux1(m, vel, &g, nz); HO(vf); }
        for (int nz = nl12 + 1; nz <= g.nl2; nz++) { double vf = vflux2(m, vel, &g, nz); HO(vf); }
#undef HO
    }
}

void or_adv_tra_hor_muscl(const or_mesh *m, const double *vel, const double *ttf, double num_ord, double *flux,
                          const double *edge_up_dn_grad, const int *nboundary_lay, int init_zero) {
    hor_ho(m, vel, ttf, num_ord, flux, edge_up_dn_grad, nboundary_lay, 1, init_zero);
}
void or_adv_tra_hor_mfct(const or_mesh *m, const double *vel, const double *ttf, double num_ord, double *flux,
                         const double *edge_up_dn_grad, int init_zero) {
    hor_ho(m, vel, ttf, num_ord, flux, edge_up_dn_grad, NULL, 0, init_zero);
}

/* ========================================================================== */
/* vertical fluxes (src/oce_adv_tra_ver.F90:244-434)                           */
/* ========================================================================== */
void or_adv_tra_ver_upw1(const or_mesh *m, const double *W, const double *ttf, double *flux, int init_zero) {
    const int NL = m->nl, L1 = NL - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)NL * (size_t)m->nod2D);
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        int nz = nzmin;
        flux[IXN(nz, n)] = -(W[IXN(nz, n)] * ttf[IX1(nz, n)] * m->area[IXN(nz, n)]) - flux[IXN(nz, n)];
        nz = nzmax;
        flux[IXN(nz, n)] = 0.0 - flux[IXN(nz, n)];
        for (nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            double Wv = W[IXN(nz, n)];
            flux[IXN(nz, n)] = -(0.5 * (ttf[IX1(nz, n)] * (Wv + fabs(Wv)) + ttf[IX1(nz - 1, n)] * (Wv - fabs(Wv))) *
                                 m->area[IXN(nz, n)]) -
                               flux[IXN(nz, n)];
        }
    }
}

void or_adv_tra_ver_qr4c(const or_mesh *m, const double *W, const double *ttf, double num_ord, double *flux,
                         int init_zero) {
    const int NL = m->nl, L1 = NL - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)NL * (size_t)m->nod2D);
    const double *Zn = m->Z_3d_n, *zb = m->zbar_3d_n;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        int nz = nzmin;
        flux[IXN(nz, n)] = -(ttf[IX1(nz, n)] * W[IXN(nz, n)] * m->area[IXN(nz, n)]) - flux[IXN(nz, n)];
        nz = nzmin + 1;
        flux[IXN(nz, n)] = -(0.5 * (ttf[IX1(nz - 1, n)] + ttf[IX1(nz, n)]) * W[IXN(nz, n)] * m->area[IXN(nz, n)]) -
                           flux[IXN(nz, n)];
        nz = nzmax - 1;
        flux[IXN(nz, n)] = -(0.5 * (ttf[IX1(nz - 1, n)] + ttf[IX1(nz, n)]) * W[IXN(nz, n)] * m->area[IXN(nz, n)]) -
                           flux[IXN(nz, n)];
        nz = nzmax;
        flux[IXN(nz, n)] = 0.0 - flux[IXN(nz, n)];
        for (nz = nzmin + 2; nz <= nzmax - 2; nz++) {
            double qc = (ttf[IX1(nz - 1, n)] - ttf[IX1(nz, n)]) / (Zn[IX1(nz - 1, n)] - Zn[IX1(nz, n)]);
            double qu = (ttf[IX1(nz, n)] - ttf[IX1(nz + 1, n)]) / (Zn[IX1(nz, n)] - Zn[IX1(nz + 1, n)]);
            double qd = (ttf[IX1(nz - 2, n)] - ttf[IX1(nz - 1, n)]) / (Zn[IX1(nz - 2, n)] - Zn[IX1(nz - 1, n)]);
            double Tmean1 = ttf[IX1(nz, n)] + (2.0 * qc + qu) * (zb[IXN(nz, n)] - Zn[IX1(nz, n)]) / 3.0;
            double Tmean2 = ttf[IX1(nz - 1, n)] + (2.0 * qc + qd) * (zb[IXN(nz, n)] - Zn[IX1(nz - 1, n)]) / 3.0;
            double Wv = W[IXN(nz, n)];
            double Tmean = (Wv + fabs(Wv)) * Tmean1 + (Wv - fabs(Wv)) * Tmean2;
            flux[IXN(nz, n)] = (-(0.5 * (1.0 - num_ord) * Tmean) - num_ord * (0.5 * (Tmean1 + Tmean2)) * Wv) *
                                   m->area[IXN(nz, n)] -
                               flux[IXN(nz, n)];
        }
    }
}

/* adv_tra_ver_cdiff (src/oce_adv_tra_ver.F90:635-695): centred interface values; the flux
 * of the bottom interface is left as it was (only nzmin..nlevels-1 are written) */
void or_adv_tra_ver_cdiff(const or_mesh *m, const double *W, const double *ttf, double *flux, int init_zero) {
    const int NL = m->nl, L1 = NL - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)NL * (size_t)m->nod2D);
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double tvert[NL + 2];
        const int nzmax = m->nlevels_nod2D[n] - 1, nzmin = m->ulevels_nod2D[n];
        tvert[nzmin] = -(W[IXN(nzmin, n)] * ttf[IX1(nzmin, n)] * m->area[IXN(nzmin, n)]);
        tvert[nzmax + 1] = 0.0;
        for (int nz = nzmin + 1; nz <= nzmax; nz++) {
            double tv = 0.5 * (ttf[IX1(nz - 1, n)] + ttf[IX1(nz, n)]);
            tvert[nz] = -(tv * W[IXN(nz, n)] * m->area[IXN(nz, n)]);
        }
        for (int nz = nzmin; nz <= nzmax; nz++) flux[IXN(nz, n)] = tvert[nz] - flux[IXN(nz, n)];
    }
}

/* Fortran sign(1.0, b): the sign of b, -1 for -0.0 as well */
static inline double sign1(double b) { return signbit(b) ? -1.0 : 1.0; }
static inline double min3(double a, double b, double c) { double x = a < b ? a : b; return x < c ? x : c; }

/* adv_tra_vert_ppm (src/oce_adv_tra_ver.F90:438-631): interface values of the non-uniform
 * piecewise parabolic reconstruction on the new thicknesses (Colella and Woodward 1984,
 * eqs. 1.6-1.8; centred values next to the surface and the bottom), then per layer a
 * monotonised parabola integrated over the part swept upwind in dt (old thickness) */
void or_adv_tra_vert_ppm(const or_mesh *m, double dt, const double *W, const double *ttf, double *flux,
                         int init_zero) {
    const int NL = m->nl, L1 = NL - 1;
    if (init_zero) memset(flux, 0, sizeof(double) * (size_t)NL * (size_t)m->nod2D);
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double tvert[NL + 2], tv[NL + 2];
        const int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        const double *T = &ttf[IX1(1, n)] - 1, *hn = &m->hnode_new[IX1(1, n)] - 1, *ho = &m->hnode[IX1(1, n)] - 1;
        const double *w = &W[IXN(1, n)] - 1, *ar = &m->area[IXN(1, n)] - 1;
        tv[nzmin] = T[nzmin];
        tv[nzmin + 1] = 0.5 * (T[nzmin] + T[nzmin + 1]);
        tv[nzmax - 1] = 0.5 * (T[nzmax - 2] + T[nzmax - 1]);
        tv[nzmax] = T[nzmax - 1];
        for (int nz = nzmin + 1; nz <= nzmax - 3; nz++) {
            const double dzjm1 = hn[nz - 1], dzj = hn[nz], dzjp1 = hn[nz + 1], dzjp2 = hn[nz + 2];
            double deltaj = dzj / (dzjm1 + dzj + dzjp1) *
                            ((2.0 * dzjm1 + dzj) / (dzjp1 + dzj) * (T[nz + 1] - T[nz]) +
                             (dzj + 2.0 * dzjp1) / (dzjm1 + dzj) * (T[nz] - T[nz - 1]));
            double deltajp1 = dzjp1 / (dzj + dzjp1 + dzjp2) *
                              ((2.0 * dzj + dzjp1) / (dzjp2 + dzjp1) * (T[nz + 2] - T[nz + 1]) +
                               (dzjp1 + 2.0 * dzjp2) / (dzj + dzjp1) * (T[nz + 1] - T[nz]));
            if ((T[nz + 1] - T[nz]) * (T[nz] - T[nz - 1]) > 0.0)
                deltaj = min3(fabs(deltaj), 2.0 * fabs(T[nz + 1] - T[nz]), 2.0 * fabs(T[nz] - T[nz - 1])) * sign1(deltaj);
            else
                deltaj = 0.0;
            if ((T[nz + 2] - T[nz + 1]) * (T[nz + 1] - T[nz]) > 0.0)
                deltajp1 = min3(fabs(deltajp1), 2.0 * fabs(T[nz + 2] - T[nz + 1]), 2.0 * fabs(T[nz + 1] - T[nz])) *
                           sign1(deltajp1);
            else
                deltajp1 = 0.0;
            tv[nz + 1] = T[nz] + dzj / (dzj + dzjp1) * (T[nz + 1] - T[nz]) +
                         1.0 / (dzjm1 + dzj + dzjp1 + dzjp2) *
                             ((2.0 * dzjp1 * dzj) / (dzj + dzjp1) *
                                  ((dzjm1 + dzj) / (2.0 * dzj + dzjp1) - (dzjp2 + dzjp1) / (2.0 * dzjp1 + dzj)) *
                                  (T[nz + 1] - T[nz]) -
                              dzj * (dzjm1 + dzj) / (2.0 * dzj + dzjp1) * deltajp1 +
                              dzjp1 * (dzjp1 + dzjp2) / (dzj + 2.0 * dzjp1) * deltaj);
        }
        for (int k = 1; k <= nzmax; k++) tvert[k] = 0.0;
        for (int nz = nzmin; nz <= nzmax - 1; nz++) {
            if (w[nz] <= 0.0 && w[nz + 1] >= 0.0) continue;
            double aL = tv[nz], aR = tv[nz + 1];
            if ((aR - T[nz]) * (T[nz] - aL) <= 0.0) {
                aL = T[nz];
                aR = T[nz];
            }
            if ((aR - aL) * (T[nz] - 0.5 * (aL + aR)) > (aR - aL) * (aR - aL) / 6.0) aL = 3.0 * T[nz] - 2.0 * aR;
            if ((aR - aL) * (T[nz] - 0.5 * (aR + aL)) < -((aR - aL) * (aR - aL) / 6.0)) aR = 3.0 * T[nz] - 2.0 * aL;
            const double dzj = ho[nz];
            const double aj = 6.0 * (T[nz] - 0.5 * (aL + aR));
            if (w[nz] > 0.0) {
                double x = fmin(w[nz] * dt / dzj, 1.0);
                tvert[nz] = -aL - 0.5 * x * (aR - aL + (1.0 - 2.0 / 3.0 * x) * aj);
                tvert[nz] = tvert[nz] * ar[nz] * w[nz];
            }
            if (w[nz + 1] < 0.0) {
                double x = fmin(-(w[nz + 1] * dt / dzj), 1.0);
                tvert[nz + 1] = -aR + 0.5 * x * (aR - aL - (1.0 - 2.0 / 3.0 * x) * aj);
                tvert[nz + 1] = tvert[nz + 1] * ar[nz + 1] * w[nz + 1];
            }
        }
        tvert[nzmin] = -(tv[nzmin] * w[nzmin] * ar[nzmin]);
        tvert[nzmax] = 0.0;
        for (int nz = nzmin; nz <= nzmax; nz++) flux[IXN(nz, n)] = tvert[nz] - flux[IXN(nz, n)];
    }
}

/* adv_tra_vert_impl (src/oce_adv_tra_ver.F90:90-240): implicit upwind advection by W of a
 * column field, in place (a tridiagonal solve per column on the new thicknesses) */
void or_adv_tra_vert_impl(const or_mesh *m, double dt, const double *W, double *ttf) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double a[NL + 1], b[NL + 1], c[NL + 1], tr[NL + 1], cp[NL + 1], tp[NL + 1];
        for (int k = 0; k <= NL; k++) a[k] = b[k] = c[k] = tr[k] = cp[k] = tp[k] = 0.0;
        const int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        const double *hn = &m->hnode_new[IX1(1, n)] - 1, *w = &W[IXN(1, n)] - 1;
        const double *ar = &m->area[IXN(1, n)] - 1, *av = &m->areasvol[IXN(1, n)] - 1;
        double *T = &ttf[IX1(1, n)] - 1;
        const double zinv = 1.0 * dt;
        int nz = nzmin;
        a[nz] = 0.0;
        double v_adv = zinv * ar[nz] / av[nz];
        b[nz] = hn[nz] + w[nz] * v_adv;
        v_adv = zinv * ar[nz + 1] / av[nz];
        b[nz] = b[nz] - fmin(0.0, w[nz + 1]) * v_adv;
        c[nz] = -(fmax(0.0, w[nz + 1]) * v_adv);
        for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
            v_adv = zinv * ar[nz] / av[nz];
            a[nz] = fmin(0.0, w[nz]) * v_adv;
            b[nz] = hn[nz] + fmax(0.0, w[nz]) * v_adv;
            v_adv = zinv * ar[nz + 1] / av[nz];
            b[nz] = b[nz] - fmin(0.0, w[nz + 1]) * v_adv;
            c[nz] = -(fmax(0.0, w[nz + 1]) * v_adv);
        }
        nz = nzmax - 1;
        v_adv = zinv * ar[nz] / av[nz];
        a[nz] = fmin(0.0, w[nz]) * v_adv;
        b[nz] = hn[nz] + fmax(0.0, w[nz]) * v_adv;
        c[nz] = 0.0;
        nz = nzmin;
        tr[nz] = -((b[nz] - hn[nz]) * T[nz]) - c[nz] * T[nz + 1];
        for (nz = nzmin + 1; nz <= nzmax - 2; nz++)
            tr[nz] = -(a[nz] * T[nz - 1]) - (b[nz] - hn[nz]) * T[nz] - c[nz] * T[nz + 1];
        nz = nzmax - 1;
        tr[nz] = -(a[nz] * T[nz - 1]) - (b[nz] - hn[nz]) * T[nz];
        cp[nzmin] = c[nzmin] / b[nzmin];
        tp[nzmin] = tr[nzmin] / b[nzmin];
        for (nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            double mm = b[nz] - cp[nz - 1] * a[nz];
            cp[nz] = c[nz] / mm;
            tp[nz] = (tr[nz] - tp[nz - 1] * a[nz]) / mm;
        }
        tr[nzmax - 1] = tp[nzmax - 1];
        for (nz = nzmax - 2; nz >= nzmin; nz--) tr[nz] = tp[nz] - cp[nz] * tr[nz + 1];
        for (nz = nzmin; nz <= nzmax - 1; nz++) T[nz] = T[nz] + tr[nz];
    }
}

/* ========================================================================== */
/* FCT limiter (src/oce_adv_tra_fct.F90:72-512)                                */
/* ========================================================================== */
static inline void edge_scatter_range(const or_mesh *m, int edge, int *nu12, int *nl12) {
    int el1 = m->edge_tri[2 * edge], el2 = m->edge_tri[2 * edge + 1];
    int nl1 = m->nlevels[el1] - 1, nu1 = m->ulevels[el1];
    int nl2 = 0, nu2 = 0;
    if (el2 >= 0) {
        nl2 = m->nlevels[el2] - 1;
        nu2 = m->ulevels[el2];
    }
    *nl12 = nl1 > nl2 ? nl1 : nl2;
    *nu12 = nu1;
    if (nu2 > 0) *nu12 = nu1 < nu2 ? nu1 : nu2;
}

void or_oce_tra_adv_fct(const or_mesh *m, double dt, const double *ttf, const double *lo, double *adf_h,
                        double *adf_v, or_work *w) {
    const int NL = m->nl, L1 = NL - 1;
    const double flux_eps = 1e-16, bignumber = 1e3;
    double *fmax = w->fct_ttf_max, *fmin = w->fct_ttf_min, *fplus = w->fct_plus, *fminus = w->fct_minus;
    double *tmax = w->tvert_max, *tmin = w->tvert_min;
    double *AUX = w->edge_up_dn_grad; /* AUX(1:2, nz, elem) aliases edge_up_dn_grad */
#define AUXA(k, nz, el) AUX[4 * IX1(nz, el) + (k) - 1]
    locks_ensure(m->nod2D);
    /* a1 */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++)
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            fmax[IX1(nz, n)] = dmax(lo[IX1(nz, n)], ttf[IX1(nz, n)]);
            fmin[IX1(nz, n)] = dmin(lo[IX1(nz, n)], ttf[IX1(nz, n)]);
        }
    /* a2 */
    OMP_FOR
    for (int elem = 0; elem < m->elem2D; elem++) {
        const int *en = &m->elem2D_nodes[3 * elem];
        int nu1 = m->ulevels[elem], nl1 = m->nlevels[elem];
        if (nu1 > 1)
            for (int nz = 1; nz <= nu1 - 1; nz++) { AUXA(1, nz, elem) = -bignumber; AUXA(2, nz, elem) = bignumber; }
        for (int nz = nu1; nz <= nl1 - 1; nz++) {
            AUXA(1, nz, elem) = dmax(dmax(fmax[IX1(nz, en[0])], fmax[IX1(nz, en[1])]), fmax[IX1(nz, en[2])]);
            AUXA(2, nz, elem) = dmin(dmin(fmin[IX1(nz, en[0])], fmin[IX1(nz, en[1])]), fmin[IX1(nz, en[2])]);
        }
        if (nl1 <= NL - 1)
            for (int nz = nl1; nz <= NL - 1; nz++) { AUXA(1, nz, elem) = -bignumber; AUXA(2, nz, elem) = bignumber; }
    }
    /* a3 */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int k0 = m->nod_in_elem2D_ptr[n], k1 = m->nod_in_elem2D_ptr[n + 1];
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            tmax[IX1(nz, n)] = AUXA(1, nz, m->nod_in_elem2D[k0]);
            tmin[IX1(nz, n)] = AUXA(2, nz, m->nod_in_elem2D[k0]);
            for (int k = k0 + 1; k < k1; k++) {
                tmax[IX1(nz, n)] = dmax(tmax[IX1(nz, n)], AUXA(1, nz, m->nod_in_elem2D[k]));
                tmin[IX1(nz, n)] = dmin(tmin[IX1(nz, n)], AUXA(2, nz, m->nod_in_elem2D[k]));
            }
        }
    }
    /* bound increments */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nu1 = m->ulevels_nod2D[n], nl1 = m->nlevels_nod2D[n];
        fmax[IX1(nu1, n)] = tmax[IX1(nu1, n)] - lo[IX1(nu1, n)];
        fmin[IX1(nu1, n)] = tmin[IX1(nu1, n)] - lo[IX1(nu1, n)];
        for (int nz = nu1 + 1; nz <= nl1 - 2; nz++) {
            fmax[IX1(nz, n)] = dmax(dmax(tmax[IX1(nz - 1, n)], tmax[IX1(nz, n)]), tmax[IX1(nz + 1, n)]) - lo[IX1(nz, n)];
            fmin[IX1(nz, n)] = dmin(dmin(tmin[IX1(nz - 1, n)], tmin[IX1(nz, n)]), tmin[IX1(nz + 1, n)]) - lo[IX1(nz, n)];
        }
        int nz = nl1 - 1;
        fmax[IX1(nz, n)] = tmax[IX1(nz, n)] - lo[IX1(nz, n)];
        fmin[IX1(nz, n)] = tmin[IX1(nz, n)] - lo[IX1(nz, n)];
    }
    /* b1: vertical part */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++)
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            fplus[IX1(nz, n)] = 0.0;
            fminus[IX1(nz, n)] = 0.0;
        }
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++)
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            fplus[IX1(nz, n)] = fplus[IX1(nz, n)] + (dmax(0.0, adf_v[IXN(nz, n)]) + dmax(0.0, -adf_v[IXN(nz + 1, n)]));
            fminus[IX1(nz, n)] = fminus[IX1(nz, n)] + (dmin(0.0, adf_v[IXN(nz, n)]) + dmin(0.0, -adf_v[IXN(nz + 1, n)]));
        }
    /* b1: horizontal scatter */
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        int n1 = m->edges[2 * edge], n2 = m->edges[2 * edge + 1], nu12, nl12;
        edge_scatter_range(m, edge, &nu12, &nl12);
        LOCK(n1);
        for (int nz = nu12; nz <= nl12; nz++) {
            fplus[IX1(nz, n1)] = fplus[IX1(nz, n1)] + dmax(0.0, adf_h[IX1(nz, edge)]);
            fminus[IX1(nz, n1)] = fminus[IX1(nz, n1)] + dmin(0.0, adf_h[IX1(nz, edge)]);
        }
        UNLOCK(n1);
        LOCK(n2);
        for (int nz = nu12; nz <= nl12; nz++) {
            fplus[IX1(nz, n2)] = fplus[IX1(nz, n2)] + dmax(0.0, -adf_h[IX1(nz, edge)]);
            fminus[IX1(nz, n2)] = fminus[IX1(nz, n2)] + dmin(0.0, -adf_h[IX1(nz, edge)]);
        }
        UNLOCK(n2);
    }
    /* b2 */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++)
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            double flux = fplus[IX1(nz, n)] * dt / m->areasvol[IXN(nz, n)] / m->hnode_new[IX1(nz, n)] + flux_eps;
            fplus[IX1(nz, n)] = dmin(1.0, fmax[IX1(nz, n)] / flux);
            flux = fminus[IX1(nz, n)] * dt / m->areasvol[IXN(nz, n)] / m->hnode_new[IX1(nz, n)] - flux_eps;
            fminus[IX1(nz, n)] = dmin(1.0, fmin[IX1(nz, n)] / flux);
        }
    /* b3: vertical */
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nu1 = m->ulevels_nod2D[n], nl1 = m->nlevels_nod2D[n];
        int nz = nu1;
        double ae = 1.0, flux = adf_v[IXN(nz, n)];
        if (flux >= 0.0) ae = dmin(ae, fplus[IX1(nz, n)]);
        else ae = dmin(ae, fminus[IX1(nz, n)]);
        adf_v[IXN(nz, n)] = ae * adf_v[IXN(nz, n)];
        for (nz = nu1 + 1; nz <= nl1 - 1; nz++) {
            ae = 1.0;
            flux = adf_v[IXN(nz, n)];
            if (flux >= 0.0) {
                ae = dmin(ae, fminus[IX1(nz - 1, n)]);
                ae = dmin(ae, fplus[IX1(nz, n)]);
            } else {
                ae = dmin(ae, fplus[IX1(nz - 1, n)]);
                ae = dmin(ae, fminus[IX1(nz, n)]);
            }
            adf_v[IXN(nz, n)] = ae * adf_v[IXN(nz, n)];
        }
    }
    /* b3: horizontal */
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        int n1 = m->edges[2 * edge], n2 = m->edges[2 * edge + 1], nu12, nl12;
        edge_scatter_range(m, edge, &nu12, &nl12);
        for (int nz = nu12; nz <= nl12; nz++) {
            double ae = 1.0, flux = adf_h[IX1(nz, edge)];
            if (flux >= 0.0) {
                ae = dmin(ae, fplus[IX1(nz, n1)]);
                ae = dmin(ae, fminus[IX1(nz, n2)]);
            } else {
                ae = dmin(ae, fminus[IX1(nz, n1)]);
                ae = dmin(ae, fplus[IX1(nz, n2)]);
            }
            adf_h[IX1(nz, edge)] = ae * adf_h[IX1(nz, edge)];
        }
    }
#undef AUXA
}

/* ========================================================================== */
/* oce_tra_adv_flux2dtracer (src/oce_adv_tra_driver.F90:494-646)               */
/* ========================================================================== */
void or_oce_tra_adv_flux2dtracer(const or_mesh *m, double dt, double *dttf_h, double *dttf_v,
                                 const double *flux_h, const double *flux_v, int use_lo, const double *ttf,
                                 const double *lo) {
    const int NL = m->nl, L1 = NL - 1;
    locks_ensure(m->nod2D);
    if (use_lo) {
        OMP_FOR
        for (int n = 0; n < m->nod2D; n++)
            for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++)
                dttf_v[IX1(nz, n)] = dttf_v[IX1(nz, n)] - ttf[IX1(nz, n)] * m->hnode[IX1(nz, n)] +
                                     lo[IX1(nz, n)] * m->hnode_new[IX1(nz, n)];
    }
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++)
        for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++)
            dttf_v[IX1(nz, n)] = dttf_v[IX1(nz, n)] + (flux_v[IXN(nz, n)] - flux_v[IXN(nz + 1, n)]) * dt /
                                                          m->areasvol[IXN(nz, n)];
    OMP_FOR
    for (int edge = 0; edge < m->edge2D; edge++) {
        int n1 = m->edges[2 * edge], n2 = m->edges[2 * edge + 1], nu12, nl12;
        edge_scatter_range(m, edge, &nu12, &nl12);
        LOCK(n1);
        for (int nz = nu12; nz <= nl12; nz++)
            dttf_h[IX1(nz, n1)] = dttf_h[IX1(nz, n1)] + flux_h[IX1(nz, edge)] * dt / m->areasvol[IXN(nz, n1)];
        UNLOCK(n1);
        LOCK(n2);
        for (int nz = nu12; nz <= nl12; nz++)
            dttf_h[IX1(nz, n2)] = dttf_h[IX1(nz, n2)] - flux_h[IX1(nz, edge)] * dt / m->areasvol[IXN(nz, n2)];
        UNLOCK(n2);
    }
}

/* ========================================================================== */
/* do_oce_adv_tra (src/oce_adv_tra_driver.F90:46-490)                          */
/* ========================================================================== */
int or_do_oce_adv_tra(const or_mesh *m, double dt, const double *vel, const double *W, const double *WI,
                      const double *WE, const or_tra_cfg *c, const double *ttf, const double *ttfAB,
                      or_work *w) {
    const int NL = m->nl, L1 = NL - 1;
    locks_ensure(m->nod2D);
    if (c->hor < 0 || c->hor > 2 || c->ver < 0 || c->ver > 3) return 1;
    double *fct_LO = w->fct_LO, *afh = w->adv_flux_hor, *afv = w->adv_flux_ver;
    if (c->lim_fct) {
        or_adv_tra_hor_upw1(m, vel, ttf, afh, 1);
        OMP_FOR
        for (long i = 0; i < (long)L1 * m->nod2D; i++) fct_LO[i] = 0.0;
        OMP_FOR
        for (int e = 0; e < m->edge2D; e++) {
            int n1 = m->edges[2 * e], n2 = m->edges[2 * e + 1], nu12, nl12;
            edge_scatter_range(m, e, &nu12, &nl12);
            LOCK(n1);
            for (int nz = nu12; nz <= nl12; nz++) fct_LO[IX1(nz, n1)] = fct_LO[IX1(nz, n1)] + afh[IX1(nz, e)];
            UNLOCK(n1);
            LOCK(n2);
            for (int nz = nu12; nz <= nl12; nz++) fct_LO[IX1(nz, n2)] = fct_LO[IX1(nz, n2)] - afh[IX1(nz, e)];
            UNLOCK(n2);
        }
        or_adv_tra_ver_upw1(m, WE, ttf, afv, 1);
        OMP_FOR
        for (int n = 0; n < m->nod2D; n++)
            for (int nz = m->ulevels_nod2D[n]; nz <= m->nlevels_nod2D[n] - 1; nz++)
                fct_LO[IX1(nz, n)] = (ttf[IX1(nz, n)] * m->hnode[IX1(nz, n)] +
                                      (fct_LO[IX1(nz, n)] + (afv[IXN(nz, n)] - afv[IXN(nz + 1, n)])) * dt /
                                          m->areasvol[IXN(nz, n)]) /
                                     m->hnode_new[IX1(nz, n)];
        if (c->wsplit) {
            /* w split (:323-334): the implicit part w_i advects LO implicitly; the LO part of
             * the antidiffusive vertical flux is the upwind flux of the full w */
            or_adv_tra_vert_impl(m, dt, WI, fct_LO);
            or_adv_tra_ver_upw1(m, W, ttf, afv, 1);
        }
    }
    int zero = c->lim_fct ? 0 : 1;
    if (c->hor == OR_HOR_MUSCL)
        or_adv_tra_hor_muscl(m, vel, ttfAB, c->ph, afh, w->edge_up_dn_grad, w->nboundary_lay, zero);
    else if (c->hor == OR_HOR_MFCT)
        or_adv_tra_hor_mfct(m, vel, ttfAB, c->ph, afh, w->edge_up_dn_grad, zero);
    else
        or_adv_tra_hor_upw1(m, vel, ttfAB, afh, zero);
    const double *pw = c->lim_fct ? W : WE;
    if (c->ver == OR_VER_QR4C)
        or_adv_tra_ver_qr4c(m, pw, ttfAB, c->pv, afv, zero);
    else if (c->ver == OR_VER_CDIFF)
        or_adv_tra_ver_cdiff(m, pw, ttfAB, afv, zero);
    else if (c->ver == OR_VER_PPM)
        or_adv_tra_vert_ppm(m, dt, pw, ttfAB, afv, zero);
    else
        or_adv_tra_ver_upw1(m, pw, ttfAB, afv, zero);
    if (c->lim_fct) {
        or_oce_tra_adv_fct(m, dt, ttf, fct_LO, afh, afv, w);
        or_oce_tra_adv_flux2dtracer(m, dt, w->del_ttf_advhoriz, w->del_ttf_advvert, afh, afv, 1, ttf, fct_LO);
    } else {
        or_oce_tra_adv_flux2dtracer(m, dt, w->del_ttf_advhoriz, w->del_ttf_advvert, afh, afv, 0, NULL, NULL);
    }
    return 0;
}

/* ========================================================================== */
/* diff_ver_part_impl_ale (src/oce_ale_tracer.F90:907-1435)                    */
/* ========================================================================== */
void or_diff_ver_part_impl_ale(const or_mesh *m, double dt, const double *Kv, const double *bc_surf,
                               double *values) {
    or_diff_ver_part_impl_ale_w(m, dt, Kv, bc_surf, NULL, 0, values);
}

void or_diff_ver_part_impl_ale_w(const or_mesh *m, double dt, const double *Kv, const double *bc_surf,
                                 const double *WI, int do_wimpl, double *values) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double a[NL + 1], b[NL + 1], c[NL + 1], tr[NL + 1], cp[NL + 1], tp[NL + 1];
        double zbar_n[NL + 1], Z_n[NL + 1];
        for (int k = 0; k <= NL; k++) { a[k] = b[k] = c[k] = tr[k] = tp[k] = cp[k] = 0.0; zbar_n[k] = 0.0; Z_n[k] = 0.0; }
        const double *hn = &m->hnode_new[IX1(1, n)] - 1;   /* hn[nz], nz 1-based */
        const double *ar = &m->area[IXN(1, n)] - 1;
        const double *av = &m->areasvol[IXN(1, n)] - 1;
        const double *kv = &Kv[IXN(1, n)] - 1;
        double *T = &values[IX1(1, n)] - 1;
        int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        zbar_n[nzmax] = m->zbar_n_bot[n];
        Z_n[nzmax - 1] = zbar_n[nzmax] + hn[nzmax - 1] / 2.0;
        for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
            zbar_n[nz] = zbar_n[nz + 1] + hn[nz];
            Z_n[nz - 1] = zbar_n[nz] + hn[nz - 1] / 2.0;
        }
        zbar_n[nzmin] = zbar_n[nzmin + 1] + hn[nzmin];
        int nz = nzmin;
        double zinv2 = 1.0 / (Z_n[nz] - Z_n[nz + 1]);
        double zinv = 1.0 * dt;
        const double *wi = WI ? &WI[IXN(1, n)] - 1 : NULL;
        double v_adv;
        a[nz] = 0.0;
        c[nz] = -(kv[nz + 1] * zinv2 * zinv * ar[nz + 1] / av[nz]);
        b[nz] = -c[nz] + hn[nz];
        if (do_wimpl) { /* implicit part of the split vertical velocity (:1134-1147) */
            v_adv = zinv * (ar[nz] / av[nz]);
            b[nz] = b[nz] + wi[nz] * v_adv;
            v_adv = zinv * ar[nz + 1] / av[nz];
            b[nz] = b[nz] - fmin(0.0, wi[nz + 1]) * v_adv;
            c[nz] = c[nz] - fmax(0.0, wi[nz + 1]) * v_adv;
        }
        double zinv1 = zinv2;
        for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
            zinv2 = 1.0 / (Z_n[nz] - Z_n[nz + 1]);
            a[nz] = -(kv[nz] * zinv1 * zinv * (ar[nz] / av[nz]));
            c[nz] = -(kv[nz + 1] * zinv2 * zinv * ar[nz + 1] / av[nz]);
            b[nz] = -a[nz] - c[nz] + hn[nz];
            zinv1 = zinv2;
            if (do_wimpl) { /* :1176-1189 */
                v_adv = zinv * (ar[nz] / av[nz]);
                a[nz] = a[nz] + fmin(0.0, wi[nz]) * v_adv;
                b[nz] = b[nz] + fmax(0.0, wi[nz]) * v_adv;
                v_adv = zinv * ar[nz + 1] / av[nz];
                b[nz] = b[nz] - fmin(0.0, wi[nz + 1]) * v_adv;
                c[nz] = c[nz] - fmax(0.0, wi[nz + 1]) * v_adv;
            }
        }
        nz = nzmax - 1;
        zinv = 1.0 * dt;
        a[nz] = -(kv[nz] * zinv1 * zinv * (ar[nz] / av[nz]));
        c[nz] = 0.0;
        b[nz] = -a[nz] + hn[nz];
        if (do_wimpl) { /* :1207-1216 */
            v_adv = zinv * (ar[nz] / av[nz]);
            a[nz] = a[nz] + fmin(0.0, wi[nz]) * v_adv;
            b[nz] = b[nz] + fmax(0.0, wi[nz]) * v_adv;
        }
        nz = nzmin;
        double dz = hn[nz];
        tr[nz] = -((b[nz] - dz) * T[nz]) - c[nz] * T[nz + 1];
        for (nz = nzmin + 1; nz <= nzmax - 2; nz++) {
            dz = hn[nz];
            tr[nz] = -(a[nz] * T[nz - 1]) - (b[nz] - dz) * T[nz] - c[nz] * T[nz + 1];
        }
        nz = nzmax - 1;
        dz = hn[nz];
        tr[nz] = -(a[nz] * T[nz - 1]) - (b[nz] - dz) * T[nz];
        tr[nzmin] = tr[nzmin] + bc_surf[n];
        cp[nzmin] = c[nzmin] / b[nzmin];
        tp[nzmin] = tr[nzmin] / b[nzmin];
        for (nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            double mm = b[nz] - cp[nz - 1] * a[nz];
            cp[nz] = c[nz] / mm;
            tp[nz] = (tr[nz] - tp[nz - 1] * a[nz]) / mm;
        }
        tr[nzmax - 1] = tp[nzmax - 1];
        for (nz = nzmax - 2; nz >= nzmin; nz--) tr[nz] = tp[nz] - cp[nz] * tr[nz + 1];
        for (nz = nzmin; nz <= nzmax - 1; nz++) T[nz] = T[nz] + tr[nz];
    }
}

/* ========================================================================== */
/* per-tracer body of solve_tracers_ale (src/oce_ale_tracer.F90:303-351,       */
/* 743-772)                                                                    */
/* ========================================================================== */
/* ========================================================================== */
/* diffusion parts of diff_tracers_ale (src/oce_ale_tracer.F90:560-772)        */
/* ========================================================================== */
/* The isoneutral (Redi) parts take the tapered neutral slopes slope(3, nl-1, nod2D) and the
 * vertical gradient tr_z (nl per node, tracer_gradient_z of the values); slope == NULL is
 * Redi = .false. (isredi = 0): the flux is Kh grad T alone. */
#define SLP(k, nz, n) (slope[3 * IX1(nz, n) + (k)])
void or_diff_part_hor_redi_s(const or_mesh *m, double dt, const double *Ki, const double *slope,
                             const double *tr_xy, const double *tr_z, double *del_ttf) {
    const int NL = m->nl, L1 = NL - 1;
    double rhs1[NL + 1], rhs2[NL + 1];
    for (int edge = 0; edge < m->edge2D; edge++) {
        for (int k = 0; k <= NL; k++) rhs1[k] = rhs2[k] = 0.0;
        const double dX1 = m->edge_cross_dxdy[4 * (size_t)edge], dY1 = m->edge_cross_dxdy[4 * (size_t)edge + 1];
        double dX2 = 0.0, dY2 = 0.0;
        const int el1 = m->edge_tri[2 * edge], el2 = m->edge_tri[2 * edge + 1];
        const int n1 = m->edges[2 * edge], n2 = m->edges[2 * edge + 1];
        const int nl1 = m->nlevels[el1] - 1, ul1 = m->ulevels[el1];
        int nl2 = 0, ul2 = 0;
        if (el2 >= 0) {
            nl2 = m->nlevels[el2] - 1;
            ul2 = m->ulevels[el2];
            dX2 = m->edge_cross_dxdy[4 * (size_t)edge + 2];
            dY2 = m->edge_cross_dxdy[4 * (size_t)edge + 3];
        }
        int nl12 = nl1 < nl2 ? nl1 : nl2, ul12 = ul1 > ul2 ? ul1 : ul2;
        /* Kh (grad T + slope x mean T_z at the edge's nodes) of one element (segments A/D: el1,
         * B/E: el2, C: mean of both), Tz(j) = (tr_z(nz) + tr_z(nz+1)) / 2 at node j */
#define KH(nz) ((Ki[IX1(nz, n1)] + Ki[IX1(nz, n2)]) / 2.0)
#define TXY(k, nz, el) (tr_xy[2 * IX1(nz, el) + (k)])
#define FLUX(nz, Tx, Ty, Fx, Fy)                                                                          \
    do {                                                                                                  \
        const double Kh_ = KH(nz);                                                                        \
        if (slope) {                                                                                      \
            const double tz1 = 0.5 * (tr_z[IXN(nz, n1)] + tr_z[IXN(nz + 1, n1)]);                         \
            const double tz2 = 0.5 * (tr_z[IXN(nz, n2)] + tr_z[IXN(nz + 1, n2)]);                         \
            const double sx = (tz1 * SLP(0, nz, n1) + tz2 * SLP(0, nz, n2)) / 2.0;                        \
            const double sy = (tz1 * SLP(1, nz, n1) + tz2 * SLP(1, nz, n2)) / 2.0;                        \
            Fx = Kh_ * ((Tx) + sx);                                                                       \
            Fy = Kh_ * ((Ty) + sy);                                                                       \
        } else {                                                                                          \
            Fx = Kh_ * (Tx);                                                                              \
            Fy = Kh_ * (Ty);                                                                              \
        }                                                                                                 \
    } while (0)
        double Fx, Fy;
        for (int nz = ul1; nz <= ul12 - 1; nz++) { /* (A) */
            double dz = m->helem[IX1(nz, el1)];
            FLUX(nz, TXY(0, nz, el1), TXY(1, nz, el1), Fx, Fy);
            double cc = (-dX1 * Fy + dY1 * Fx) * dz;
            rhs1[nz] = rhs1[nz] + cc;
            rhs2[nz] = rhs2[nz] - cc;
        }
        if (ul2 > 0)
            for (int nz = ul2; nz <= ul12 - 1; nz++) { /* (B) */
                double dz = m->helem[IX1(nz, el2)];
                FLUX(nz, TXY(0, nz, el2), TXY(1, nz, el2), Fx, Fy);
                double cc = (dX2 * Fy - dY2 * Fx) * dz;
                rhs1[nz] = rhs1[nz] + cc;
                rhs2[nz] = rhs2[nz] - cc;
            }
        for (int nz = ul12; nz <= nl12; nz++) { /* (C) */
            double dz = (m->helem[IX1(nz, el1)] + m->helem[IX1(nz, el2)]) / 2.0;
            double Tx = 0.5 * (TXY(0, nz, el1) + TXY(0, nz, el2)), Ty = 0.5 * (TXY(1, nz, el1) + TXY(1, nz, el2));
            FLUX(nz, Tx, Ty, Fx, Fy);
            double cc = ((dX2 - dX1) * Fy - (dY2 - dY1) * Fx) * dz;
            rhs1[nz] = rhs1[nz] + cc;
            rhs2[nz] = rhs2[nz] - cc;
        }
        for (int nz = nl12 + 1; nz <= nl1; nz++) { /* (D) */
            double dz = m->helem[IX1(nz, el1)];
            FLUX(nz, TXY(0, nz, el1), TXY(1, nz, el1), Fx, Fy);
            double cc = (-dX1 * Fy + dY1 * Fx) * dz;
            rhs1[nz] = rhs1[nz] + cc;
            rhs2[nz] = rhs2[nz] - cc;
        }
        for (int nz = nl12 + 1; nz <= nl2; nz++) { /* (E) */
            double dz = m->helem[IX1(nz, el2)];
            FLUX(nz, TXY(0, nz, el2), TXY(1, nz, el2), Fx, Fy);
            double cc = (dX2 * Fy - dY2 * Fx) * dz;
            rhs1[nz] = rhs1[nz] + cc;
            rhs2[nz] = rhs2[nz] - cc;
        }
#undef KH
#undef TXY
#undef FLUX
        nl12 = nl1 > nl2 ? nl1 : nl2;
        ul12 = ul1;
        if (ul2 > 0) ul12 = ul1 < ul2 ? ul1 : ul2;
        for (int nz = ul12; nz <= nl12; nz++) {
            del_ttf[IX1(nz, n1)] = del_ttf[IX1(nz, n1)] + rhs1[nz] * dt / m->areasvol[IXN(nz, n1)];
            del_ttf[IX1(nz, n2)] = del_ttf[IX1(nz, n2)] + rhs2[nz] * dt / m->areasvol[IXN(nz, n2)];
        }
    }
}

void or_diff_part_hor_redi(const or_mesh *m, double dt, const double *Ki, const double *tr_xy, double *del_ttf) {
    or_diff_part_hor_redi_s(m, dt, Ki, NULL, tr_xy, NULL, del_ttf);
}

/* diff_ver_part_redi_expl (src/oce_ale_tracer.F90:1439-1518): the horizontal part of the
 * isoneutral flux projected on the vertical.  Node gradients tr_xynodes = sum over the node's
 * elements wet at nz of tr_xy elem_area, / 3 / areasvol (:1470-1487); depths zbar_n / z_n of the
 * column from hnode, bottom up from zbar_n_bot (:1496-1503); interface flux vd(nz) of the two
 * layers around it weighted by their half thicknesses (:1506-1511); increment
 * (vd(nz) - vd(nz+1)) dt / areasvol (:1512-1514). */
void or_diff_ver_part_redi_expl(const or_mesh *m, double dt, const double *Ki, const double *slope,
                                const double *tr_xy, double *del_ttf) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double gx[NL + 1], gy[NL + 1], vd[NL + 2], zbar_n[NL + 2], z_n[NL + 1];
        const int nl1 = m->nlevels_nod2D[n] - 1, ul1 = m->ulevels_nod2D[n];
        for (int nz = ul1; nz <= nl1; nz++) {
            double tx = 0.0, ty = 0.0;
            for (int k = m->nod_in_elem2D_ptr[n]; k < m->nod_in_elem2D_ptr[n + 1]; k++) {
                const int elem = m->nod_in_elem2D[k];
                if (nz <= m->nlevels[elem] - 1 && nz >= m->ulevels[elem]) {
                    tx = tx + tr_xy[2 * IX1(nz, elem)] * m->elem_area[elem];
                    ty = ty + tr_xy[2 * IX1(nz, elem) + 1] * m->elem_area[elem];
                }
            }
            gx[nz] = tx / 3.0 / m->areasvol[IXN(nz, n)];
            gy[nz] = ty / 3.0 / m->areasvol[IXN(nz, n)];
        }
        for (int k = 0; k <= NL + 1; k++) vd[k] = zbar_n[k] = 0.0;
        for (int k = 0; k <= NL; k++) z_n[k] = 0.0;
        const double *hn = &m->hnode[IX1(1, n)] - 1;
        zbar_n[nl1 + 1] = m->zbar_n_bot[n];
        z_n[nl1] = zbar_n[nl1 + 1] + hn[nl1] / 2.0;
        for (int nz = nl1; nz >= ul1 + 1; nz--) {
            zbar_n[nz] = zbar_n[nz + 1] + hn[nz];
            z_n[nz - 1] = zbar_n[nz] + hn[nz - 1] / 2.0;
        }
        for (int nz = ul1 + 1; nz <= nl1; nz++) {
            double v = (z_n[nz - 1] - zbar_n[nz]) * (SLP(0, nz - 1, n) * gx[nz - 1] + SLP(1, nz - 1, n) * gy[nz - 1]) *
                       Ki[IX1(nz - 1, n)];
            v = v + (zbar_n[nz] - z_n[nz]) * (SLP(0, nz, n) * gx[nz] + SLP(1, nz, n) * gy[nz]) * Ki[IX1(nz, n)];
            vd[nz] = v / (z_n[nz - 1] - z_n[nz]) * m->area[IXN(nz, n)];
        }
        for (int nz = ul1; nz <= nl1; nz++)
            del_ttf[IX1(nz, n)] = del_ttf[IX1(nz, n)] + (vd[nz] - vd[nz + 1]) * dt / m->areasvol[IXN(nz, n)];
    }
}

/* K_33 = Kv + Kd s^2 of diff_ver_part_impl_ale with Redi (src/oce_ale_tracer.F90:1099-1204): at
 * interface nz of a column (nzmin < nz < nzmax), with zbar_n / Z_n from hnode_new bottom up,
 * Ty = (zbar_n(nz) - Z_n(nz)) / dZ s3(nz-1)^2 Ki(nz-1) + (Z_n(nz-1) - zbar_n(nz)) / dZ s3(nz)^2
 * Ki(nz), 1/dZ = 1 / (Z_n(nz-1) - Z_n(nz)) (Ty of the layer below = Ty1 of the layer above);
 * other interfaces keep Kv.  The implicit solve with K33 in place of Kv is the reference's. */
void or_redi_k33(const or_mesh *m, const double *Kv, const double *Ki, const double *slope, double *K33) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double zbar_n[NL + 1], Z_n[NL + 1];
        for (int k = 0; k <= NL; k++) zbar_n[k] = Z_n[k] = 0.0;
        for (int nz = 1; nz <= NL; nz++) K33[IXN(nz, n)] = Kv[IXN(nz, n)];
        const double *hn = &m->hnode_new[IX1(1, n)] - 1;
        const int nzmax = m->nlevels_nod2D[n], nzmin = m->ulevels_nod2D[n];
        zbar_n[nzmax] = m->zbar_n_bot[n];
        Z_n[nzmax - 1] = zbar_n[nzmax] + hn[nzmax - 1] / 2.0;
        for (int nz = nzmax - 1; nz >= nzmin + 1; nz--) {
            zbar_n[nz] = zbar_n[nz + 1] + hn[nz];
            Z_n[nz - 1] = zbar_n[nz] + hn[nz - 1] / 2.0;
        }
        for (int nz = nzmin + 1; nz <= nzmax - 1; nz++) {
            const double zinv = 1.0 / (Z_n[nz - 1] - Z_n[nz]);
            const double sa = SLP(2, nz - 1, n), sb = SLP(2, nz, n);
            const double Ty = (zbar_n[nz] - Z_n[nz]) * zinv * (sa * sa) * Ki[IX1(nz - 1, n)] +
                              (Z_n[nz - 1] - zbar_n[nz]) * zinv * (sb * sb) * Ki[IX1(nz, n)];
            K33[IXN(nz, n)] = Kv[IXN(nz, n)] + Ty;
        }
    }
}
#undef SLP

void or_diff_ver_part_expl_ale(const or_mesh *m, double dt, const double *Kv, const double *flux_surf,
                               const double *values, double *del_ttf) {
    const int NL = m->nl, L1 = NL - 1;
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        double vd[NL + 1];
        for (int k = 0; k <= NL; k++) vd[k] = 0.0;
        const int nl1 = m->nlevels_nod2D[n] - 1, ul1 = m->ulevels_nod2D[n];
        vd[ul1] = flux_surf ? flux_surf[n] : 0.0;
        for (int nz = ul1 + 1; nz <= nl1; nz++) {
            double zinv1 = 1.0 / (m->Z_3d_n[IX1(nz - 1, n)] - m->Z_3d_n[IX1(nz, n)]);
            vd[nz] = Kv[IXN(nz, n)] * (values[IX1(nz - 1, n)] - values[IX1(nz, n)]) * zinv1 * m->area[IXN(nz, n)];
        }
        for (int nz = ul1; nz <= nl1 - 1; nz++)
            del_ttf[IX1(nz, n)] = del_ttf[IX1(nz, n)] + (vd[nz] - vd[nz + 1]) /
                                                            (m->zbar_3d_n[IXN(nz, n)] - m->zbar_3d_n[IXN(nz + 1, n)]) *
                                                            dt / m->areasvol[IXN(nz, n)];
        del_ttf[IX1(nl1, n)] = del_ttf[IX1(nl1, n)] +
                               (vd[nl1] / (m->zbar_3d_n[IXN(nl1, n)] - m->zbar_3d_n[IXN(nl1 + 1, n)])) * dt /
                                   m->areasvol[IXN(nl1, n)];
    }
}

int or_tracer_step(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                   const double *WI, const double *WE, const double *Kv, const double *bc_surf,
                   double *values, double *valuesAB, double *valuesold, or_work *w) {
    return or_tracer_step_ex(m, c, dt, vel, W, WI, WE, Kv, bc_surf, NULL, values, valuesAB, valuesold, w);
}

int or_tracer_step_ex(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                      const double *WI, const double *WE, const double *Kv, const double *bc_surf, const double *Ki,
                      double *values, double *valuesAB, double *valuesold, or_work *w) {
    return or_tracer_step_redi(m, c, dt, vel, W, WI, WE, Kv, bc_surf, Ki, NULL, values, valuesAB, valuesold, w);
}

int or_tracer_step_redi(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                        const double *WI, const double *WE, const double *Kv, const double *bc_surf, const double *Ki,
                        const double *slope, double *values, double *valuesAB, double *valuesold, or_work *w) {
    if (slope && !Ki) return 3;
    const int L1 = m->nl - 1;
    if (c->ab_order != 2 && c->ab_order != 3) return 2;
    or_init_tracers_AB(m, c, values, valuesAB, valuesold, w);
    int rc = or_do_oce_adv_tra(m, dt, vel, W, WI, WE, c, values, valuesAB, w);
    if (rc) return rc;
    const size_t N = (size_t)L1 * (size_t)m->nod2D;
    OMP_FOR
    for (long i = 0; i < (long)N; i++) w->del_ttf[i] = w->del_ttf[i] + w->del_ttf_advhoriz[i] + w->del_ttf_advvert[i];
    /* diff_tracers_ale (:595-607): horizontal diffusion, then the explicit vertical one */
    if (Ki) or_diff_part_hor_redi_s(m, dt, Ki, slope, w->tr_xy, w->tr_z, w->del_ttf);
    if (!c->i_vert_diff) or_diff_ver_part_expl_ale(m, dt, Kv, bc_surf, values, w->del_ttf);
    /* :623 */
    if (slope) or_diff_ver_part_redi_expl(m, dt, Ki, slope, w->tr_xy, w->del_ttf);
    OMP_FOR
    for (int n = 0; n < m->nod2D; n++) {
        int nzmax = m->nlevels_nod2D[n] - 1, nzmin = m->ulevels_nod2D[n];
        for (int nz = nzmin; nz <= nzmax; nz++) {
            size_t i = IX1(nz, n);
            w->del_ttf[i] = w->del_ttf[i] + values[i] * (m->hnode[i] - m->hnode_new[i]);
            values[i] = values[i] + w->del_ttf[i] / m->hnode_new[i];
        }
    }
    /* the w_i part goes into the implicit solve only without the limiter (:961) */
    if (c->i_vert_diff) {
        double *K33 = NULL;
        if (slope) {
            K33 = (double *)malloc(sizeof(double) * (size_t)m->nl * (size_t)m->nod2D);
            if (!K33) return 4;
            or_redi_k33(m, Kv, Ki, slope, K33);
        }
        or_diff_ver_part_impl_ale_w(m, dt, K33 ? K33 : Kv, bc_surf, WI, c->wsplit && !c->lim_fct, values);
        free(K33);
    }
    return 0;
}

/* ========================================================================== */
/* tail of solve_tracers_ale (src/oce_ale_tracer.F90:353-375, 497-525)         */
/* ========================================================================== */
static const double kDecay14 = 3.8561e-12, kDecay39 = 8.1708e-11; /* src/mod_transit.F90:49-50 */

/* relax_to_clim (src/oce_tracer_mod.F90:236-298) for tracer values of ID id */
static void relax_to_clim(const or_mesh *m, double dt, int id, double clim_relax, const double *relax2clim,
                          const double *Tclim, const double *Sclim, double *values) {
    const int L1 = m->nl - 1;
    const double *clim = id == 1 ? Tclim : (id == 2 ? Sclim : NULL);
    if (!(clim_relax > 1.0e-8) || !clim) return;
    for (int n = 0; n < m->nod2D; n++) {
        int nzmin = m->ulevels_nod2D[n], nzmax = m->nlevels_nod2D[n];
        for (int nz = nzmin; nz <= nzmax - 1; nz++) {
            size_t i = IX1(nz, n);
            values[i] = values[i] + relax2clim[n] * dt * (clim[i] - values[i]);
        }
    }
}

/* relax_zonal_temp (src/toy_channel_soufflet.F90:91-121) */
static void relax_zonal_temp(const or_mesh *m, double dt, const or_tail_cfg *tc, const double *Tclim,
                             const double *ztem, double *values) {
    const int L1 = m->nl - 1;
    for (int n = 0; n < m->nod2D; n++) {
        double yy = m->coord_nod2D[2 * n + 1] - tc->lat0, a = 0.0;
        int nn, nn1;
        if (yy < tc->dy / 2.0) {
            nn = 1;
            nn1 = 1;
        } else {
            nn = (int)floor(yy / tc->dy - 0.5) + 1;
            if (nn > tc->nbins) nn = tc->nbins;  /* outside the table (the reference reads past it) */
            nn1 = nn + 1;
            if (nn1 > tc->nbins) nn1 = nn;
            a = yy / tc->dy + 0.5 - nn;
        }
        for (int nz = 1; nz <= m->nlevels_nod2D[n] - 1; nz++) {
            double Tzon = (1.0 - a) * ztem[(nz - 1) + (size_t)(nn - 1) * L1] + a * ztem[(nz - 1) + (size_t)(nn1 - 1) * L1];
            size_t i = IX1(nz, n);
            values[i] = values[i] + dt * tc->tau_inv * (Tclim[i] - Tzon);
        }
    }
}

void or_tracer_tail(const or_mesh *m, int ntr, const int *ids, double dt, const or_tail_cfg *tc,
                    const double *relax2clim, const double *Tclim, const double *Sclim, const double *ztem,
                    double **values) {
    const int L1 = m->nl - 1;
    const size_t N = (size_t)L1 * (size_t)m->nod2D;
    for (int t = 0; t < ntr; t++) {
        /* radioactive decay of the whole field (:355-356) */
        if (ids[t] == 14 || ids[t] == 39) {
            const double f = exp(-(ids[t] == 14 ? kDecay14 : kDecay39) * dt);
            for (size_t i = 0; i < N; i++) values[t][i] = values[t][i] * f;
        }
        if (tc->zonal_relax) relax_zonal_temp(m, dt, tc, Tclim, ztem, values[0]);
        else relax_to_clim(m, dt, ids[t], tc->clim_relax, relax2clim, Tclim, Sclim, values[t]);
    }
    for (int k = 0; k < 2; k++) {
        int t = k == 0 ? tc->salt_index : tc->age_index;
        if (t < 0 || t >= ntr) continue;
        for (int n = 0; n < m->nod2D; n++) {
            int nzmax = m->nlevels_nod2D[n] - 1, nzmin = m->ulevels_nod2D[n];
            for (int nz = nzmin; nz <= nzmax; nz++) {
                double *v = &values[t][IX1(nz, n)];
                if (k == 0) {
                    if (*v > 45.0) *v = 45.0;
                    if (*v < 3.0) *v = 3.0;
                } else if (*v < 0.0) {
                    *v = 0.0;
                }
            }
        }
    }
}
