/*
 * tracer_oracle.h -- FP64 CPU restatement of FESOM2's tracer-transport step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the CUDA path: only the
 * test suite, the smoke test and the benchmark's CPU-baseline leg may load it.
 * The product library never links or calls it.
 *
 * Parity status: the reference (Fortran + MPI) cannot be compiled in this
 * image and its own tests hold no golden vectors for this path, so the
 * restatement is pinned only by the hand-derived known-answer tests under
 * tests/golden/ ("parity unpinned" against the reference binary itself).
 *
 * Layout: every array keeps the reference's Fortran layout a(level, entity),
 * i.e. index [entity * ld + (level - 1)] with ld = nl-1 or nl.  Entity
 * indices are 0-based; edge_tri[2*e+1] < 0 marks a boundary edge.  Level
 * counts (nlevels, ulevels, ...) keep the reference's 1-based values.
 */
#ifndef FESOM_TRACER_ORACLE_H
#define FESOM_TRACER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_mesh {
    int nod2D, elem2D, edge2D, nl;
    const int *elem2D_nodes;       /* 3*T2 */
    const int *edges;              /* 2*E2 */
    const int *edge_tri;           /* 2*E2 */
    const int *nod_in_elem2D_ptr;  /* N2+1 */
    const int *nod_in_elem2D;      /* nnz, ascending element order per node */
    const int *nlevels, *ulevels;                 /* T2 */
    const int *nlevels_nod2D, *ulevels_nod2D;     /* N2 */
    const int *nlevels_nod2D_min, *ulevels_nod2D_max;
    const double *coord_nod2D;     /* 2*N2 */
    const double *elem_area, *elem_cos;           /* T2 */
    const double *edge_dxdy;       /* 2*E2 */
    const double *edge_cross_dxdy; /* 4*E2 */
    const double *gradient_sca;    /* 6*T2 */
    const double *area, *areasvol; /* nl*N2 */
    const double *hnode, *hnode_new; /* (nl-1)*N2 */
    const double *helem;           /* (nl-1)*T2 */
    const double *Z_3d_n;          /* (nl-1)*N2 */
    const double *zbar_3d_n;       /* nl*N2 */
    const double *zbar_n_bot;      /* N2 */
    double cyclic_length;
} or_mesh;

/* scheme tuple of T_TRACER_DATA (src/MOD_TRACER.F90:10-27) */
enum { OR_HOR_MUSCL = 0, OR_HOR_MFCT = 1, OR_HOR_UPW1 = 2 };
enum { OR_VER_QR4C = 0, OR_VER_UPW1 = 1, OR_VER_CDIFF = 2, OR_VER_PPM = 3 };
typedef struct or_tra_cfg {
    int hor, ver;
    int lim_fct;       /* 1: 'FCT', 0: no limiter */
    double ph, pv;     /* tra_adv_ph / tra_adv_pv */
    int ab_order;      /* 2 or 3 */
    int i_vert_diff;   /* implicit vertical diffusion on/off */
    int wsplit;        /* dynamics%use_wsplit: vertical velocity split into w_e + w_i */
} or_tra_cfg;

/* T_TRACER_WORK (src/MOD_TRACER.F90:30-72) plus the module arrays tr_xy/tr_z */
typedef struct or_work {
    int *nboundary_lay;        /* N2 */
    int *edge_up_dn_tri;       /* 2*E2, -1 = none */
    double *edge_up_dn_grad;   /* 4*(nl-1)*E2 (also the FCT AUX array) */
    double *tr_xy;             /* 2*(nl-1)*T2 */
    double *tr_z;              /* nl*N2 */
    double *fct_LO;            /* (nl-1)*N2 */
    double *adv_flux_hor;      /* (nl-1)*E2 */
    double *adv_flux_ver;      /* nl*N2 */
    double *fct_ttf_max, *fct_ttf_min, *fct_plus, *fct_minus; /* (nl-1)*N2 */
    double *tvert_max, *tvert_min;                           /* (nl-1)*N2 */
    double *del_ttf, *del_ttf_advhoriz, *del_ttf_advvert;    /* (nl-1)*N2 */
} or_work;

/* threads: 1 = serial "exact" mode (edge scatters in ascending edge order);
 * >1 = OpenMP mode with per-node locks around scatters, as the reference's
 * default OpenMP build (nondeterministic at round-off level). */
void or_set_threads(int nthreads);
int or_get_threads(void);

/* muscl_adv_init + find_up_downwind_triangles (src/oce_muscl_adv.F90:32-352) */
void or_muscl_adv_init(const or_mesh *m, or_work *w);

/* init_tracers_AB (src/oce_tracer_mod.F90:13-143) incl. gradients and fill_up_dn_grad */
void or_init_tracers_AB(const or_mesh *m, const or_tra_cfg *c, double *values, double *valuesAB,
                        double *valuesold, or_work *w);
void or_tracer_gradient_elements(const or_mesh *m, const double *ttf, double *tr_xy);
void or_tracer_gradient_z(const or_mesh *m, const double *ttf, double *tr_z);
void or_fill_up_dn_grad(const or_mesh *m, or_work *w);

/* individual flux routines (o_init_zero as in the reference) */
void or_adv_tra_hor_upw1(const or_mesh *m, const double *vel, const double *ttf, double *flux, int init_zero);
void or_adv_tra_hor_muscl(const or_mesh *m, const double *vel, const double *ttf, double num_ord, double *flux,
                          const double *edge_up_dn_grad, const int *nboundary_lay, int init_zero);
void or_adv_tra_hor_mfct(const or_mesh *m, const double *vel, const double *ttf, double num_ord, double *flux,
                         const double *edge_up_dn_grad, int init_zero);
void or_adv_tra_ver_upw1(const or_mesh *m, const double *W, const double *ttf, double *flux, int init_zero);
void or_adv_tra_ver_cdiff(const or_mesh *m, const double *W, const double *ttf, double *flux, int init_zero);
void or_adv_tra_vert_ppm(const or_mesh *m, double dt, const double *W, const double *ttf, double *flux,
                         int init_zero);
void or_adv_tra_vert_impl(const or_mesh *m, double dt, const double *W, double *ttf);
void or_adv_tra_ver_qr4c(const or_mesh *m, const double *W, const double *ttf, double num_ord, double *flux,
                         int init_zero);
void or_oce_tra_adv_fct(const or_mesh *m, double dt, const double *ttf, const double *lo, double *adf_h,
                        double *adf_v, or_work *w);
void or_oce_tra_adv_flux2dtracer(const or_mesh *m, double dt, double *dttf_h, double *dttf_v,
                                 const double *flux_h, const double *flux_v, int use_lo, const double *ttf,
                                 const double *lo);

/* do_oce_adv_tra (src/oce_adv_tra_driver.F90:46-490), use_wsplit = .false. */
int or_do_oce_adv_tra(const or_mesh *m, double dt, const double *vel, const double *W, const double *WI,
                      const double *WE, const or_tra_cfg *c, const double *ttf, const double *ttfAB,
                      or_work *w);

/* diff_ver_part_impl_ale (src/oce_ale_tracer.F90:907-1435), Redi/KPP/SW/icebergs off;
 * bc_surf(n) is the bc_surface() value added at nzmin. */
void or_diff_ver_part_impl_ale(const or_mesh *m, double dt, const double *Kv, const double *bc_surf,
                               double *values);
/* the same with the implicit advection by the w_i part of a split vertical velocity
 * (do_wimpl: split velocity and no limiter, :961, 1134-1216) */
void or_diff_ver_part_impl_ale_w(const or_mesh *m, double dt, const double *Kv, const double *bc_surf,
                                 const double *WI, int do_wimpl, double *values);

/* diff_part_hor_redi (src/oce_ale_tracer.F90:1526-1689) with Redi off: edge fluxes of
 * Ki-weighted element gradients tr_xy, scattered into del_ttf in ascending edge order. */
void or_diff_part_hor_redi(const or_mesh *m, double dt, const double *Ki, const double *tr_xy, double *del_ttf);
/* Redi = .true.: the isoneutral parts with the tapered neutral slopes slope(3, nl-1, nod2D)
 * (slope_tapered) as input.  diff_part_hor_redi with the slope terms (tr_z: nl per node,
 * tracer_gradient_z of the values); diff_ver_part_redi_expl (src/oce_ale_tracer.F90:1439-1518);
 * K33 (nl per node) = Kv + Kd s^2 of diff_ver_part_impl_ale's Redi terms (:1099-1204), the
 * diffusivity of the implicit solve. */
void or_diff_part_hor_redi_s(const or_mesh *m, double dt, const double *Ki, const double *slope,
                             const double *tr_xy, const double *tr_z, double *del_ttf);
void or_diff_ver_part_redi_expl(const or_mesh *m, double dt, const double *Ki, const double *slope,
                                const double *tr_xy, double *del_ttf);
void or_redi_k33(const or_mesh *m, const double *Kv, const double *Ki, const double *slope, double *K33);
/* diff_ver_part_expl_ale (src/oce_ale_tracer.F90:841-902): explicit vertical diffusion of
 * values into del_ttf; flux_surf(n) is the surface flux vd_flux(ulevels) (NULL: zero). */
void or_diff_ver_part_expl_ale(const or_mesh *m, double dt, const double *Kv, const double *flux_surf,
                               const double *values, double *del_ttf);

/* The per-tracer body of solve_tracers_ale with the horizontal diffusion of diff_tracers_ale
 * (Ki = NULL: K_hor = 0) and, for tracers without implicit vertical diffusion, the explicit
 * one (bc_surf then holds its surface flux). */
int or_tracer_step_ex(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                      const double *WI, const double *WE, const double *Kv, const double *bc_surf, const double *Ki,
                      double *values, double *valuesAB, double *valuesold, or_work *w);
/* The same with Redi = .true. when slope != NULL (Ki required; returns 3 without it): the slope
 * terms of the horizontal diffusion, diff_ver_part_redi_expl after the explicit vertical part
 * (:623), K33 in the implicit solve. */
int or_tracer_step_redi(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                        const double *WI, const double *WE, const double *Kv, const double *bc_surf, const double *Ki,
                        const double *slope, double *values, double *valuesAB, double *valuesold, or_work *w);

/* The per-tracer body of solve_tracers_ale (src/oce_ale_tracer.F90:303-351):
 * init_tracers_AB, do_oce_adv_tra, del_ttf sum, diff_tracers_ale (T* update,
 * implicit vertical diffusion).  Horizontal (Redi) diffusion is off. */
int or_tracer_step(const or_mesh *m, const or_tra_cfg *c, double dt, const double *vel, const double *W,
                   const double *WI, const double *WE, const double *Kv, const double *bc_surf,
                   double *values, double *valuesAB, double *valuesold, or_work *w);

/* Tail of the tracer loop of solve_tracers_ale (src/oce_ale_tracer.F90:353-375) and of the
 * routine (:497-525): radioactive decay of IDs 14 and 39 (decay constants of
 * src/mod_transit.F90:49-50), relax_to_clim (src/oce_tracer_mod.F90:236-298) or, in the
 * Soufflet channel, relax_zonal_temp of tracer 1 (src/toy_channel_soufflet.F90:91-121) at
 * every tracer iteration, then the salinity clamp to [3, 45] and the age-tracer floor. */
typedef struct or_tail_cfg {
    double clim_relax;
    int salt_index;   /* 0-based, -1: none */
    int age_index;    /* 0-based, -1: none */
    int zonal_relax;  /* 1: relax_zonal_temp of tracer 0 instead of relax_to_clim */
    int nbins;        /* bins of ztem (ztem(nl-1, nbins)) */
    double lat0, dy, tau_inv;
} or_tail_cfg;
void or_tracer_tail(const or_mesh *m, int ntr, const int *ids, double dt, const or_tail_cfg *tc,
                    const double *relax2clim, const double *Tclim, const double *Sclim, const double *ztem,
                    double **values);

#ifdef __cplusplus
}
#endif
#endif
