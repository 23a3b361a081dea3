/*
 * fesom_gpu.h -- C ABI of the GB300 (sm_103a) FESOM2 tracer-transport step.
 *
 * The library replaces, call for call, the tracer-transport routines of
 * FESOM2 (reference paths are relative to the FESOM2 source tree):
 *
 *   fesom_gpu_init_tracers_ab   init_tracers_AB          src/oce_tracer_mod.F90:13-143
 *   fesom_gpu_tracer_gradient_z tracer_gradient_z        src/oce_tracer_mod.F90:192-232
 *   fesom_gpu_adv_tra           do_oce_adv_tra           src/oce_adv_tra_driver.F90:46-490
 *   fesom_gpu_vdiff_impl        diff_ver_part_impl_ale   src/oce_ale_tracer.F90:907-1435
 *   fesom_gpu_tracer_step       body of the tracer loop  src/oce_ale_tracer.F90:280-351
 *                               (init_tracers_AB, do_oce_adv_tra, del_ttf sum,
 *                               diff_tracers_ale's T* update and implicit
 *                               vertical diffusion) for all tracers at once
 *   fesom_gpu_diff_hor          diff_part_hor_redi       src/oce_ale_tracer.F90:1526-1689 (Redi off)
 *   fesom_gpu_diff_hor_redi     diff_part_hor_redi       src/oce_ale_tracer.F90:1526-1689 (Redi on)
 *   fesom_gpu_diff_ver_expl     diff_ver_part_expl_ale   src/oce_ale_tracer.F90:841-902
 *   fesom_gpu_diff_ver_redi_expl diff_ver_part_redi_expl src/oce_ale_tracer.F90:1439-1518
 *   fesom_gpu_redi_k33          K_33 = Kv + Kd s^2 of diff_ver_part_impl_ale with Redi
 *                               src/oce_ale_tracer.F90:1099-1204
 *   fesom_gpu_tracer_tail       tail of solve_tracers_ale src/oce_ale_tracer.F90:353-375, 497-525
 *   fesom_gpu_init              setup of the mesh-derived work arrays:
 *                               oce_adv_tra_fct_init  src/oce_adv_tra_fct.F90:35-67,
 *                               muscl_adv_init        src/oce_muscl_adv.F90:32-352,
 *                               find_levels_min_e2n   src/oce_mesh.F90:1656-1694
 *
 * and adds device-resident stepping (fesom_gpu_state_setup / _forcing_upload /
 * _run_steps, CUDA-graph replay), a host-array FP32 step with the transfers
 * overlapped (fesom_gpu_step_host_f32, group order fesom_gpu_set_host_groups) and a batch of independent meshes
 * (fesom_gpu_batch_*).
 *
 * All arrays are passed by address in the reference's Fortran layout
 * a(level, entity) (column-major, level-contiguous), exactly as the derived
 * types t_mesh / t_tracer / t_dyn hold them, so a Fortran caller passes
 * c_loc() of its arrays with no copy.  An array argument may be a host or a
 * device pointer: the copies inside each call take their direction from the
 * pointer (unified addressing), so a caller whose arrays already live on the
 * GPU (an OpenACC build passing `host_data use_device` addresses) moves nothing
 * over the host link.  fesom_gpu_tracer_device_ptr gives the device-resident
 * state of an FP64 context; fesom_gpu_vdiff_impl_noalloc works on the caller's
 * device arrays in place.
 *
 * Error convention: every entry point returns 0 on success and a FESOM_ERR_*
 * code otherwise (the reference aborts through par_ex on the same conditions);
 * fesom_gpu_last_error() gives a message.  No call blocks without a bound and
 * no kernel traps.
 */
#ifndef FESOM_GPU_H
#define FESOM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FESOM_GPU_ABI_VERSION 1

/* status codes */
#define FESOM_OK 0
#define FESOM_ERR_ARG 1          /* bad argument / null pointer / size mismatch */
#define FESOM_ERR_SCHEME 2       /* unknown advection scheme or limiter */
#define FESOM_ERR_MESH 3         /* mesh fails validation (index out of range, < 2 layers, ...) */
#define FESOM_ERR_CUDA 4         /* a CUDA runtime call failed */
#define FESOM_ERR_NOMEM 5        /* device allocation failed */
#define FESOM_ERR_TIMEOUT 6      /* a bounded wait on the device expired */
#define FESOM_ERR_NUMERIC 7      /* device status word reports NaN/Inf in a result */
#define FESOM_ERR_STATE 8        /* call order violated (e.g. step before forcing upload) */

/* precision of the device-side step */
#define FESOM_PREC_FP64 0        /* plain form: the reference's FP64 arithmetic, bit-for-bit order */
#define FESOM_PREC_FP32 1        /* batched form: FP32 storage/arithmetic, FP64 Thomas solve and sums */

/* tra_adv_hor / tra_adv_ver / tra_adv_lim strings of namelist.tra */
#define FESOM_ADV_HOR_MUSCL 0
#define FESOM_ADV_HOR_MFCT 1
#define FESOM_ADV_HOR_UPW1 2
#define FESOM_ADV_VER_QR4C 0
#define FESOM_ADV_VER_UPW1 1
#define FESOM_ADV_VER_CDIFF 2    /* adv_tra_ver_cdiff, src/oce_adv_tra_ver.F90:635-695 */
#define FESOM_ADV_VER_PPM 3      /* adv_tra_vert_ppm, src/oce_adv_tra_ver.F90:438-631 */
#define FESOM_ADV_LIM_NONE 0
#define FESOM_ADV_LIM_FCT 1

/* device status word bits (fesom_gpu_status) */
#define FESOM_STATUS_NAN 0x1u        /* a non-finite tracer value was produced */
#define FESOM_STATUS_FCT_BOUND 0x2u  /* (FP32 form built with FESOM_FCT_CLAMP=1) an advected value
                                        left its FCT bounds by more than round-off */
#define FESOM_STATUS_INDEX 0x4u      /* a kernel met an index outside its array and skipped it */

/* Per-tracer scheme tuple of T_TRACER_DATA (src/MOD_TRACER.F90:10-27). */
typedef struct fesom_tra_cfg {
    int32_t adv_hor;      /* FESOM_ADV_HOR_* */
    int32_t adv_ver;      /* FESOM_ADV_VER_* */
    int32_t adv_lim;      /* FESOM_ADV_LIM_* */
    int32_t ab_order;     /* 2 or 3 */
    double adv_ph;        /* tra_adv_ph: fourth-order fraction of the horizontal scheme */
    double adv_pv;        /* tra_adv_pv: fourth-order fraction of QR4C */
    int32_t i_vert_diff;  /* 1: implicit vertical diffusion */
    int32_t id;           /* tracer ID (1 = temperature, 2 = salinity, ...), informational */
} fesom_tra_cfg;

/*
 * Mesh description: the t_mesh members the path reads (src/MOD_MESH.F90:22-160),
 * in Fortran layout.  Integer indices are index_base-based (1 for Fortran
 * callers); edge_tri(2,e) <= index_base-1 marks a boundary edge (the reference
 * stores -999).  nod_in_elem2D is the reference's 2-D array (ld_nie, nod2D)
 * with nod_in_elem2D_num(nod2D) valid entries per node.  nboundary_lay and
 * edge_up_dn_tri (t_tracer_work, filled by muscl_adv_init) are optional: when
 * NULL the library computes them as muscl_adv_init does.
 *
 * Thicknesses (hnode, hnode_new, helem, Z_3d_n, zbar_3d_n) change with ALE;
 * fesom_gpu_update_thickness() refreshes them between steps.
 */
typedef struct fesom_mesh_desc {
    int32_t nod2D, elem2D, edge2D, nl;
    int32_t index_base;
    int32_t ld_nie;
    const int32_t *elem2D_nodes;       /* (3, elem2D) */
    const int32_t *edges;              /* (2, edge2D) */
    const int32_t *edge_tri;           /* (2, edge2D) */
    const int32_t *nod_in_elem2D_num;  /* (nod2D) */
    const int32_t *nod_in_elem2D;      /* (ld_nie, nod2D) */
    const int32_t *nlevels, *ulevels;                  /* (elem2D) */
    const int32_t *nlevels_nod2D, *ulevels_nod2D;      /* (nod2D) */
    const int32_t *nlevels_nod2D_min, *ulevels_nod2D_max; /* (nod2D) */
    const double *coord_nod2D;         /* (2, nod2D), rotated lon/lat in radians */
    const double *elem_area, *elem_cos;                /* (elem2D) */
    const double *edge_dxdy;           /* (2, edge2D) */
    const double *edge_cross_dxdy;     /* (4, edge2D) */
    const double *gradient_sca;        /* (6, elem2D) */
    const double *area, *areasvol;     /* (nl, nod2D) */
    const double *hnode, *hnode_new;   /* (nl-1, nod2D) */
    const double *helem;               /* (nl-1, elem2D) */
    const double *Z_3d_n;              /* (nl-1, nod2D) */
    const double *zbar_3d_n;           /* (nl, nod2D) */
    const double *zbar_n_bot;          /* (nod2D) */
    double cyclic_length;
    const int32_t *nboundary_lay;      /* optional (nod2D) */
    const int32_t *edge_up_dn_tri;     /* optional (2, edge2D), <= index_base-1 = none */
} fesom_mesh_desc;

typedef struct fesom_gpu_ctx fesom_gpu_ctx;

/* ---- lifetime ------------------------------------------------------------ */
/* Validates the mesh, builds the node->edge and node->element gather lists
 * (ascending edge / element order, so every node sum adds its terms in the
 * reference's serial scatter order) and copies topology and geometry to the
 * current CUDA device.  max_tracers bounds the batched entry points. */
int fesom_gpu_init(const fesom_mesh_desc *mesh, int32_t precision, int32_t max_tracers, fesom_gpu_ctx **ctx);
int fesom_gpu_finalize(fesom_gpu_ctx *ctx);
/* Host-only: validates the mesh and returns the derived muscl_adv_init arrays
 * (index_base-based, either output may be NULL) without touching the GPU; on
 * failure the message is written to errbuf (errlen bytes, NUL-terminated). */
int fesom_gpu_mesh_check(const fesom_mesh_desc *mesh, int32_t *nboundary_lay, int32_t *edge_up_dn_tri, char *errbuf,
                         int32_t errlen);
/* Launch everything on this stream (a cudaStream_t); NULL = the legacy default stream. */
int fesom_gpu_set_stream(fesom_gpu_ctx *ctx, void *stream);
const char *fesom_gpu_last_error(const fesom_gpu_ctx *ctx);
int fesom_gpu_abi_version(void);
/* Page-locked host memory (cudaHostAlloc) for the arrays of the host-array steps: copies from and
 * into it run at the host link's full rate without page-locking a caller's allocation later.
 * fesom_gpu_host_free releases it (NULL: nothing). */
int fesom_gpu_host_alloc(size_t bytes, void **ptr);
int fesom_gpu_host_free(void *ptr);
/* Copies of the derived init arrays, index_base-based: nboundary_lay (nod2D),
 * edge_up_dn_tri (2, edge2D).  Either pointer may be NULL. */
int fesom_gpu_get_muscl_init(fesom_gpu_ctx *ctx, int32_t *nboundary_lay, int32_t *edge_up_dn_tri);
/* Reads and clears the device status word (FESOM_STATUS_* bits); waits at
 * most timeout_ms for the stream, returns FESOM_ERR_TIMEOUT beyond. */
int fesom_gpu_status(fesom_gpu_ctx *ctx, uint32_t *status, int32_t timeout_ms);
/* ALE: new hnode/hnode_new/helem/Z_3d_n/zbar_3d_n (any may be NULL = unchanged). */
int fesom_gpu_update_thickness(fesom_gpu_ctx *ctx, const double *hnode, const double *hnode_new,
                               const double *helem, const double *Z_3d_n, const double *zbar_3d_n);

/* ---- per-routine drop-ins (FP64, host arrays, one tracer per call) -------
 * They stage their arrays in the buffers of the context's first tracer slot,
 * so between them and device-resident stepping (fesom_gpu_state_setup /
 * fesom_gpu_run_steps) of the same context, slot 0's device state is not
 * kept: a caller mixing the two re-uploads it (fesom_gpu_tracer_upload). */
/* init_tracers_AB: valuesAB from values/valuesold (AB2/AB3), valuesold shift,
 * element gradients (tr_xy) and edge_up_dn_grad kept on the device.
 * valuesold is (ab_order-1, nl-1, nod2D). */
int fesom_gpu_init_tracers_ab(fesom_gpu_ctx *ctx, const fesom_tra_cfg *cfg, const double *values,
                              double *valuesAB, double *valuesold);
/* tracer_gradient_z (src/oce_tracer_mod.F90:192-232), FP64 contexts: tr_z(nz, n) of values
 * (nl-1, nod2D) into tr_z (nl, nod2D) -- (T(nz-1) - T(nz)) / (0.5 (hnode(nz-1) + hnode(nz)))
 * for nzmin < nz < nzmax, zero at nzmin and nzmax; the other entries of tr_z keep their
 * values.  The reference computes it in init_tracers_AB for the modules outside the tracer
 * step (the step itself does not read it). */
int fesom_gpu_tracer_gradient_z(fesom_gpu_ctx *ctx, const double *values, double *tr_z);
/* do_oce_adv_tra with use_wsplit = .false.: vel (2, nl-1, elem2D), w/wi/we
 * (nl, nod2D), ttf = values, ttfAB = valuesAB (nl-1, nod2D).  Writes
 * dttf_h / dttf_v (del_ttf_advhoriz / del_ttf_advvert, (nl-1, nod2D)); they
 * are overwritten (the reference adds to arrays that init_tracers_AB zeroed). */
int fesom_gpu_adv_tra(fesom_gpu_ctx *ctx, double dt, const double *vel, const double *w, const double *wi,
                      const double *we, const fesom_tra_cfg *cfg, const double *ttf, const double *ttfAB,
                      double *dttf_h, double *dttf_v);
/* diff_ver_part_impl_ale (Redi, KPP non-local, shortwave and iceberg terms
 * off): Kv (nl, nod2D), bc_surf (nod2D) = the bc_surface() term added at
 * nzmin; values (nl-1, nod2D) updated in place. */
int fesom_gpu_vdiff_impl(fesom_gpu_ctx *ctx, double dt, const fesom_tra_cfg *cfg, const double *Kv,
                         const double *bc_surf, double *values);
/* The same with the w_i terms of a split vertical velocity (wi(nl, nod2D); NULL: none) for a
 * tracer without the limiter, as diff_ver_part_impl_ale with do_wimpl. */
int fesom_gpu_vdiff_impl_wi(fesom_gpu_ctx *ctx, double dt, const fesom_tra_cfg *cfg, const double *Kv,
                            const double *bc_surf, const double *wi, double *values);

/* ---- the whole tracer step for all tracers (host arrays) ----------------- */
/* values[t] (nl-1, nod2D), valuesold[t] (ab_order-1, nl-1, nod2D) updated in
 * place; bc_surf is (nod2D, ntr) or NULL (zero).  In FESOM_PREC_FP32 the data
 * are rounded to FP32 on the device and the results widened back. */
int fesom_gpu_tracer_step(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs, double dt,
                          const double *uv, const double *w, const double *wi, const double *we,
                          const double *Kv, const double *bc_surf, double *const *values,
                          double *const *valuesold);

/* ---- device-resident stepping (the form a time loop uses) ---------------- */
/* Tracer state lives on the device in the context's precision.  Forcing
 * (uv, w, wi, we, Kv, bc_surf) is uploaded once per model step; steps then run
 * from a captured CUDA graph with no host traffic.  FP64 host arrays are
 * converted on the device in FESOM_PREC_FP32. */
int fesom_gpu_state_setup(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs);
int fesom_gpu_forcing_upload(fesom_gpu_ctx *ctx, const double *uv, const double *w, const double *wi,
                             const double *we, const double *Kv, const double *bc_surf);
int fesom_gpu_tracer_upload(fesom_gpu_ctx *ctx, int32_t tr, const double *values, const double *valuesold);
int fesom_gpu_tracer_download(fesom_gpu_ctx *ctx, int32_t tr, double *values, double *valuesold);
/* FP32 host buffers (FESOM_PREC_FP32 only): no widening on the way. */
int fesom_gpu_tracer_upload_f32(fesom_gpu_ctx *ctx, int32_t tr, const float *values, const float *valuesold);
int fesom_gpu_tracer_download_f32(fesom_gpu_ctx *ctx, int32_t tr, float *values, float *valuesold);
int fesom_gpu_forcing_upload_f32(fesom_gpu_ctx *ctx, const float *uv, const float *w, const float *wi,
                                 const float *we, const float *Kv, const float *bc_surf);
/* Runs nsteps tracer steps of dt on the device (graph replay when use_graph). */
int fesom_gpu_run_steps(fesom_gpu_ctx *ctx, double dt, int32_t nsteps, int32_t use_graph);
/* Tracers per launch of each stage (0 = as many as the work arrays hold; the
 * FP64 plain form uses 1, one tracer per launch as the reference loops; the
 * FP32 form rounds n up to whole tracer groups). */
int fesom_gpu_set_tracers_per_launch(fesom_gpu_ctx *ctx, int32_t n);
/* One step without the graph, with CUDA events around every stage on the
 * context stream; stage_ms[i] receives the summed time of stage i over all
 * tracer groups and launches[i] the number of launches (arrays of
 * FESOM_NUM_STAGES entries, stage order: ab, trxy, edge_flux, node_lo,
 * bounds, rpm, update, vdiff, vflux, vfactors, lo_ad; the FP64 form uses the
 * first eight, the FP32 form vflux, vfactors, lo_ad, bounds, update). */
#define FESOM_NUM_STAGES 11
int fesom_gpu_profile_step(fesom_gpu_ctx *ctx, double dt, float *stage_ms, int32_t *launches);
/* Copy of an internal per-tracer work array of tracer slot tr (FP64 contexts,
 * for testing): name is one of "T", "Told", "TAB", "trxy", "FLO", "ADh", "LO",
 * "ADv", "bmax", "bmin" (bmax/bmin hold R+/R- after a step), "dttf_h",
 * "dttf_v"; count is the number of doubles out can hold. */
int fesom_gpu_debug_fetch(fesom_gpu_ctx *ctx, const char *name, int32_t tr, double *out, size_t count);
/* Kernel launches one device-resident step issues. */
int fesom_gpu_launches_per_step(fesom_gpu_ctx *ctx, int32_t *launches);
/* ---- allocation-free vertical diffusion ----------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * FESOM2's OpenACC build, whose `!$ACC DATA` regions own every device array
 * and pass them out as device addresses (`!$ACC HOST_DATA USE_DEVICE`), and
 * codes held to a fixed device-memory budget.  Same computation as
 * fesom_gpu_vdiff_impl (diff_ver_part_impl_ale, FP64, bit-identical results)
 * on arrays the caller already holds on the current device -- every pointer is
 * a DEVICE pointer in the layout of fesom_mesh_desc -- with no context and no
 * allocation: the column-solve scratch is a fixed device array inside the
 * library, FESOM_GPU_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB, held by every
 * GPU that loads the library until the process exits).  Meshes with
 * 3*nl*nod2D above that are rejected with FESOM_ERR_ARG and a message in
 * errbuf.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * Columns must satisfy 1 <= ulevels_nod2D(n), nlevels_nod2D(n) <= nl and
 * nlevels_nod2D(n) - ulevels_nod2D(n) >= 2 (two wet layers); the kernel skips
 * any other column, leaving its values untouched, and the call returns
 * FESOM_ERR_MESH.  The work runs on `stream` (a cudaStream_t, NULL = legacy
 * stream); the call waits for it (at most 60 s, else FESOM_ERR_TIMEOUT) and
 * reads the kernel's status word back, so the values are final on return.
 * All calls share the scratch and the status word: calls that overlap on the
 * GPU (other streams, other host threads) race on them. */
#define FESOM_GPU_NOALLOC_SCRATCH_DOUBLES ((size_t)4194304)
int fesom_gpu_vdiff_impl_noalloc(int32_t nod2D, int32_t nl, const int32_t *nlevels_nod2D,
                                 const int32_t *ulevels_nod2D, const double *zbar_n_bot, const double *hnode_new,
                                 const double *area, const double *areasvol, const double *Kv, const double *bc_surf,
                                 double dt, double *values, void *stream, char *errbuf, int32_t errlen);

/* Global content sum_nodes sum_levels values*hnode_new*areasvol per tracer, in FP64. */
int fesom_gpu_tracer_content(fesom_gpu_ctx *ctx, double *content);
/* Device pointer of tracer tr's values, for zero-copy users (FP64 contexts; an FP32
 * context stores its tracers interleaved in groups and returns FESOM_ERR_STATE). */
int fesom_gpu_tracer_device_ptr(fesom_gpu_ctx *ctx, int32_t tr, void **values, void **valuesold);

/* Horizontal diffusion of diff_tracers_ale (diff_part_hor_redi, src/oce_ale_tracer.F90:1526-1689,
 * Redi off): Ki(nl-1, nod2D) = K_hor (mesh_resolution / 100 km)^2 (src/oce_setup_step.F90:968-972).
 * fesom_gpu_set_hdiff makes every later step of the context add it (NULL: none, as K_hor = 0);
 * the FP64 and FP32 forms both take it. */
int fesom_gpu_set_hdiff(fesom_gpu_ctx *ctx, const double *Ki);
/* dynamics%use_wsplit (src/MOD_DYN.F90:156, off by default): the vertical velocity is split
 * into the explicit w_e and the implicit w_i (the forcing's we / wi).  With it on, FCT tracers
 * advect their LO values implicitly by w_i (adv_tra_vert_impl, src/oce_adv_tra_ver.F90:90-240)
 * and take the upwind flux of the full w as the LO part of the antidiffusive vertical flux
 * (src/oce_adv_tra_driver.F90:323-334); tracers without the limiter add w_i to the implicit
 * vertical solve (src/oce_ale_tracer.F90:961, 1134-1216).  Applies to every later step and to
 * fesom_gpu_adv_tra, which then needs wi. */
int fesom_gpu_set_wsplit(fesom_gpu_ctx *ctx, int32_t on);
/* Performance setting of the FP32 form (results do not change): tracers per launch of the
 * node/edge stages, stage 0 = LO and vertical fluxes, 1 = horizontal high-order fluxes,
 * 2 = FCT bounds, 3 = limited update, rounded up to whole tracer groups; 0 (the default) =
 * every group of the launch group in one launch. */
int fesom_gpu_set_stage_tracers(fesom_gpu_ctx *ctx, int32_t stage, int32_t tracers);
/* Performance setting of the FP32 form (results do not change): grid of the node/edge stage
 * kernels (stages as in fesom_gpu_set_stage_tracers): blocks_per_sm > 0 launches at most
 * blocks_per_sm x 152 blocks whose warps loop over the units (nodes, edges); 0 (the default)
 * launches one warp per unit. */
int fesom_gpu_set_launch_shape(fesom_gpu_ctx *ctx, int32_t stage, int32_t blocks_per_sm);
/* Performance setting of the FP32 form: kernel variant of stage 0 (lo_ad), 1 (the edge fluxes),
 * 2 (bounds) or 3 (update): bit 0 clear gathers each pass's entries into registers, set stages
 * them in shared memory with asynchronous copies while the previous pass computes (fewer resident
 * warps, no register limit on the gathers in flight).  Stage 3 only, bit 1 (values 2, 3): the
 * implicit vertical diffusion runs as its own kernel after the update; clear (the default), each
 * node's column is diffused by the warp that has just updated it, in the same launch.  Defaults:
 * lo_ad 1, the others 0.  The variants are separate compilations and agree to FP32 round-off. */
int fesom_gpu_set_stage_variant(fesom_gpu_ctx *ctx, int32_t stage, int32_t variant);
/* Autotuner of the FP32 form's launch settings (results do not change): times the step of the
 * context's own state under the library defaults, then by coordinate descent over the four node/edge
 * stages under each kernel variant, blocks per SM (0, 2, 4) and, for bounds and update with more
 * than 8 tracer slots, 8 tracers per launch; a candidate is kept when it is more than 1 % faster.
 * Each candidate runs one untimed and `steps` timed steps (CUDA events on the context's stream).
 * The fastest settings stay on the context; the tracer state and its time levels are restored
 * afterwards (one extra copy of the time levels on the device while tuning). */
typedef struct fesom_tune_result {
    float default_ms, tuned_ms;   /* ms per step under the defaults and under the chosen settings */
    int32_t candidates;           /* settings timed */
    int32_t stage_tracers[4];     /* chosen, per stage (fesom_gpu_set_stage_tracers) */
    int32_t blocks_per_sm[4];     /* (fesom_gpu_set_launch_shape) */
    int32_t variant[4];           /* (fesom_gpu_set_stage_variant) */
} fesom_tune_result;
int fesom_gpu_autotune(fesom_gpu_ctx *ctx, double dt, int32_t steps, fesom_tune_result *res);
/* The routine alone (FP64 contexts): del_ttf += the edge diffusion fluxes of the element
 * gradients of values, in ascending edge order. */
int fesom_gpu_diff_hor(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *values, double *del_ttf);
/* Redi = .true. (isoneutral diffusion, src/oce_ale_tracer.F90:594-623, 1099-1204, 1439-1689) with
 * the tapered neutral slopes slope(3, nl-1, nod2D) (slope_tapered of compute_neutral_slope,
 * src/oce_ale_pressure_bv.F90:3039-3157) as input.  fesom_gpu_set_redi copies the slopes to the
 * context (call it again whenever they change, e.g. before every step; NULL: Redi off); every
 * later step of either form then adds the slope terms to the horizontal diffusion, applies
 * diff_ver_part_redi_expl after the explicit vertical part, and diffuses implicitly with
 * K33 = Kv + Kd s^2.  Needs the horizontal diffusivity (fesom_gpu_set_hdiff; FESOM_ERR_STATE
 * without it); clearing Ki suspends Redi.  The multi-instance batch does not take Redi. */
int fesom_gpu_set_redi(fesom_gpu_ctx *ctx, const double *slope);
/* The routines alone (FP64 contexts): diff_part_hor_redi with the slope terms (slope NULL:
 * fesom_gpu_diff_hor), diff_ver_part_redi_expl (del_ttf += the vertical projection of the
 * isoneutral flux of values), and K33(nl, nod2D) = Kv + Ty at the interfaces nzmin < nz < nzmax
 * of each column (Kv elsewhere). */
int fesom_gpu_diff_hor_redi(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *slope, const double *values,
                            double *del_ttf);
int fesom_gpu_diff_ver_redi_expl(fesom_gpu_ctx *ctx, double dt, const double *Ki, const double *slope,
                                 const double *values, double *del_ttf);
int fesom_gpu_redi_k33(fesom_gpu_ctx *ctx, const double *Kv, const double *Ki, const double *slope, double *K33);
/* diff_ver_part_expl_ale (src/oce_ale_tracer.F90:841-902, FP64 contexts): del_ttf += the explicit
 * vertical diffusion of values with Kv(nl, nod2D); flux_surf(nod2D) is the surface flux
 * vd_flux(ulevels) (-heat_flux/vcpw for temperature, the salt fluxes for salinity; NULL: 0).
 * The steps apply it to the tracers with i_vert_diff = 0, with the bc_surf entries of those
 * tracers as their surface flux. */
int fesom_gpu_diff_ver_expl(fesom_gpu_ctx *ctx, double dt, const double *Kv, const double *flux_surf,
                            const double *values, double *del_ttf);

/* Tail of the tracer loop of solve_tracers_ale (src/oce_ale_tracer.F90:353-375, 497-525):
 * radioactive decay of the tracers with ID 14 and 39; relax_to_clim (src/oce_tracer_mod.F90:
 * 236-298) of the tracers with ID 1 and 2 when clim_relax > 1e-8 -- or, with zonal_relax,
 * the Soufflet channel's relax_zonal_temp (src/toy_channel_soufflet.F90:91-121) of tracer 1,
 * applied once per tracer of the loop as the reference does; then the salinity tracer
 * clamped to [3, 45] and the age tracer floored at 0.  FP64 contexts, host arrays in place. */
typedef struct fesom_tail_cfg {
    double clim_relax;     /* namelist clim_relax (src/oce_modules.F90:46) */
    int32_t salt_index;    /* 0-based tracer clamped to [3, 45] (the reference: tracer 2); -1: none */
    int32_t age_index;     /* 0-based age tracer (use_age_tracer); -1: none */
    int32_t zonal_relax;   /* 1: relax_zonal_temp instead of relax_to_clim */
    int32_t nbins;         /* relax_zonal_temp: bins of ztem(nl-1, nbins) */
    double lat0, dy, tau_inv;
} fesom_tail_cfg;
int fesom_gpu_tracer_tail(fesom_gpu_ctx *ctx, int32_t ntr, const fesom_tra_cfg *cfgs, double dt,
                          const fesom_tail_cfg *tc, const double *relax2clim, const double *Tclim, const double *Sclim,
                          const double *ztem, double *const *values);

/* FP32 form, tracer groups (no counterpart in the reference): the tracers sit in groups of
 * `width` (4, or 2) slots of one scheme (limiter, horizontal and vertical scheme, implicit
 * vertical diffusion), interleaved in every (level, node) entry of the device arrays, so one
 * vector load serves a whole group.  fesom_gpu_state_setup places the tracers in order, each
 * into the first group of its scheme with room; the width is the one with the fewest slots
 * (4 on a tie) unless fesom_gpu_set_tracer_width (0 = automatic, 2, 4) asked for one before
 * the setup.  fesom_gpu_tracer_groups reports the placement: the group count, the width and,
 * per tracer (arrays of the tracer count, NULL to skip), its group and slot. */
int fesom_gpu_set_tracer_width(fesom_gpu_ctx *ctx, int32_t width);
int fesom_gpu_tracer_groups(fesom_gpu_ctx *ctx, int32_t *groups, int32_t *width, int32_t *group_of,
                            int32_t *slot_of);
/* One step of an FP32 context from and to host arrays (FP32, the caller's layout), with the
 * transfers overlapped with the compute: the tracer groups move in pipeline stages -- a stage
 * is packed into the group layout and computed as soon as its values and previous levels are
 * resident, and is unpacked and copied back as soon as it is done, while later stages upload
 * and earlier ones download (two staging buffers each way, allocated on the first call).  The
 * first stage's upload and the last stage's download are not hidden, so by default both stages
 * are small and the stages between double up to the groups per launch
 * (fesom_gpu_set_tracers_per_launch; L groups per launch: max(1, L/3) groups first and last);
 * fesom_gpu_set_host_groups sets another order.  values_out / valuesold_out may be the input
 * arrays (in-place update, as the reference's tracer arrays); valuesold_out may be NULL: the
 * previous level after the step is the values the step started from, so a caller that keeps
 * two time-level arrays and swaps them (values_out = valuesold_in, then exchange the roles)
 * moves only the new values back.  AB3 previous levels are interleaved valuesold(2, level,
 * node) as in the reference.  Blocks until the results are in host memory; page-locked host
 * arrays give the full transfer rate.  fesom_gpu_tracer_step of an FP32 context runs the same
 * pipeline on its FP64 host arrays (converted on the device). */
/* Pipeline stages of fesom_gpu_step_host_f32 / fesom_gpu_tracer_step, in order: n sizes of 1
 * to the groups per launch each, in tracer groups, summing to the context's group count
 * (FESOM_ERR_ARG otherwise); n = 0 restores the default.  Cleared by
 * fesom_gpu_set_tracers_per_launch and by a state setup that places the tracers anew. */
int fesom_gpu_set_host_groups(fesom_gpu_ctx *ctx, int32_t n, const int32_t *sizes);
int fesom_gpu_step_host_f32(fesom_gpu_ctx *ctx, double dt, const float *uv, const float *w, const float *wi,
                            const float *we, const float *Kv, const float *bc_surf, const float *const *values_in,
                            const float *const *valuesold_in, float *const *values_out, float *const *valuesold_out);

/* ---- multi-instance batch of the FP32 form --------------------------------------------
 * No counterpart in the reference: FESOM2 steps one mesh per MPI rank.  Independent FP32
 * contexts -- each with its own mesh, tracer state (fesom_gpu_state_setup, all tracers in
 * one launch group) and forcing uploaded, all with one Adams-Bashforth order -- step
 * together with one kernel launch per stage over all of them.  The results agree with
 * stepping each context alone (fesom_gpu_run_steps) to FP32 rounding; afterwards each
 * context is read with its own calls (fesom_gpu_tracer_download_f32, fesom_gpu_tracer_content).
 * At most 64 contexts per batch.  The batch keeps pointers to the contexts: destroy it
 * before them. */
typedef struct fesom_gpu_batch fesom_gpu_batch;
int fesom_gpu_batch_create(fesom_gpu_ctx *const *ctxs, int32_t n, fesom_gpu_batch **out);
/* stream of the batch launches (NULL = legacy stream); the contexts' own streams are not used */
int fesom_gpu_batch_set_stream(fesom_gpu_batch *b, void *stream);
/* nsteps steps of every instance; use_graph != 0 replays a captured CUDA graph per step */
int fesom_gpu_batch_run_steps(fesom_gpu_batch *b, double dt, int32_t nsteps, int32_t use_graph);
int fesom_gpu_batch_launches_per_step(fesom_gpu_batch *b, int32_t *launches);
const char *fesom_gpu_batch_last_error(const fesom_gpu_batch *b);
int fesom_gpu_batch_destroy(fesom_gpu_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* FESOM_GPU_H */
