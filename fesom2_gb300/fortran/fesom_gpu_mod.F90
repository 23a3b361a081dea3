! fesom_gpu_mod.F90 -- ISO_C_BINDING interface of libfesom_gpu.so (include/fesom_gpu.h) for
! FESOM2's Fortran code.
!
! A maintainer adds this file to FESOM2's src/ (next to fvom_init.F90, whose call of the C
! partitioner, src/fvom_init.F90:1750 <-> src/fort_part.c:47, is the existing precedent of a
! bind(C) call) and links libfesom_gpu.so.  Every array argument is type(c_ptr), passed as
! c_loc() of the derived types' own arrays in their own layout (values(nl-1, nod2D),
! UV(2, nl-1, elem2D), Wvel(nl, nod2D), ...) with no copy; inside `!$acc host_data use_device`
! the same calls take the device addresses.  Indices stay 1-based (index_base = 1).  A nonzero
! return code is mapped to par_ex, as the reference does for an unknown scheme.
!
! fesom_gpu_shims.F90 holds the drop-in replacements of the routines themselves.
module fesom_gpu_mod
  use iso_c_binding
  implicit none

  integer(c_int32_t), parameter :: FESOM_PREC_FP64 = 0, FESOM_PREC_FP32 = 1
  integer(c_int), parameter :: FESOM_OK = 0, FESOM_ERR_ARG = 1, FESOM_ERR_SCHEME = 2, FESOM_ERR_MESH = 3, &
                               FESOM_ERR_CUDA = 4, FESOM_ERR_NOMEM = 5, FESOM_ERR_TIMEOUT = 6, &
                               FESOM_ERR_NUMERIC = 7, FESOM_ERR_STATE = 8

  ! one row of nml_tracer_list (config/namelist.tra) plus AB_order and i_vert_diff
  type, bind(C) :: fesom_tra_cfg
     integer(c_int32_t) :: adv_hor, adv_ver, adv_lim, ab_order
     real(c_double)     :: adv_ph, adv_pv
     integer(c_int32_t) :: i_vert_diff, id
  end type fesom_tra_cfg

  ! the members of t_mesh the path reads (src/MOD_MESH.F90:22-160)
  type, bind(C) :: fesom_mesh_desc
     integer(c_int32_t) :: nod2D, elem2D, edge2D, nl, index_base, ld_nie
     type(c_ptr) :: elem2D_nodes, edges, edge_tri, nod_in_elem2D_num, nod_in_elem2D
     type(c_ptr) :: nlevels, ulevels, nlevels_nod2D, ulevels_nod2D, nlevels_nod2D_min, ulevels_nod2D_max
     type(c_ptr) :: coord_nod2D, elem_area, elem_cos, edge_dxdy, edge_cross_dxdy, gradient_sca
     type(c_ptr) :: area, areasvol, hnode, hnode_new, helem, Z_3d_n, zbar_3d_n, zbar_n_bot
     real(c_double) :: cyclic_length
     type(c_ptr) :: nboundary_lay, edge_up_dn_tri
  end type fesom_mesh_desc

  ! tail of solve_tracers_ale (src/oce_ale_tracer.F90:353-375, 497-525)
  type, bind(C) :: fesom_tail_cfg
     real(c_double)     :: clim_relax
     integer(c_int32_t) :: salt_index, age_index, zonal_relax, nbins
     real(c_double)     :: lat0, dy, tau_inv
  end type fesom_tail_cfg

  ! result of the FP32 launch-settings autotuner (fesom_gpu_autotune)
  type, bind(C) :: fesom_tune_result
     real(c_float)      :: default_ms, tuned_ms
     integer(c_int32_t) :: candidates
     integer(c_int32_t) :: stage_tracers(4), blocks_per_sm(4), variant(4)
  end type fesom_tune_result

  interface
     integer(c_int) function fesom_gpu_abi_version() bind(C, name="fesom_gpu_abi_version")
       import
     end function fesom_gpu_abi_version
     type(c_ptr) function fesom_gpu_last_error(ctx) bind(C, name="fesom_gpu_last_error")
       import
       type(c_ptr), value :: ctx
     end function fesom_gpu_last_error
     ! setup of the FCT / MUSCL work (src/oce_adv_tra_fct.F90:35-67, src/oce_muscl_adv.F90:32-352)
     integer(c_int) function fesom_gpu_init(mesh, precision, max_tracers, ctx) bind(C, name="fesom_gpu_init")
       import
       type(fesom_mesh_desc), intent(in) :: mesh
       integer(c_int32_t), value :: precision, max_tracers
       type(c_ptr), intent(out) :: ctx
     end function fesom_gpu_init
     integer(c_int) function fesom_gpu_finalize(ctx) bind(C, name="fesom_gpu_finalize")
       import
       type(c_ptr), value :: ctx
     end function fesom_gpu_finalize
     integer(c_int) function fesom_gpu_mesh_check(mesh, nboundary_lay, edge_up_dn_tri, errbuf, errlen) &
          bind(C, name="fesom_gpu_mesh_check")
       import
       type(fesom_mesh_desc), intent(in) :: mesh
       type(c_ptr), value :: nboundary_lay, edge_up_dn_tri
       character(kind=c_char), intent(out) :: errbuf(*)
       integer(c_int32_t), value :: errlen
     end function fesom_gpu_mesh_check
     integer(c_int) function fesom_gpu_status(ctx, status, timeout_ms) bind(C, name="fesom_gpu_status")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: status
       integer(c_int32_t), value :: timeout_ms
     end function fesom_gpu_status
     ! the ALE thickness update feeding the next step (src/oce_ale.F90:3819)
     integer(c_int) function fesom_gpu_update_thickness(ctx, hnode, hnode_new, helem, Z_3d_n, zbar_3d_n) &
          bind(C, name="fesom_gpu_update_thickness")
       import
       type(c_ptr), value :: ctx, hnode, hnode_new, helem, Z_3d_n, zbar_3d_n
     end function fesom_gpu_update_thickness
     ! init_tracers_AB (src/oce_tracer_mod.F90:13-143)
     integer(c_int) function fesom_gpu_init_tracers_ab(ctx, cfg, values, valuesAB, valuesold) &
          bind(C, name="fesom_gpu_init_tracers_ab")
       import
       type(c_ptr), value :: ctx
       type(fesom_tra_cfg), intent(in) :: cfg
       type(c_ptr), value :: values, valuesAB, valuesold
     end function fesom_gpu_init_tracers_ab
     ! tracer_gradient_z (src/oce_tracer_mod.F90:192-232)
     integer(c_int) function fesom_gpu_tracer_gradient_z(ctx, values, tr_z) bind(C, name="fesom_gpu_tracer_gradient_z")
       import
       type(c_ptr), value :: ctx, values, tr_z
     end function fesom_gpu_tracer_gradient_z
     ! do_oce_adv_tra (src/oce_adv_tra_driver.F90:46-490)
     integer(c_int) function fesom_gpu_adv_tra(ctx, dt, vel, w, wi, we, cfg, ttf, ttfAB, dttf_h, dttf_v) &
          bind(C, name="fesom_gpu_adv_tra")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(c_ptr), value :: vel, w, wi, we
       type(fesom_tra_cfg), intent(in) :: cfg
       type(c_ptr), value :: ttf, ttfAB, dttf_h, dttf_v
     end function fesom_gpu_adv_tra
     ! diff_ver_part_impl_ale (src/oce_ale_tracer.F90:907-1435)
     integer(c_int) function fesom_gpu_vdiff_impl(ctx, dt, cfg, Kv, bc_surf, values) bind(C, name="fesom_gpu_vdiff_impl")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(fesom_tra_cfg), intent(in) :: cfg
       type(c_ptr), value :: Kv, bc_surf, values
     end function fesom_gpu_vdiff_impl
     ! the same with the w_i terms of a split vertical velocity (do_wimpl, :961, 1134-1216)
     integer(c_int) function fesom_gpu_vdiff_impl_wi(ctx, dt, cfg, Kv, bc_surf, wi, values) &
          bind(C, name="fesom_gpu_vdiff_impl_wi")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(fesom_tra_cfg), intent(in) :: cfg
       type(c_ptr), value :: Kv, bc_surf, wi, values
     end function fesom_gpu_vdiff_impl_wi
     ! the body of the tracer loop of solve_tracers_ale (src/oce_ale_tracer.F90:280-351), all tracers
     integer(c_int) function fesom_gpu_tracer_step(ctx, ntr, cfgs, dt, uv, w, wi, we, Kv, bc_surf, values, valuesold) &
          bind(C, name="fesom_gpu_tracer_step")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: ntr
       type(fesom_tra_cfg), intent(in) :: cfgs(*)
       real(c_double), value :: dt
       type(c_ptr), value :: uv, w, wi, we, Kv, bc_surf
       type(c_ptr), intent(in) :: values(*), valuesold(*)
     end function fesom_gpu_tracer_step
     ! diff_part_hor_redi (Redi off) and diff_ver_part_expl_ale (src/oce_ale_tracer.F90:1526-1689, 841-902)
     integer(c_int) function fesom_gpu_set_hdiff(ctx, Ki) bind(C, name="fesom_gpu_set_hdiff")
       import
       type(c_ptr), value :: ctx, Ki
     end function fesom_gpu_set_hdiff
     integer(c_int) function fesom_gpu_diff_hor(ctx, dt, Ki, values, del_ttf) bind(C, name="fesom_gpu_diff_hor")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(c_ptr), value :: Ki, values, del_ttf
     end function fesom_gpu_diff_hor
     ! Redi = .true. with slope_tapered(3, nl-1, nod2D) as input (src/oce_ale_tracer.F90:594-623,
     ! 1099-1204, 1439-1689): set once per change of the slopes; the routines alone (FP64)
     integer(c_int) function fesom_gpu_set_redi(ctx, slope) bind(C, name="fesom_gpu_set_redi")
       import
       type(c_ptr), value :: ctx, slope
     end function fesom_gpu_set_redi
     integer(c_int) function fesom_gpu_diff_hor_redi(ctx, dt, Ki, slope, values, del_ttf) &
          bind(C, name="fesom_gpu_diff_hor_redi")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(c_ptr), value :: Ki, slope, values, del_ttf
     end function fesom_gpu_diff_hor_redi
     integer(c_int) function fesom_gpu_diff_ver_redi_expl(ctx, dt, Ki, slope, values, del_ttf) &
          bind(C, name="fesom_gpu_diff_ver_redi_expl")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(c_ptr), value :: Ki, slope, values, del_ttf
     end function fesom_gpu_diff_ver_redi_expl
     integer(c_int) function fesom_gpu_redi_k33(ctx, Kv, Ki, slope, K33) bind(C, name="fesom_gpu_redi_k33")
       import
       type(c_ptr), value :: ctx, Kv, Ki, slope, K33
     end function fesom_gpu_redi_k33
     integer(c_int) function fesom_gpu_diff_ver_expl(ctx, dt, Kv, flux_surf, values, del_ttf) &
          bind(C, name="fesom_gpu_diff_ver_expl")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       type(c_ptr), value :: Kv, flux_surf, values, del_ttf
     end function fesom_gpu_diff_ver_expl
     ! dynamics%use_wsplit (src/MOD_DYN.F90:156)
     integer(c_int) function fesom_gpu_set_wsplit(ctx, on) bind(C, name="fesom_gpu_set_wsplit")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: on
     end function fesom_gpu_set_wsplit
     ! tail of solve_tracers_ale (src/oce_ale_tracer.F90:353-375, 497-525)
     integer(c_int) function fesom_gpu_tracer_tail(ctx, ntr, cfgs, dt, tc, relax2clim, Tclim, Sclim, ztem, values) &
          bind(C, name="fesom_gpu_tracer_tail")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: ntr
       type(fesom_tra_cfg), intent(in) :: cfgs(*)
       real(c_double), value :: dt
       type(fesom_tail_cfg), intent(in) :: tc
       type(c_ptr), value :: relax2clim, Tclim, Sclim, ztem
       type(c_ptr), intent(in) :: values(*)
     end function fesom_gpu_tracer_tail
     ! device-resident stepping (no counterpart in the reference)
     integer(c_int) function fesom_gpu_state_setup(ctx, ntr, cfgs) bind(C, name="fesom_gpu_state_setup")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: ntr
       type(fesom_tra_cfg), intent(in) :: cfgs(*)
     end function fesom_gpu_state_setup
     integer(c_int) function fesom_gpu_forcing_upload(ctx, uv, w, wi, we, Kv, bc_surf) &
          bind(C, name="fesom_gpu_forcing_upload")
       import
       type(c_ptr), value :: ctx, uv, w, wi, we, Kv, bc_surf
     end function fesom_gpu_forcing_upload
     integer(c_int) function fesom_gpu_tracer_upload(ctx, tr, values, valuesold) bind(C, name="fesom_gpu_tracer_upload")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: tr
       type(c_ptr), value :: values, valuesold
     end function fesom_gpu_tracer_upload
     integer(c_int) function fesom_gpu_tracer_download(ctx, tr, values, valuesold) &
          bind(C, name="fesom_gpu_tracer_download")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: tr
       type(c_ptr), value :: values, valuesold
     end function fesom_gpu_tracer_download
     integer(c_int) function fesom_gpu_run_steps(ctx, dt, nsteps, use_graph) bind(C, name="fesom_gpu_run_steps")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       integer(c_int32_t), value :: nsteps, use_graph
     end function fesom_gpu_run_steps
     integer(c_int) function fesom_gpu_tracer_content(ctx, content) bind(C, name="fesom_gpu_tracer_content")
       import
       type(c_ptr), value :: ctx, content
     end function fesom_gpu_tracer_content
     ! FP32 launch settings chosen by timing the context's own step (state restored afterwards)
     integer(c_int) function fesom_gpu_autotune(ctx, dt, steps, res) bind(C, name="fesom_gpu_autotune")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: dt
       integer(c_int32_t), value :: steps
       type(fesom_tune_result), intent(out) :: res
     end function fesom_gpu_autotune
     ! allocation-free implicit vertical diffusion on device arrays the caller holds
     integer(c_int) function fesom_gpu_vdiff_impl_noalloc(nod2D, nl, nlevels_nod2D, ulevels_nod2D, zbar_n_bot, &
          hnode_new, area, areasvol, Kv, bc_surf, dt, values, stream, errbuf, errlen) &
          bind(C, name="fesom_gpu_vdiff_impl_noalloc")
       import
       integer(c_int32_t), value :: nod2D, nl
       type(c_ptr), value :: nlevels_nod2D, ulevels_nod2D, zbar_n_bot, hnode_new, area, areasvol, Kv, bc_surf
       real(c_double), value :: dt
       type(c_ptr), value :: values, stream
       character(kind=c_char), intent(out) :: errbuf(*)
       integer(c_int32_t), value :: errlen
     end function fesom_gpu_vdiff_impl_noalloc
  end interface

  ! the context of the run (one mesh, one GPU), created once after mesh_setup / ocean_setup
  type(c_ptr), save :: gpu_ctx = c_null_ptr

contains

  ! namelist strings -> scheme codes (src/oce_adv_tra_driver.F90:343-379); an unknown string
  ! gets a code the library rejects with FESOM_ERR_SCHEME
  function to_cfg(hor, ver, lim, ph, pv, ab_order, ivd, id) result(c)
    character(len=*), intent(in) :: hor, ver, lim
    real(kind=8), intent(in) :: ph, pv
    integer, intent(in) :: ab_order, id
    logical, intent(in) :: ivd
    type(fesom_tra_cfg) :: c
    select case (trim(hor))
    case ('MUSCL'); c%adv_hor = 0
    case ('MFCT');  c%adv_hor = 1
    case ('UPW1');  c%adv_hor = 2
    case default;   c%adv_hor = -1
    end select
    select case (trim(ver))
    case ('QR4C');  c%adv_ver = 0
    case ('UPW1');  c%adv_ver = 1
    case ('CDIFF'); c%adv_ver = 2
    case ('PPM');   c%adv_ver = 3
    case default;   c%adv_ver = -1
    end select
    c%adv_lim = merge(1, 0, trim(lim) == 'FCT')
    c%adv_ph = ph
    c%adv_pv = pv
    c%ab_order = ab_order
    c%i_vert_diff = merge(1, 0, ivd)
    c%id = id
  end function to_cfg

  ! the library's message for a nonzero return code
  function gpu_error_message() result(msg)
    character(len=512) :: msg
    character(kind=c_char), pointer :: s(:)
    type(c_ptr) :: p
    integer :: k
    msg = ''
    p = fesom_gpu_last_error(gpu_ctx)
    if (.not. c_associated(p)) return
    call c_f_pointer(p, s, [512])
    do k = 1, 512
       if (s(k) == c_null_char) exit
       msg(k:k) = s(k)
    end do
  end function gpu_error_message
end module fesom_gpu_mod
