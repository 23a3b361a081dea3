! fesom_gpu_shims.F90 -- drop-in replacements of FESOM2's tracer-transport routines that call
! libfesom_gpu through fesom_gpu_mod.
!
! Same names and arguments as the reference routines, so FESOM2's driver and derived types stay
! unchanged; a build selects them with FESOM_GPU (the reference's own bodies compile otherwise).
! They use the reference's modules (MOD_MESH, MOD_PARTIT, MOD_TRACER, MOD_DYN, g_config,
! par_ex) and build inside FESOM2's source tree only.  The path runs on one GPU over the whole
! mesh: the context is made with npes == 1 (eDim_nod2D == 0, no halo).
#ifdef FESOM_GPU

! once, after mesh_setup / ocean_setup (src/fesom_module.F90:379-468): the context over the
! mesh, reusing the reference's own muscl_adv_init result
subroutine fesom_gpu_setup(precision, ntracers, tracers, partit, mesh)
  use iso_c_binding
  use fesom_gpu_mod
  use MOD_MESH
  use MOD_PARTIT
  use MOD_PARSUP
  use MOD_TRACER
  use g_config, only: cyclic_length
  implicit none
  integer(c_int32_t), intent(in) :: precision
  integer, intent(in) :: ntracers
  type(t_tracer), intent(in), target :: tracers
  type(t_partit), intent(inout), target :: partit
  type(t_mesh), intent(in), target :: mesh
  type(fesom_mesh_desc) :: d
  integer(c_int) :: rc
  if (partit%npes /= 1) call par_ex(partit%MPI_COMM_FESOM, partit%mype, 1)
  d%nod2D = mesh%nod2D;  d%elem2D = mesh%elem2D;  d%edge2D = mesh%edge2D;  d%nl = mesh%nl
  d%index_base = 1
  d%ld_nie = size(mesh%nod_in_elem2D, 1)
  d%elem2D_nodes = c_loc(mesh%elem2D_nodes);  d%edges = c_loc(mesh%edges);  d%edge_tri = c_loc(mesh%edge_tri)
  d%nod_in_elem2D_num = c_loc(mesh%nod_in_elem2D_num);  d%nod_in_elem2D = c_loc(mesh%nod_in_elem2D)
  d%nlevels = c_loc(mesh%nlevels);  d%ulevels = c_loc(mesh%ulevels)
  d%nlevels_nod2D = c_loc(mesh%nlevels_nod2D);  d%ulevels_nod2D = c_loc(mesh%ulevels_nod2D)
  d%nlevels_nod2D_min = c_loc(mesh%nlevels_nod2D_min);  d%ulevels_nod2D_max = c_loc(mesh%ulevels_nod2D_max)
  d%coord_nod2D = c_loc(mesh%coord_nod2D)
  d%elem_area = c_loc(mesh%elem_area);  d%elem_cos = c_loc(mesh%elem_cos)
  d%edge_dxdy = c_loc(mesh%edge_dxdy);  d%edge_cross_dxdy = c_loc(mesh%edge_cross_dxdy)
  d%gradient_sca = c_loc(mesh%gradient_sca)
  d%area = c_loc(mesh%area);  d%areasvol = c_loc(mesh%areasvol)
  d%hnode = c_loc(mesh%hnode);  d%hnode_new = c_loc(mesh%hnode_new);  d%helem = c_loc(mesh%helem)
  d%Z_3d_n = c_loc(mesh%Z_3d_n);  d%zbar_3d_n = c_loc(mesh%zbar_3d_n);  d%zbar_n_bot = c_loc(mesh%zbar_n_bot)
  d%cyclic_length = cyclic_length
  d%nboundary_lay = c_loc(tracers%work%nboundary_lay)
  d%edge_up_dn_tri = c_loc(tracers%work%edge_up_dn_tri)
  rc = fesom_gpu_init(d, precision, int(ntracers, c_int32_t), gpu_ctx)
  if (rc /= FESOM_OK) call par_ex(partit%MPI_COMM_FESOM, partit%mype, 1)
end subroutine fesom_gpu_setup

! do_oce_adv_tra (src/oce_adv_tra_driver.F90:46-490), use_wsplit = .false.
subroutine do_oce_adv_tra(dt, vel, w, wi, we, tr_num, dynamics, tracers, partit, mesh)
  use iso_c_binding
  use fesom_gpu_mod
  use MOD_MESH
  use MOD_TRACER
  use MOD_PARTIT
  use MOD_PARSUP
  use MOD_DYN
  implicit none
  real(kind=WP),  intent(in),    target :: dt
  integer,        intent(in)            :: tr_num
  type(t_mesh)  , intent(in)   , target :: mesh
  type(t_partit), intent(inout), target :: partit
  type(t_tracer), intent(inout), target :: tracers
  type(t_dyn)   , intent(inout), target :: dynamics
  real(kind=WP),  intent(in), target    :: vel(2, mesh%nl-1, partit%myDim_elem2D+partit%eDim_elem2D)
  real(kind=WP),  intent(in), target    :: W(mesh%nl,    partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP),  intent(in), target    :: WI(mesh%nl,   partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP),  intent(in), target    :: WE(mesh%nl,   partit%myDim_nod2D+partit%eDim_nod2D)
  type(fesom_tra_cfg) :: c
  integer(c_int) :: rc
  associate (td => tracers%data(tr_num))
    c = to_cfg(td%tra_adv_hor, td%tra_adv_ver, td%tra_adv_lim, td%tra_adv_ph, td%tra_adv_pv, &
               td%AB_order, td%i_vert_diff, td%ID)
    rc = fesom_gpu_adv_tra(gpu_ctx, dt, c_loc(vel), c_loc(W), c_loc(WI), c_loc(WE), c, c_loc(td%values), &
                           c_loc(td%valuesAB), c_loc(tracers%work%del_ttf_advhoriz), &
                           c_loc(tracers%work%del_ttf_advvert))
  end associate
  if (rc /= FESOM_OK) call par_ex(partit%MPI_COMM_FESOM, partit%mype, 1)
end subroutine do_oce_adv_tra

! diff_ver_part_impl_ale (src/oce_ale_tracer.F90:907-1435) with the Redi, KPP non-local,
! shortwave and iceberg terms off; bc(n) is the bc_surface() term of :1382 for every node
subroutine diff_ver_part_impl_ale_gpu(tr_num, dt, Kv, bc, dynamics, tracers, partit, mesh)
  use iso_c_binding
  use fesom_gpu_mod
  use MOD_MESH
  use MOD_TRACER
  use MOD_PARTIT
  use MOD_PARSUP
  use MOD_DYN
  implicit none
  integer, intent(in) :: tr_num
  real(kind=WP), intent(in) :: dt
  type(t_mesh), intent(in), target :: mesh
  type(t_partit), intent(inout), target :: partit
  type(t_tracer), intent(inout), target :: tracers
  type(t_dyn), intent(inout), target :: dynamics
  real(kind=WP), intent(in), target :: Kv(mesh%nl, partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP), intent(in), target :: bc(partit%myDim_nod2D+partit%eDim_nod2D)
  type(fesom_tra_cfg) :: c
  integer(c_int) :: rc
  associate (td => tracers%data(tr_num))
    c = to_cfg(td%tra_adv_hor, td%tra_adv_ver, td%tra_adv_lim, td%tra_adv_ph, td%tra_adv_pv, &
               td%AB_order, td%i_vert_diff, td%ID)
    if (dynamics%use_wsplit .and. trim(td%tra_adv_lim) /= 'FCT') then
       ! do_wimpl: the implicit part of the vertical velocity joins the solve (:961)
       rc = fesom_gpu_vdiff_impl_wi(gpu_ctx, dt, c, c_loc(Kv), c_loc(bc), c_loc(dynamics%w_i), c_loc(td%values))
    else
       rc = fesom_gpu_vdiff_impl(gpu_ctx, dt, c, c_loc(Kv), c_loc(bc), c_loc(td%values))
    end if
  end associate
  if (rc /= FESOM_OK) call par_ex(partit%MPI_COMM_FESOM, partit%mype, 1)
end subroutine diff_ver_part_impl_ale_gpu

! the body of the tracer loop of solve_tracers_ale (src/oce_ale_tracer.F90:280-351) for all
! tracers in one call; bc_all(nod2D, num_tracers) holds each tracer's bc_surface() term
subroutine solve_tracers_gpu(dt, UV, Wvel, Wvel_i, Wvel_e, Kv, bc_all, tracers, partit, mesh)
  use iso_c_binding
  use fesom_gpu_mod
  use MOD_MESH
  use MOD_TRACER
  use MOD_PARTIT
  use MOD_PARSUP
  implicit none
  real(kind=WP), intent(in) :: dt
  type(t_mesh), intent(in), target :: mesh
  type(t_partit), intent(inout), target :: partit
  type(t_tracer), intent(inout), target :: tracers
  real(kind=WP), intent(in), target :: UV(2, mesh%nl-1, partit%myDim_elem2D+partit%eDim_elem2D)
  real(kind=WP), intent(in), target :: Wvel(mesh%nl, partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP), intent(in), target :: Wvel_i(mesh%nl, partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP), intent(in), target :: Wvel_e(mesh%nl, partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP), intent(in), target :: Kv(mesh%nl, partit%myDim_nod2D+partit%eDim_nod2D)
  real(kind=WP), intent(in), target :: bc_all(partit%myDim_nod2D+partit%eDim_nod2D, tracers%num_tracers)
  type(fesom_tra_cfg) :: cfgs(tracers%num_tracers)
  type(c_ptr) :: vp(tracers%num_tracers), op(tracers%num_tracers)
  integer :: tr_num
  integer(c_int) :: rc
  do tr_num = 1, tracers%num_tracers
     associate (td => tracers%data(tr_num))
       cfgs(tr_num) = to_cfg(td%tra_adv_hor, td%tra_adv_ver, td%tra_adv_lim, td%tra_adv_ph, td%tra_adv_pv, &
                             td%AB_order, td%i_vert_diff, td%ID)
       vp(tr_num) = c_loc(td%values)
       op(tr_num) = c_loc(td%valuesold)
     end associate
  end do
  rc = fesom_gpu_tracer_step(gpu_ctx, int(tracers%num_tracers, c_int32_t), cfgs, dt, c_loc(UV), c_loc(Wvel), &
                             c_loc(Wvel_i), c_loc(Wvel_e), c_loc(Kv), c_loc(bc_all), vp, op)
  if (rc /= FESOM_OK) call par_ex(partit%MPI_COMM_FESOM, partit%mype, 1)
end subroutine solve_tracers_gpu

#endif
