! hyb_dvm.f90 -- ISO_C_BINDING interface to the C ABI in hyb_dvm.h.
!
! The Fortran host of Hybrid2D keeps its mesh, input and restart handling and
! calls the GB300 kinetic solver through these interfaces; every function
! returns the int status of the C side (0 = ok, negative = HYB_ERR_*).
module hyb_dvm
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: HYB_OK = 0, HYB_ERR_INVALID = -1, HYB_ERR_NOMEM = -2, &
       HYB_ERR_CUDA = -3, HYB_ERR_NONFINITE = -4, HYB_ERR_TIMEOUT = -5, &
       HYB_ERR_UNSUPPORTED = -6, HYB_ERR_TEMPERATURE = -7, HYB_ERR_NODEVICE = -8
  integer(c_int), parameter :: HYB_BC_WALL = -2, HYB_BC_PERIODIC = 1
  integer(c_int), parameter :: HYB_SCHEME_UP1 = 0, HYB_SCHEME_NND = 1, HYB_SCHEME_WENO3 = 3
  integer(c_int), parameter :: HYB_PREC_FP64 = 0, HYB_PREC_MIXED = 1
  integer(c_int), parameter :: HYB_SWEEP_REFERENCE = 0, HYB_SWEEP_UPWIND = 1
  integer(c_int), parameter :: HYB_STALL_NONE = 0, HYB_STALL_SWEEP_ROW = 1, HYB_STALL_NS_BARRIER = 2
  integer(c_int), parameter :: HYB_NSUM = 11, HYB_NRD = 2
  integer(c_int), parameter :: HYB_NOALLOC_MAX_CELLS = 209715

  type, bind(c) :: hyb_mesh
     integer(c_int) :: nx, ny
     type(c_ptr)    :: x, y
     integer(c_int) :: bc(4)
     type(c_ptr)    :: wall_u(4), wall_v(4), wall_t(4)
  end type hyb_mesh

  type, bind(c) :: hyb_vgrid
     integer(c_int) :: nvi, nvj
     type(c_ptr)    :: vi, vj, wi, wj
  end type hyb_vgrid

  type, bind(c) :: hyb_params
     real(c_double) :: dt, cfc, cpr, x1s, r00, t00
     integer(c_int) :: scheme, precision
     real(c_double) :: gamma, ma, pr, re, omega_ns
     integer(c_int) :: device
     integer(c_int) :: sweep_order, mass_pin
     integer(c_int) :: reserved(5)
  end type hyb_params

  type, bind(c) :: hyb_residual
     real(c_double) :: res_max(4), res_rms(4), max_rms
  end type hyb_residual

  type, bind(c) :: hyb_gsis_params
     integer(c_int) :: enable, max_inner
     real(c_double) :: inner_tol, inner_rtol, cfl, dtmax, dtmin
     integer(c_int) :: flux, ns_scheme, mlp_warm_after, ns_solver
     integer(c_int) :: correct_f, no_mass_projection, lusgs_planes, mlp_warm_inner
     real(c_double) :: mlp_warm_rtol
     integer(c_int) :: wall_band, relax_pct, line_mean
  end type hyb_gsis_params

  interface
     integer(c_int) function hyb_create(mesh, vgrid, params, ctx) bind(c, name="hyb_create")
       import :: c_int, c_ptr, hyb_mesh, hyb_vgrid, hyb_params
       type(hyb_mesh), intent(in) :: mesh
       type(hyb_vgrid), intent(in) :: vgrid
       type(hyb_params), intent(in) :: params
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function hyb_destroy(ctx) bind(c, name="hyb_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function hyb_last_error(ctx) bind(c, name="hyb_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function hyb_version() bind(c, name="hyb_version")
       import :: c_ptr
     end function
     integer(c_int) function hyb_init_maxwellian(ctx, rho, u, v, t) bind(c, name="hyb_init_maxwellian")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: rho, u, v, t
     end function
     integer(c_int) function hyb_upload_f(ctx, frd) bind(c, name="hyb_upload_f")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: frd(*)
     end function
     integer(c_int) function hyb_download_f(ctx, frd) bind(c, name="hyb_download_f")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: frd(*)
     end function
     integer(c_int) function hyb_download_moments(ctx, s_gkua, cf) bind(c, name="hyb_download_moments")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: s_gkua(*), cf(*)
     end function
     integer(c_int) function hyb_download_hot(ctx, tao_i, q_i, tao_j, q_j) bind(c, name="hyb_download_hot")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: tao_i(*), q_i(*), tao_j(*), q_j(*)
     end function
     integer(c_int) function hyb_download_hoq(ctx, hot, hoq) bind(c, name="hyb_download_hoq")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: hot(*), hoq(*)
     end function
     integer(c_int) function hyb_step(ctx, n_iter, res) bind(c, name="hyb_step")
       import :: c_int, c_ptr, hyb_residual
       type(c_ptr), value :: ctx
       integer(c_int), value :: n_iter
       type(hyb_residual), intent(out) :: res
     end function
     integer(c_int) function hyb_phy_boundary(ctx) bind(c, name="hyb_phy_boundary")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function hyb_kinetic_step(ctx) bind(c, name="hyb_kinetic_step")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function hyb_detfp(ctx) bind(c, name="hyb_detfp")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function hyb_convert_ns(ctx) bind(c, name="hyb_convert_ns")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function hyb_detfp_res(ctx, res) bind(c, name="hyb_detfp_res")
       import :: c_int, c_ptr, hyb_residual
       type(c_ptr), value :: ctx
       type(hyb_residual), intent(out) :: res
     end function
     integer(c_int) function hyb_gsis_configure(ctx, gp) bind(c, name="hyb_gsis_configure")
       import :: c_int, c_ptr, hyb_gsis_params
       type(c_ptr), value :: ctx
       type(hyb_gsis_params), intent(in) :: gp
     end function
     integer(c_int) function hyb_gsis_last_inner(ctx, n_inner) bind(c, name="hyb_gsis_last_inner")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: n_inner
     end function
     integer(c_int) function hyb_gsis_skipped(ctx, count) bind(c, name="hyb_gsis_skipped")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: count
     end function
     integer(c_int) function hyb_set_precision(ctx, precision) bind(c, name="hyb_set_precision")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: precision
     end function
     integer(c_int) function hyb_test_stall(ctx, site, spin_cycles) bind(c, name="hyb_test_stall")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: ctx
       integer(c_int), value :: site
       integer(c_long_long), value :: spin_cycles
     end function
     integer(c_int) function hyb_set_walls(ctx, face, wall_u, wall_v, wall_t) bind(c, name="hyb_set_walls")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: face
       real(c_double), intent(in) :: wall_u(*), wall_v(*), wall_t(*)
     end function
     integer(c_int) function hyb_detfp_noalloc(nx, ny, nvi, nvj, frd_dev, vi_dev, vj_dev, wi_dev, wj_dev, &
          params, s_gkua_dev, cf_dev, stream) bind(c, name="hyb_detfp_noalloc")
       import :: c_int, c_ptr, hyb_params
       integer(c_int), value :: nx, ny, nvi, nvj
       type(c_ptr), value :: frd_dev, vi_dev, vj_dev, wi_dev, wj_dev, s_gkua_dev, cf_dev, stream
       type(hyb_params), intent(in) :: params
     end function
     integer(c_int) function hyb_profile_enable(ctx, enable) bind(c, name="hyb_profile_enable")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: enable
     end function
     integer(c_int) function hyb_profile_read(ctx, ms, launches, n) bind(c, name="hyb_profile_read")
       import :: c_int, c_ptr, c_double, c_long_long
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: ms(*)
       integer(c_long_long), intent(out) :: launches(*)
       integer(c_int), value :: n
     end function
     integer(c_int) function hyb_launch_count(ctx, count) bind(c, name="hyb_launch_count")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: ctx
       integer(c_long_long), intent(out) :: count
     end function
     integer(c_int) function hyb_last_step_ms(ctx, ms) bind(c, name="hyb_last_step_ms")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: ms
     end function
     integer(c_int) function hyb_stream(ctx, stream) bind(c, name="hyb_stream")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       type(c_ptr), intent(out) :: stream
     end function
     integer(c_int) function hyb_autotune(ctx, reps, cpt, vpb) bind(c, name="hyb_autotune")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: reps
       integer(c_int), intent(out) :: cpt, vpb
     end function
     integer(c_int) function hyb_batch_create(n, meshes, vgrids, params, batch) bind(c, name="hyb_batch_create")
       import :: c_int, c_ptr, hyb_mesh, hyb_vgrid, hyb_params
       integer(c_int), value :: n
       type(hyb_mesh), intent(in) :: meshes(*)
       type(hyb_vgrid), intent(in) :: vgrids(*)
       type(hyb_params), intent(in) :: params(*)
       type(c_ptr), intent(out) :: batch
     end function
     integer(c_int) function hyb_batch_destroy(batch) bind(c, name="hyb_batch_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
     end function
     type(c_ptr) function hyb_batch_last_error(batch) bind(c, name="hyb_batch_last_error")
       import :: c_ptr
       type(c_ptr), value :: batch
     end function
     integer(c_int) function hyb_batch_size(batch, n) bind(c, name="hyb_batch_size")
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int), intent(out) :: n
     end function
     integer(c_int) function hyb_batch_instance(batch, k, ctx) bind(c, name="hyb_batch_instance")
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int), value :: k
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function hyb_batch_init_maxwellian(batch, rho, u, v, t) bind(c, name="hyb_batch_init_maxwellian")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: batch
       real(c_double), value :: rho, u, v, t
     end function
     integer(c_int) function hyb_batch_autotune(batch, reps) bind(c, name="hyb_batch_autotune")
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int), value :: reps
     end function
     integer(c_int) function hyb_batch_step(batch, n_iter, res) bind(c, name="hyb_batch_step")
       import :: c_int, c_ptr, hyb_residual
       type(c_ptr), value :: batch
       integer(c_int), value :: n_iter
       type(hyb_residual), intent(out) :: res(*)
     end function
     integer(c_int) function hyb_batch_last_step_ms(batch, ms) bind(c, name="hyb_batch_last_step_ms")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: batch
       real(c_double), intent(out) :: ms
     end function
     integer(c_int) function hyb_batch_launch_count(batch, count) bind(c, name="hyb_batch_launch_count")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: batch
       integer(c_long_long), intent(out) :: count
     end function
     integer(c_int) function hyb_mlp_create(device, seed, net) bind(c, name="hyb_mlp_create")
       import :: c_int, c_ptr, c_long_long
       integer(c_int), value :: device
       integer(c_long_long), value :: seed
       type(c_ptr), intent(out) :: net
     end function
     integer(c_int) function hyb_mlp_destroy(net) bind(c, name="hyb_mlp_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: net
     end function
     type(c_ptr) function hyb_mlp_last_error(net) bind(c, name="hyb_mlp_last_error")
       import :: c_ptr
       type(c_ptr), value :: net
     end function
     integer(c_int) function hyb_mlp_param_count() bind(c, name="hyb_mlp_param_count")
       import :: c_int
     end function
     integer(c_int) function hyb_mlp_get_params(net, w) bind(c, name="hyb_mlp_get_params")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(out) :: w(*)
     end function
     integer(c_int) function hyb_mlp_set_params(net, w) bind(c, name="hyb_mlp_set_params")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(in) :: w(*)
     end function
     integer(c_int) function hyb_mlp_set_norm(net, in_mean, in_std, out_mean, out_std) bind(c, name="hyb_mlp_set_norm")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(in) :: in_mean(8), in_std(8), out_mean(4), out_std(4)
     end function
     integer(c_int) function hyb_mlp_set_data(net, x, y, n) bind(c, name="hyb_mlp_set_data")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(in) :: x(*), y(*)
       integer(c_int), value :: n
     end function
     integer(c_int) function hyb_mlp_train_epoch(net, perm, batch, lr, mean_loss) bind(c, name="hyb_mlp_train_epoch")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       integer(c_int), intent(in) :: perm(*)
       integer(c_int), value :: batch
       real(c_float), value :: lr
       real(c_float), intent(out) :: mean_loss
     end function
     integer(c_int) function hyb_mlp_grad(net, x, y, n, grad, loss) bind(c, name="hyb_mlp_grad")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(in) :: x(*), y(*)
       integer(c_int), value :: n
       real(c_float), intent(out) :: grad(*), loss
     end function
     integer(c_int) function hyb_mlp_predict(net, x, n, y) bind(c, name="hyb_mlp_predict")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float), intent(in) :: x(*)
       integer(c_int), value :: n
       real(c_float), intent(out) :: y(*)
     end function
     integer(c_int) function hyb_mlp_forward_dev(net, x_dev, n, y_dev, stream) bind(c, name="hyb_mlp_forward_dev")
       import :: c_int, c_ptr
       type(c_ptr), value :: net, x_dev, y_dev, stream
       integer(c_int), value :: n
     end function
     integer(c_int) function hyb_mlp_last_ms(net, ms) bind(c, name="hyb_mlp_last_ms")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: net
       real(c_double), intent(out) :: ms
     end function
     integer(c_int) function hyb_mlp_launch_count(net, count) bind(c, name="hyb_mlp_launch_count")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: net
       integer(c_long_long), intent(out) :: count
     end function
     integer(c_int) function hyb_gsis_attach_mlp(ctx, net) bind(c, name="hyb_gsis_attach_mlp")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, net
     end function
     integer(c_int) function hyb_gsis_warm_start(ctx) bind(c, name="hyb_gsis_warm_start")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function hyb_closure_samples(ctx, x, y, cap, n) bind(c, name="hyb_closure_samples")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: ctx
       real(c_float), intent(out) :: x(*), y(*)
       integer(c_int), value :: cap
       integer(c_int), intent(out) :: n
     end function
  end interface
end module hyb_dvm
