! swap_gpu_iface.f90 -- ISO_C_BINDING face of libswap_gpu.so for the
! SWAP Fortran driver.  Two modules:
!
!   swap_gpu_iface   bind(C) interfaces to include/swap_gpu.h and the one
!                    context per MPI rank (swap_gpu_ctx);
!   swap_gpu_calls   wrappers with the reference's subroutine names and
!                    argument lists (gutsp.f, gutsf.f, grid_interp.f,
!                    boundary.f) that forward to the C entries and stop on a
!                    nonzero status, as inputs.f:199 stops on a bad input,
!                    and swap_gpu_init, which creates the context from the
!                    reference's own modules.
!
! Build with the reference's own flags (makefile:1), e.g.
!   mpif90 -i4 -real-size 32 -O2 -c swap_gpu_iface.f90
! and link -L<repo>/swap_gb300/_lib -lswap_gpu.  Real arrays are declared
! real(wp) with wp = kind(1.0), the default real that -real-size selects, and
! swap_gpu_init tells the library that size (swap_dims%real_bytes), so the
! same source serves -real-size 32 (float arrays) and 64 (double).  No
! Fortran compiler exists in the image this file was written in, so it has
! not been compiled here; the C entries it binds are exercised through ctypes
! by the test suite, with 4-byte and 8-byte reals.
module swap_gpu_iface
  use iso_c_binding
  implicit none

  ! The caller's default real: 4 bytes under -real-size 32, 8 under 64.
  integer, parameter :: wp = kind(1.0)

  type, bind(C) :: swap_dims_t
     integer(c_int32_t) :: nx, ny, nz, real_bytes
     integer(c_int64_t) :: ni_max
  end type swap_dims_t

  type, bind(C) :: swap_params_t
     real(c_double) :: dt, alpha, beta, dx, dy, grad_pe
     integer(c_int32_t) :: ntsub, flags
  end type swap_params_t

  type, bind(C) :: swap_coords_t
     type(c_ptr) :: qx, qy, qz, dx_grid, dy_grid, dz_grid
     type(c_ptr) :: dx_cell, dy_cell, dz_cell, xrat, yrat, zrat
  end type swap_coords_t

  type, bind(C) :: swap_sources_t
     integer(c_int64_t) :: seed
     real(c_double) :: ndot, vsw, beta_pu, mrat_pu, delz_ref
     integer(c_int32_t) :: x_open, inflow_ppc
     real(c_double) :: inflow_vth, inflow_ux, inflow_uy, inflow_uz
     real(c_double) :: cloud_N0, cloud_r0, cloud_x, cloud_y, cloud_z, nu_ion, mrat_heavy, beta_heavy
     real(c_double) :: cx_a, cx_b
  end type swap_sources_t

  type, bind(C) :: swap_diag_spec_t
     integer(c_int32_t) :: nt, nout, real_bytes, rank
     real(c_double) :: dtsub_init, vtop, vbottom, mion, m_pu, m_heavy, np_top, np_bottom, b0_top, b0_bottom, &
                       vth_top, vth_bottom
  end type swap_diag_spec_t

  type(c_ptr), save :: swap_gpu_ctx = c_null_ptr
  ! The ion step number for the random draws of res_chex, whose reference
  ! argument list has none: set it to the main loop's m before the call.
  integer(c_int32_t), save :: swap_step = 0

  interface
     integer(c_int) function swap_init(ctx, dims, params, coords) bind(C, name="swap_init")
       import :: c_int, c_ptr, swap_dims_t, swap_params_t, swap_coords_t
       type(c_ptr) :: ctx
       type(swap_dims_t) :: dims
       type(swap_params_t) :: params
       type(swap_coords_t) :: coords
     end function swap_init
     integer(c_int) function swap_finalize(ctx) bind(C, name="swap_finalize")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_finalize
     type(c_ptr) function swap_last_error(ctx) bind(C, name="swap_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function swap_last_error
     integer(c_int) function swap_bind_particles(ctx, xp, vp, vp1, mrat, beta_p, ijkp, ni_tot) &
          bind(C, name="swap_bind_particles")
       import :: c_int, c_ptr, c_double, c_int32_t, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*), vp(*), vp1(*), mrat(*), beta_p(*)
       integer(c_int32_t) :: ijkp(*), ni_tot
     end function swap_bind_particles
     integer(c_int) function swap_bind_fields(ctx, b0, b1, b12, b1p2, bt, btc, np, up, aj, E, nu) &
          bind(C, name="swap_bind_fields")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b0(*), b1(*), b12(*), b1p2(*), bt(*), btc(*), np(*), up(*), aj(*), E(*), nu(*)
     end function swap_bind_fields
     integer(c_int) function swap_bind_array(ctx, a, nbytes) bind(C, name="swap_bind_array")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx, a
       integer(c_int64_t), value :: nbytes
     end function swap_bind_array
     integer(c_int) function swap_sync_to_host(ctx, a) bind(C, name="swap_sync_to_host")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, a
     end function swap_sync_to_host
     integer(c_int) function swap_mark_host_dirty(ctx, a) bind(C, name="swap_mark_host_dirty")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, a
     end function swap_mark_host_dirty
     integer(c_int) function swap_set_host_direct(ctx, on) bind(C, name="swap_set_host_direct")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: on
     end function swap_set_host_direct
     integer(c_int) function swap_transfer_bytes(ctx, h2d, d2h, reset) bind(C, name="swap_transfer_bytes")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t), intent(out) :: h2d, d2h
       integer(c_int), value :: reset
     end function swap_transfer_bytes
     ! --- gutsp.f ---
     integer(c_int) function c_get_interp_weights(ctx, xp) bind(C, name="swap_get_interp_weights")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*)
     end function c_get_interp_weights
     integer(c_int) function c_update_np(ctx, np) bind(C, name="swap_update_np")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: np(*)
     end function c_update_np
     integer(c_int) function c_update_up(ctx, vp, np, up) bind(C, name="swap_update_up")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: vp(*), np(*), up(*)
     end function c_update_up
     integer(c_int) function c_extrapol_up(ctx, up, vp, vp1, np) bind(C, name="swap_extrapol_up")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: up(*), vp(*), vp1(*), np(*)
     end function c_extrapol_up
     integer(c_int) function c_get_Ep(ctx, Ep, aj, np, up, btc, nu) bind(C, name="swap_get_Ep")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: Ep(*), aj(*), np(*), up(*), btc(*), nu(*)
     end function c_get_Ep
     integer(c_int) function c_get_vplus_vminus(ctx, Ep, btc, vp, vplus, vminus) bind(C, name="swap_get_vplus_vminus")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: Ep(*), btc(*), vp(*), vplus(*), vminus(*)
     end function c_get_vplus_vminus
     integer(c_int) function c_improve_up(ctx, vp1, vplus, vminus, up, np) bind(C, name="swap_improve_up")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: vp1(*), vplus(*), vminus(*), up(*), np(*)
     end function c_improve_up
     integer(c_int) function c_get_vp_final(ctx, Ep, vp, vp1, vplus) bind(C, name="swap_get_vp_final")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: Ep(*), vp(*), vp1(*), vplus(*)
     end function c_get_vp_final
     integer(c_int) function c_move_ion_half(ctx, xp, vp, vp1, input_p) bind(C, name="swap_move_ion_half")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*), vp(*), vp1(*), input_p(*)
     end function c_move_ion_half
     ! --- gutsf.f / grid_interp.f / boundary.f ---
     integer(c_int) function c_curlB(ctx, bt, np, aj) bind(C, name="swap_curlB")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: bt(*), np(*), aj(*)
     end function c_curlB
     integer(c_int) function c_edge_to_center(ctx, bt, btc) bind(C, name="swap_edge_to_center")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: bt(*), btc(*)
     end function c_edge_to_center
     integer(c_int) function c_face_to_center(ctx, v, vc) bind(C, name="swap_face_to_center")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: v(*), vc(*)
     end function c_face_to_center
     integer(c_int) function c_get_E(ctx, E, b0, bt, aj, up, np, nu) bind(C, name="swap_get_E")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: E(*), b0(*), bt(*), aj(*), up(*), np(*), nu(*)
     end function c_get_E
     integer(c_int) function c_predict_B(ctx, b0, b1, b12, b1p2, bt, E, aj, up, np, nu, dtsub) &
          bind(C, name="swap_predict_B")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b0(*), b1(*), b12(*), b1p2(*), bt(*), E(*), aj(*), up(*), np(*), nu(*)
       real(c_double), value :: dtsub
     end function c_predict_B
     integer(c_int) function c_correct_B(ctx, b0, b1, b1p2, E, aj, up, np, nu, dtsub) bind(C, name="swap_correct_B")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b0(*), b1(*), b1p2(*), E(*), aj(*), up(*), np(*), nu(*)
       real(c_double), value :: dtsub
     end function c_correct_B
     integer(c_int) function c_f_update_tlev(ctx, b1, b12, b1p2, bt, b0) bind(C, name="swap_f_update_tlev")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b1(*), b12(*), b1p2(*), bt(*), b0(*)
     end function c_f_update_tlev
     integer(c_int) function c_check_time_step(ctx, bt, np, dtsub, ntf) bind(C, name="swap_check_time_step")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: bt(*), np(*)
       real(c_double) :: dtsub, ntf
     end function c_check_time_step
     integer(c_int) function c_periodic(ctx, b) bind(C, name="swap_periodic")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b(*)
     end function c_periodic
     integer(c_int) function c_periodic_scalar(ctx, b) bind(C, name="swap_periodic_scalar")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b(*)
     end function c_periodic_scalar
     integer(c_int) function swap_set_sources(ctx, src, step0) bind(C, name="swap_set_sources")
       import :: c_int, c_ptr, c_int64_t, swap_sources_t
       type(c_ptr), value :: ctx
       type(swap_sources_t) :: src
       integer(c_int64_t), value :: step0
     end function swap_set_sources
     integer(c_int) function c_Ionize_sw_mp(ctx, np, vp, vp1, xp, m_tstep, input_p, up) &
          bind(C, name="swap_Ionize_sw_mp")
       import :: c_int, c_ptr, c_double, c_int32_t, wp
       type(c_ptr), value :: ctx
       real(wp) :: np(*), vp(*), vp1(*), xp(*), input_p(*), up(*)
       integer(c_int32_t), value :: m_tstep
     end function c_Ionize_sw_mp
     integer(c_int) function c_remove_ion(ctx, xp, vp, vp1, ion_l) bind(C, name="swap_remove_ion")
       import :: c_int, c_ptr, c_double, c_int32_t, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*), vp(*), vp1(*)
       integer(c_int32_t), value :: ion_l
     end function c_remove_ion
     integer(c_int) function c_res_chex(ctx, xp, vp, m_tstep, count) bind(C, name="swap_res_chex")
       import :: c_int, c_ptr, c_double, c_int32_t, c_int64_t, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*), vp(*)
       integer(c_int32_t), value :: m_tstep
       integer(c_int64_t) :: count
     end function c_res_chex
     integer(c_int) function c_update_rho(ctx, mnp) bind(C, name="swap_update_rho")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: mnp(*)
     end function c_update_rho
     integer(c_int) function c_get_temperature(ctx, xp, vp, np, temp_p) bind(C, name="swap_get_temperature")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: xp(*), vp(*), np(*), temp_p(*)
     end function c_get_temperature
     ! ---- whole steps (maind.f:379-484), the fused FP64 path
     integer(c_int) function swap_ion_step(ctx) bind(C, name="swap_ion_step")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_ion_step
     integer(c_int) function swap_ion_step_pre(ctx) bind(C, name="swap_ion_step_pre")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_ion_step_pre
     integer(c_int) function swap_field_subcycles(ctx) bind(C, name="swap_field_subcycles")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_field_subcycles
     integer(c_int) function swap_ion_step_post(ctx) bind(C, name="swap_ion_step_post")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_ion_step_post
     integer(c_int) function swap_run(ctx, nsteps) bind(C, name="swap_run")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: nsteps
     end function swap_run
     integer(c_int) function swap_energy(ctx, out) bind(C, name="swap_energy")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double) :: out(4)
     end function swap_energy
     integer(c_int) function swap_sync_to_device(ctx, a) bind(C, name="swap_sync_to_device")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, a
     end function swap_sync_to_device
     integer(c_int) function swap_max_abs_divB(ctx, b, out) bind(C, name="swap_max_abs_divB")
       import :: c_int, c_ptr, c_double, wp
       type(c_ptr), value :: ctx
       real(wp) :: b(*)
       real(c_double) :: out
     end function swap_max_abs_divB
     integer(c_int) function swap_check_finite(ctx) bind(C, name="swap_check_finite")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_check_finite
     ! ---- the FP32 form: n whole steps on the device
     integer(c_int) function swap_f32_begin(ctx) bind(C, name="swap_f32_begin")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_f32_begin
     integer(c_int) function swap_f32_run(ctx, nsteps) bind(C, name="swap_f32_run")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: nsteps
     end function swap_f32_run
     integer(c_int) function swap_f32_end(ctx) bind(C, name="swap_f32_end")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_f32_end
     integer(c_int) function swap_f32_energy(ctx, out) bind(C, name="swap_f32_energy")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double) :: out(4)
     end function swap_f32_energy
     integer(c_int) function swap_f32_count(ctx, n) bind(C, name="swap_f32_count")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t) :: n
     end function swap_f32_count
     integer(c_int) function swap_f32_far_movers(ctx, n) bind(C, name="swap_f32_far_movers")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t) :: n
     end function swap_f32_far_movers
     ! ---- reproducible FP64 runs (fixed-point deposits), e.g. around a restart
     integer(c_int) function swap_set_deterministic(ctx, on) bind(C, name="swap_set_deterministic")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: on
     end function swap_set_deterministic
     ! ---- sources and sinks without a reference argument list of their own
     integer(c_int) function swap_inflow_x(ctx, m_tstep) bind(C, name="swap_inflow_x")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: m_tstep
     end function swap_inflow_x
     integer(c_int) function swap_ionize_cloud(ctx, m_tstep) bind(C, name="swap_ionize_cloud")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: m_tstep
     end function swap_ionize_cloud
     integer(c_int) function swap_remove_outflow_x(ctx) bind(C, name="swap_remove_outflow_x")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_remove_outflow_x
     integer(c_int) function swap_chex_count(ctx, n) bind(C, name="swap_chex_count")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t) :: n
     end function swap_chex_count
     integer(c_int) function swap_set_mion(ctx, mion) bind(C, name="swap_set_mion")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: mion
     end function swap_set_mion
     ! ---- diagnostics writer (maind.f:237-358, 498-573)
     integer(c_int) function swap_diag_open(ctx, out_dir, spec) bind(C, name="swap_diag_open")
       import :: c_int, c_ptr, c_char, swap_diag_spec_t
       type(c_ptr), value :: ctx
       character(kind=c_char) :: out_dir(*)
       type(swap_diag_spec_t) :: spec
     end function swap_diag_open
     integer(c_int) function swap_diag_step(ctx, m) bind(C, name="swap_diag_step")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: m
     end function swap_diag_step
     integer(c_int) function swap_diag_close(ctx) bind(C, name="swap_diag_close")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function swap_diag_close
     ! ---- the learned field-subcycle surrogate of the FP32 form
     integer(c_int) function swap_surrogate_create(net, seed, max_samples) bind(C, name="swap_surrogate_create")
       import :: c_int, c_ptr, c_int64_t, c_int32_t
       type(c_ptr) :: net
       integer(c_int64_t), value :: seed
       integer(c_int32_t), value :: max_samples
     end function swap_surrogate_create
     integer(c_int) function swap_surrogate_destroy(net) bind(C, name="swap_surrogate_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: net
     end function swap_surrogate_destroy
     integer(c_int) function swap_surrogate_collect(net, ctx, nsteps) bind(C, name="swap_surrogate_collect")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: net, ctx
       integer(c_int32_t), value :: nsteps
     end function swap_surrogate_collect
     integer(c_int) function swap_surrogate_train(net, epochs, lr, loss) bind(C, name="swap_surrogate_train")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: net
       integer(c_int32_t), value :: epochs
       real(c_double), value :: lr
       real(c_double) :: loss
     end function swap_surrogate_train
     integer(c_int) function swap_surrogate_attach(ctx, net, judge_every, bound) bind(C, name="swap_surrogate_attach")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: ctx, net
       integer(c_int32_t), value :: judge_every
       real(c_double), value :: bound
     end function swap_surrogate_attach
     integer(c_int) function swap_surrogate_set_db_bound(ctx, bound_db) bind(C, name="swap_surrogate_set_db_bound")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: bound_db
     end function swap_surrogate_set_db_bound
     integer(c_int) function swap_surrogate_stats(ctx, out) bind(C, name="swap_surrogate_stats")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double) :: out(5)
     end function swap_surrogate_stats
     integer(c_int) function swap_checkpoint_write(ctx, path) bind(C, name="swap_checkpoint_write")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char) :: path(*)
     end function swap_checkpoint_write
     integer(c_int) function swap_checkpoint_read(ctx, path) bind(C, name="swap_checkpoint_read")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char) :: path(*)
     end function swap_checkpoint_read
  end interface

contains

  ! Stop with the library's message on a nonzero status (the reference's
  ! own error style, inputs.f:199).
  subroutine swap_check(ierr, where)
    integer(c_int), intent(in) :: ierr
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (ierr == 0) return
    call c_f_pointer(swap_last_error(swap_gpu_ctx), msg, [256])
    n = 0
    do while (n < 256)
       if (msg(n + 1) == c_null_char) exit
       n = n + 1
    end do
    write(*,*) 'swap_gpu error in ', where, ': ', ierr, ' ', msg(1:n)
    stop
  end subroutine swap_check

end module swap_gpu_iface


! Wrappers with the reference names.  The makefile links this module's
! object in place of the bodies of the same subroutines in gutsp.f,
! gutsf.f, grid_interp.f, boundary.f and, for the sources, chem_rates.f;
! maind.f is unchanged.  Implicit state (dt, dtsub, ijkp, wght) is held by the context.
module swap_gpu_calls
  use iso_c_binding
  use swap_gpu_iface
  use global, only: dtsub, ntf   ! /timestep/ (global.f:76-77)
  implicit none
  ! double copies of /coords/ (global.f:16-27) for swap_coords, kept for the
  ! context's lifetime
  real(c_double), allocatable, target, save :: co8(:, :)
contains
  ! Create the context from the reference's modules: dimensions.f (nx, ny,
  ! nz, Ni_max), inputs.f (dt, alpha, dx, dy, ntsub) and global.f (beta and
  ! the /coords/ arrays), with real_bytes = the size of the REAL this module is compiled with.
  ! Call after grd7 and initparameters, before the main loop (maind.f:372).
  subroutine swap_gpu_init()
    use dimensions, only: nx, ny, nz, Ni_max
    use inputs, only: dt, alpha, dx, dy, ntsub
    use global, only: beta, qx, qy, qz, dx_grid, dy_grid, dz_grid, dx_cell, dy_cell, dz_cell, xrat, yrat, zrat
    type(swap_dims_t) :: d
    type(swap_params_t) :: p
    type(swap_coords_t) :: co
    integer :: nmax
    nmax = max(nx, ny, nz)
    allocate(co8(nmax, 12))
    co8 = 0
    co8(1:nx, 1) = qx;      co8(1:ny, 2) = qy;      co8(1:nz, 3) = qz
    co8(1:nx, 4) = dx_grid; co8(1:ny, 5) = dy_grid; co8(1:nz, 6) = dz_grid
    co8(1:nx, 7) = dx_cell; co8(1:ny, 8) = dy_cell; co8(1:nz, 9) = dz_cell
    co8(1:nx, 10) = xrat;   co8(1:ny, 11) = yrat;   co8(1:nz, 12) = zrat
    co%qx = c_loc(co8(1, 1)); co%qy = c_loc(co8(1, 2)); co%qz = c_loc(co8(1, 3))
    co%dx_grid = c_loc(co8(1, 4)); co%dy_grid = c_loc(co8(1, 5)); co%dz_grid = c_loc(co8(1, 6))
    co%dx_cell = c_loc(co8(1, 7)); co%dy_cell = c_loc(co8(1, 8)); co%dz_cell = c_loc(co8(1, 9))
    co%xrat = c_loc(co8(1, 10)); co%yrat = c_loc(co8(1, 11)); co%zrat = c_loc(co8(1, 12))
    d%nx = nx; d%ny = ny; d%nz = nz
    d%real_bytes = storage_size(1.0_wp) / 8
    d%ni_max = Ni_max
    p%dt = dt; p%alpha = alpha; p%beta = beta; p%dx = dx; p%dy = dy
    p%grad_pe = 0
    p%ntsub = nint(ntsub)
    p%flags = 0
    call swap_check(swap_init(swap_gpu_ctx, d, p, co), 'swap_init')
  end subroutine swap_gpu_init

  subroutine get_interp_weights(xp)
    real(wp) :: xp(*)
    call swap_check(c_get_interp_weights(swap_gpu_ctx, xp), 'get_interp_weights')
  end subroutine get_interp_weights
  subroutine update_np(np)
    real(wp) :: np(*)
    call swap_check(c_update_np(swap_gpu_ctx, np), 'update_np')
  end subroutine update_np
  subroutine update_up(vp, np, up)
    real(wp) :: vp(*), np(*), up(*)
    call swap_check(c_update_up(swap_gpu_ctx, vp, np, up), 'update_up')
  end subroutine update_up
  subroutine extrapol_up(up, vp, vp1, np)
    real(wp) :: up(*), vp(*), vp1(*), np(*)
    call swap_check(c_extrapol_up(swap_gpu_ctx, up, vp, vp1, np), 'extrapol_up')
  end subroutine extrapol_up
  subroutine get_Ep(Ep, aj, np, up, btc, nu)
    real(wp) :: Ep(*), aj(*), np(*), up(*), btc(*), nu(*)
    call swap_check(c_get_Ep(swap_gpu_ctx, Ep, aj, np, up, btc, nu), 'get_Ep')
  end subroutine get_Ep
  subroutine get_vplus_vminus(Ep, btc, vp, vplus, vminus)
    real(wp) :: Ep(*), btc(*), vp(*), vplus(*), vminus(*)
    call swap_check(c_get_vplus_vminus(swap_gpu_ctx, Ep, btc, vp, vplus, vminus), 'get_vplus_vminus')
  end subroutine get_vplus_vminus
  subroutine improve_up(vp1, vplus, vminus, up, np)
    real(wp) :: vp1(*), vplus(*), vminus(*), up(*), np(*)
    call swap_check(c_improve_up(swap_gpu_ctx, vp1, vplus, vminus, up, np), 'improve_up')
  end subroutine improve_up
  subroutine get_vp_final(Ep, vp, vp1, vplus)
    real(wp) :: Ep(*), vp(*), vp1(*), vplus(*)
    call swap_check(c_get_vp_final(swap_gpu_ctx, Ep, vp, vp1, vplus), 'get_vp_final')
  end subroutine get_vp_final
  subroutine move_ion_half(xp, vp, vp1, input_p)
    real(wp) :: xp(*), vp(*), vp1(*), input_p(*)
    call swap_check(c_move_ion_half(swap_gpu_ctx, xp, vp, vp1, input_p), 'move_ion_half')
  end subroutine move_ion_half
  subroutine curlB(b1, np, aj)
    real(wp) :: b1(*), np(*), aj(*)
    call swap_check(c_curlB(swap_gpu_ctx, b1, np, aj), 'curlB')
  end subroutine curlB
  subroutine edge_to_center(bt, btc)
    real(wp) :: bt(*), btc(*)
    call swap_check(c_edge_to_center(swap_gpu_ctx, bt, btc), 'edge_to_center')
  end subroutine edge_to_center
  subroutine face_to_center(v, vc)
    real(wp) :: v(*), vc(*)
    call swap_check(c_face_to_center(swap_gpu_ctx, v, vc), 'face_to_center')
  end subroutine face_to_center
  subroutine get_E(E, b0, bt, aj, up, np, nu)
    real(wp) :: E(*), b0(*), bt(*), aj(*), up(*), np(*), nu(*)
    call swap_check(c_get_E(swap_gpu_ctx, E, b0, bt, aj, up, np, nu), 'get_E')
  end subroutine get_E
  subroutine predict_B(b0, b1, b12, b1p2, bt, E, aj, up, np, nu)
    real(wp) :: b0(*), b1(*), b12(*), b1p2(*), bt(*), E(*), aj(*), up(*), np(*), nu(*)
    call swap_check(c_predict_B(swap_gpu_ctx, b0, b1, b12, b1p2, bt, E, aj, up, np, nu, real(dtsub, c_double)), &
                    'predict_B')
  end subroutine predict_B
  subroutine correct_B(b0, b1, b1p2, E, aj, up, np, nu)
    real(wp) :: b0(*), b1(*), b1p2(*), E(*), aj(*), up(*), np(*), nu(*)
    call swap_check(c_correct_B(swap_gpu_ctx, b0, b1, b1p2, E, aj, up, np, nu, real(dtsub, c_double)), &
                    'correct_B')
  end subroutine correct_B
  subroutine f_update_tlev(b1, b12, b1p2, bt, b0)
    real(wp) :: b1(*), b12(*), b1p2(*), bt(*), b0(*)
    call swap_check(c_f_update_tlev(swap_gpu_ctx, b1, b12, b1p2, bt, b0), 'f_update_tlev')
  end subroutine f_update_tlev
  subroutine check_time_step(bt, np)
    real(wp) :: bt(*), np(*)
    real(c_double) :: d8, n8   ! the C entry's scalars are double at either real size
    d8 = dtsub
    n8 = ntf
    call swap_check(c_check_time_step(swap_gpu_ctx, bt, np, d8, n8), 'check_time_step')
    dtsub = d8
    ntf = n8
  end subroutine check_time_step
  subroutine periodic(b)
    real(wp) :: b(*)
    call swap_check(c_periodic(swap_gpu_ctx, b), 'periodic')
  end subroutine periodic
  subroutine periodic_scalar(b)
    real(wp) :: b(*)
    call swap_check(c_periodic_scalar(swap_gpu_ctx, b), 'periodic_scalar')
  end subroutine periodic_scalar
  subroutine Ionize_sw_mp(np, vp, vp1, xp, m_tstep, input_p, up)
    real(wp) :: np(*), vp(*), vp1(*), xp(*), input_p(*), up(*)
    integer :: m_tstep
    call swap_check(c_Ionize_sw_mp(swap_gpu_ctx, np, vp, vp1, xp, int(m_tstep, c_int32_t), input_p, up), &
                    'Ionize_sw_mp')
  end subroutine Ionize_sw_mp
  subroutine remove_ion(xp, vp, vp1, ion_l)
    real(wp) :: xp(*), vp(*), vp1(*)
    integer :: ion_l
    call swap_check(c_remove_ion(swap_gpu_ctx, xp, vp, vp1, int(ion_l, c_int32_t)), 'remove_ion')
  end subroutine remove_ion
  subroutine res_chex(xp, vp)
    real(wp) :: xp(*), vp(*)
    integer(c_int64_t) :: n
    call swap_check(c_res_chex(swap_gpu_ctx, xp, vp, swap_step, n), 'res_chex')
  end subroutine res_chex
  subroutine update_rho(mnp)
    real(wp) :: mnp(*)
    call swap_check(c_update_rho(swap_gpu_ctx, mnp), 'update_rho')
  end subroutine update_rho
  subroutine get_temperature(xp, vp, np, temp_p)
    real(wp) :: xp(*), vp(*), np(*), temp_p(*)
    call swap_check(c_get_temperature(swap_gpu_ctx, xp, vp, np, temp_p), 'get_temperature')
  end subroutine get_temperature
end module swap_gpu_calls
