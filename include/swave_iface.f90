! swave_iface.f90 - Fortran 2003 (ISO_C_BINDING) interface to libswave.so.
!
! The reference's own Fortran-to-C boundary passes every argument by
! address to trailing-underscore C symbols (libs/libwave/bandpass.c:72,187,
! called from libs/libwave/Bandpass.f90:89-149).  This module binds the
! C-ABI of include/swave.h by name instead: bind(C) derived types with the
! same field order and kinds as the C structs, and one interface per entry
! point, with scalars passed by value where the C prototype does.  Host
! arrays keep the reference's layout (a(nz,nx,ny), traces trace(nt) per
! receiver concatenated); opaque handles are type(c_ptr).
!
! A driver adds `use swave_iface` and replaces, e.g., the two
! propagator_acoustic calls of RTM_to_memory
! (progs/rtm/to_disk_to_memory_RTM.f90:358-492) with one sw_rtm call.
module swave_iface
  use iso_c_binding
  implicit none

  ! sw_status
  integer(c_int), parameter :: SW_OK = 0, SW_BAD_PARAM = 1, SW_OOM_ADMISSION = 2, &
       SW_TIMEOUT = 3, SW_NUMERIC = 4, SW_CUDA_ERR = 5, SW_UNSUPPORTED = 6
  ! sw_fd_scheme, sw_injection, sw_extraction, sw_imaging
  integer(c_int), parameter :: SW_FD_FORWARD = 0, SW_FD_ADJOINT = 1
  integer(c_int), parameter :: SW_INJ_NONE = 0, SW_INJ_SINC = 1, SW_INJ_SIMPLE = 2, &
       SW_INJ_LSRTM_SINC = 3
  integer(c_int), parameter :: SW_EXT_NONE = 0, SW_EXT_SINC = 1, SW_EXT_SIMPLE_AFWI = 2, &
       SW_EXT_LSRTM_SINC = 3, SW_EXT_SINC_AFWI = 4
  integer(c_int), parameter :: SW_IMG_NONE = 0, SW_IMG_RTM = 1, SW_IMG_LSRTM = 2, &
       SW_IMG_AFWI = 3, SW_IMG_BORN = 4, SW_IMG_AFWI_RHO = 5
  ! data norms (invparam%dat_nrm_type, libs/libinv/Inversion_types.f90:61-68)
  integer(c_int), parameter :: SW_NRM_L1 = 1, SW_NRM_L2 = 2, SW_NRM_CAUCHY = 3, &
       SW_NRM_HYPERBOLIC = 4, SW_NRM_HUBER = 12

  ! GeneralParam subset (libs/libwave/GeneralParamTypes.f90:9-48)
  type, bind(C) :: sw_genpar
     integer(c_int) :: twoD
     integer(c_int) :: nz, nx, ny
     real(c_float)  :: dz, dx, dy
     real(c_float)  :: oz, ox, oy
     real(c_float)  :: dt
     integer(c_int) :: nt
     integer(c_int) :: ntaper
     integer(c_int) :: lsinc
     integer(c_int) :: snapi
     integer(c_int) :: surf_type, shot_type, rec_type
     real(c_float)  :: fmax
  end type sw_genpar

  ! one propagator_acoustic call (libs/libwave/Propagator.f90:27-120)
  type, bind(C) :: sw_prop_desc
     type(sw_genpar) :: g
     integer(c_int)  :: tmin, tmax, tstep
     integer(c_int)  :: fd_scheme
     integer(c_int)  :: injection
     integer(c_int)  :: extraction
     integer(c_int)  :: extract_wave
     integer(c_int)  :: imaging
  end type sw_prop_desc

  type, bind(C) :: sw_prop_io
     type(c_ptr)    :: vel
     integer(c_int) :: nsou
     type(c_ptr)    :: sou_coord
     type(c_ptr)    :: sou_trace
     integer(c_int) :: nrec
     type(c_ptr)    :: rec_coord
     type(c_ptr)    :: rec_trace
     type(c_ptr)    :: wave
     type(c_ptr)    :: image
     type(c_ptr)    :: illum
     type(c_ptr)    :: ref
     type(c_ptr)    :: final_u2
     type(c_ptr)    :: rho          ! c_null_ptr unless withRho
     type(c_ptr)    :: image2       ! imagesmall_nparam(:,:,:,2) for SW_IMG_AFWI_RHO
  end type sw_prop_io

  ! one shot of a multi-shot RTM job
  type, bind(C) :: sw_shot
     real(c_float)  :: sou_coord(3)
     integer(c_int) :: nrec
     type(c_ptr)    :: rec_coord
     type(c_ptr)    :: data
     integer(c_int) :: nt
  end type sw_shot

  ! extract_coord_source_receiver_patch (ExtractPadModel.f90:19-85)
  type, bind(C) :: sw_window
     real(c_float)  :: oxw, oyw, endx, endy
     integer(c_int) :: nxw, nyw
  end type sw_window

  ! one shot of compute_fct_gdt
  type, bind(C) :: sw_fwi_shot
     real(c_float)  :: sou_coord(3)
     integer(c_int) :: nrec
     type(c_ptr)    :: rec_coord
     type(c_ptr)    :: dobs
     type(c_ptr)    :: mute         ! c_null_ptr = no mute
     type(c_ptr)    :: resid        ! c_null_ptr = residual not returned
  end type sw_fwi_shot

  type, bind(C) :: sw_fwi_desc
     type(sw_genpar) :: g
     real(c_float)   :: aperture_x, aperture_y
     real(c_float)   :: illu_pow
     integer(c_int)  :: smooth_rect1, smooth_rect2, smooth_rect3
     integer(c_int)  :: smooth_doz, smooth_dox, smooth_doy
     integer(c_int)  :: checkpoint_snaps
     integer(c_int)  :: dat_nrm_type   ! invparam%dat_nrm_type
     real(c_float)   :: dat_thresh     ! invparam%dat_thresh
     integer(c_int)  :: revolve_slots
  end type sw_fwi_desc

  ! SparseRegParam settings (libs/libwave/Sparse_regularization.f90)
  type, bind(C) :: sw_reg_desc
     integer(c_int) :: nz, nx, ny
     integer(c_int) :: wantreg, wantlog
     integer(c_int) :: derivdx, derivdy, derivdz, log_z_plus
     integer(c_int) :: ntaperz, ntaperx, ntapery
     integer(c_int) :: mod_nrm_type, hin_nrm_type
     integer(c_int) :: compute_eps, compute_eps_log
     real(c_float)  :: ratio, ratio_log
     type(c_ptr)    :: zweight        ! c_loc(sparseparam%zweight) or c_null_ptr
  end type sw_reg_desc

  type, bind(C) :: sw_reg_state
     real(c_float) :: eps, eps_log
     real(c_float) :: mod_thresh, hin_thresh
  end type sw_reg_state

  ! LBFGSOC / MCSRCHOC saved scalars (LbfgsDat.dat, McsrchDat.dat order)
  type, bind(C) :: sw_lbfgs_oc_state
     real(c_double) :: gtol, one, zero, gnorm, stp1, ftol, stpmin
     real(c_double) :: stpmax, stp, ys, yy, sq, yr, beta, xnorm
     integer(c_int) :: mp, lp, iter, nfun, point, ispt, iypt, maxfev, info
     integer(c_int) :: bound, npt, cp, i, nfev, inmc, iycn, iscn
     integer(c_int) :: finish
     integer(c_int) :: infoc, j
     integer(c_int) :: brackt, stage1
     real(c_double) :: dg, dgm, dginit, dgtest, dgx, dgxm, dgy, dgym
     real(c_double) :: finit, ftest1, fm, fx, fxm, fy, fym, stx, sty
     real(c_double) :: stmin, stmax, width, width1
  end type sw_lbfgs_oc_state

  type, bind(C) :: sw_lbfgs_oc_desc
     integer(c_int) :: n, m, nparam
     type(c_ptr)    :: xmin, xmax       ! c_loc of nparam doubles each
     integer(c_int) :: lbfgs_type, bound_type, stp1_opt
     real(c_double) :: step_init, eps, xtol
  end type sw_lbfgs_oc_desc

  type, bind(C) :: sw_tuning
     integer(c_int) :: step_kernel
     integer(c_int) :: tile_z
     integer(c_int) :: tile_x
     integer(c_int) :: tile_y
     integer(c_int) :: graph_chunk
     integer(c_int) :: use_graph
  end type sw_tuning

  type, bind(C) :: sw_stats
     integer(c_int64_t) :: launches_total
     integer(c_int64_t) :: launches_step
     integer(c_int64_t) :: points_updated
     real(c_double)     :: step_kernel_ms
     integer(c_int64_t) :: step_kernel_timed
     integer(c_int64_t) :: step_bytes
     integer(c_int64_t) :: steps_forward
     integer(c_int64_t) :: steps_backward
     integer(c_int64_t) :: ckpt_advances
     real(c_double)     :: cnn_conv_ms
     integer(c_int64_t) :: cnn_conv_timed
     integer(c_int64_t) :: cnn_conv_bytes
     integer(c_int64_t) :: cnn_conv_flops
  end type sw_stats

  interface
     ! ---- context -----------------------------------------------------------
     integer(c_int) function sw_ctx_create(device, ctx) bind(C, name="sw_ctx_create")
       import :: c_int, c_ptr
       integer(c_int), value :: device
       type(c_ptr)           :: ctx
     end function
     integer(c_int) function sw_ctx_destroy(ctx) bind(C, name="sw_ctx_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function sw_last_error(ctx) bind(C, name="sw_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function sw_version() bind(C, name="sw_version")
       import :: c_ptr
     end function
     integer(c_int) function sw_vel_check(g, vel, courant, samplerate) &
          bind(C, name="sw_vel_check")
       import :: c_int, c_float, sw_genpar
       type(sw_genpar) :: g
       real(c_float)   :: vel(*), courant, samplerate
     end function
     ! ---- propagation and operator drivers ------------------------------------
     integer(c_int) function sw_propagate(ctx, d, io) bind(C, name="sw_propagate")
       import :: c_int, c_ptr, sw_prop_desc, sw_prop_io
       type(c_ptr), value  :: ctx
       type(sw_prop_desc)  :: d
       type(sw_prop_io)    :: io
     end function
     integer(c_int) function sw_modeling(ctx, g, vel, sou, wav, nrec, rec, dat, final_u2) &
          bind(C, name="sw_modeling")
       import :: c_int, c_ptr, c_float, sw_genpar
       type(c_ptr), value    :: ctx
       type(sw_genpar)       :: g
       real(c_float)         :: vel(*), sou(3), wav(*), rec(*), dat(*)
       integer(c_int), value :: nrec
       type(c_ptr), value    :: final_u2    ! c_null_ptr or c_loc of the padded u2
     end function
     integer(c_int) function sw_rtm(ctx, g, vel, sou, wav, nrec, rec, dat, img, ill) &
          bind(C, name="sw_rtm")
       import :: c_int, c_ptr, c_float, sw_genpar
       type(c_ptr), value    :: ctx
       type(sw_genpar)       :: g
       real(c_float)         :: vel(*), sou(3), wav(*), rec(*), dat(*), img(*), ill(*)
       integer(c_int), value :: nrec
     end function
     integer(c_int) function sw_born(ctx, g, vel, ref, sou, wav, nrec, rec, dat) &
          bind(C, name="sw_born")
       import :: c_int, c_ptr, c_float, sw_genpar
       type(c_ptr), value    :: ctx
       type(sw_genpar)       :: g
       real(c_float)         :: vel(*), ref(*), sou(3), wav(*), rec(*), dat(*)
       integer(c_int), value :: nrec
     end function
     integer(c_int) function sw_lsrtm(ctx, g, vel, sou, wav, nrec, rec, dat, img, ill) &
          bind(C, name="sw_lsrtm")
       import :: c_int, c_ptr, c_float, sw_genpar
       type(c_ptr), value    :: ctx
       type(sw_genpar)       :: g
       real(c_float)         :: vel(*), sou(3), wav(*), rec(*), dat(*), img(*), ill(*)
       integer(c_int), value :: nrec
     end function
     integer(c_int) function sw_born_wavelet(wav, nt, dt) bind(C, name="sw_born_wavelet")
       import :: c_int, c_float
       real(c_float)         :: wav(*)
       integer(c_int), value :: nt
       real(c_float), value  :: dt
     end function
     integer(c_int) function sw_bandpass(ctx, ntr, nt, dt, flo, fhi, nplo, nphi, phase, &
          traces) bind(C, name="sw_bandpass")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value    :: ctx
       integer(c_int), value :: ntr, nt
       real(c_float), value  :: dt, flo, fhi
       integer(c_int), value :: nplo, nphi, phase
       real(c_float)         :: traces(*)
     end function
     integer(c_int) function sw_mute_mask(nrec, nt, dt, ot, sou, rec, v0, v1, t0, t1, &
          tramp, mask) bind(C, name="sw_mute_mask")
       import :: c_int, c_float
       integer(c_int), value :: nrec, nt
       real(c_float), value  :: dt, ot
       real(c_float)         :: sou(3), rec(*)
       real(c_float), value  :: v0, v1, t0, t1, tramp
       real(c_float)         :: mask(*)
     end function
     integer(c_int) function sw_rho_wavelet(wav, nt, lsinc) bind(C, name="sw_rho_wavelet")
       import :: c_int, c_float
       real(c_float)         :: wav(*)
       integer(c_int), value :: nt, lsinc
     end function
     ! ---- multi-shot RTM job ---------------------------------------------------
     integer(c_int) function sw_rtm_job_create(ctx, model, apx, apy, vel, wav, nshot, &
          shots, job) bind(C, name="sw_rtm_job_create")
       import :: c_int, c_ptr, c_float, sw_genpar, sw_shot
       type(c_ptr), value    :: ctx
       type(sw_genpar)       :: model
       real(c_float), value  :: apx, apy
       real(c_float)         :: vel(*), wav(*)
       integer(c_int), value :: nshot
       type(sw_shot)         :: shots(*)
       type(c_ptr)           :: job
     end function
     integer(c_int) function sw_rtm_job_set_batch(job, max_shots, mem_fraction) &
          bind(C, name="sw_rtm_job_set_batch")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: job
       integer(c_int), value :: max_shots
       real(c_double), value :: mem_fraction
     end function
     integer(c_int) function sw_rtm_job_run(job, first, count) bind(C, name="sw_rtm_job_run")
       import :: c_int, c_ptr
       type(c_ptr), value    :: job
       integer(c_int), value :: first, count
     end function
     integer(c_int) function sw_rtm_job_model(job, first, count, dat) &
          bind(C, name="sw_rtm_job_model")
       import :: c_int, c_ptr
       type(c_ptr), value    :: job
       integer(c_int), value :: first, count
       type(c_ptr)           :: dat(*)        ! c_loc of each shot's nrec*nt traces
     end function
     integer(c_int) function sw_rtm_job_admit(job, first, modeling, count) &
          bind(C, name="sw_rtm_job_admit")
       import :: c_int, c_ptr
       type(c_ptr), value    :: job
       integer(c_int), value :: first, modeling
       integer(c_int)        :: count
     end function
     integer(c_int) function sw_rtm_job_info(job, last_batch, points) &
          bind(C, name="sw_rtm_job_info")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int)     :: last_batch
       integer(c_int64_t) :: points
     end function
     integer(c_int) function sw_rtm_job_result(job, img, ill, img_norm) &
          bind(C, name="sw_rtm_job_result")
       import :: c_int, c_ptr
       type(c_ptr), value :: job, img, ill, img_norm   ! c_loc or c_null_ptr
     end function
     integer(c_int) function sw_rtm_job_reset(job) bind(C, name="sw_rtm_job_reset")
       import :: c_int, c_ptr
       type(c_ptr), value :: job
     end function
     integer(c_int) function sw_rtm_job_destroy(job) bind(C, name="sw_rtm_job_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: job
     end function
     ! ---- shot windows ---------------------------------------------------------
     integer(c_int) function sw_shot_window(model, apx, apy, sou, nrec, rec, w) &
          bind(C, name="sw_shot_window")
       import :: c_int, c_float, sw_genpar, sw_window
       type(sw_genpar)       :: model
       real(c_float), value  :: apx, apy
       real(c_float)         :: sou(3), rec(*)
       integer(c_int), value :: nrec
       type(sw_window)       :: w
     end function
     integer(c_int) function sw_window_extract(model, w, big, small) &
          bind(C, name="sw_window_extract")
       import :: c_int, c_float, sw_genpar, sw_window
       type(sw_genpar) :: model
       type(sw_window) :: w
       real(c_float)   :: big(*), small(*)
     end function
     integer(c_int) function sw_window_scatter_add(model, w, small, big) &
          bind(C, name="sw_window_scatter_add")
       import :: c_int, c_float, sw_genpar, sw_window
       type(sw_genpar) :: model
       type(sw_window) :: w
       real(c_float)   :: small(*), big(*)
     end function
     ! ---- FWI -------------------------------------------------------------------
     integer(c_int) function sw_fwi_fct_gdt(ctx, d, vel, wav, nshot, shots, vpmask, f, &
          grad, illum) bind(C, name="sw_fwi_fct_gdt")
       import :: c_int, c_ptr, c_float, c_double, sw_fwi_desc, sw_fwi_shot
       type(c_ptr), value    :: ctx
       type(sw_fwi_desc)     :: d
       real(c_float)         :: vel(*), wav(*)
       integer(c_int), value :: nshot
       type(sw_fwi_shot)     :: shots(*)
       type(c_ptr), value    :: vpmask         ! c_loc(invparam%vpmask) or c_null_ptr
       real(c_double)        :: f
       real(c_float)         :: grad(*)
       type(c_ptr), value    :: illum          ! c_loc or c_null_ptr
     end function
     integer(c_int) function sw_fwi_regularize(ctx, d, st, eval, vel, vpmask, f, grad) &
          bind(C, name="sw_fwi_regularize")
       import :: c_int, c_ptr, c_float, c_double, sw_reg_desc, sw_reg_state
       type(c_ptr), value    :: ctx
       type(sw_reg_desc)     :: d
       type(sw_reg_state)    :: st
       integer(c_int), value :: eval
       real(c_float)         :: vel(*)
       type(c_ptr), value    :: vpmask
       real(c_double)        :: f
       real(c_float)         :: grad(*)
     end function
     integer(c_int) function sw_lbfgs_create(ctx, n, m, xmin, xmax, mask, bound_type, &
          freeze_soft, xinit, s) bind(C, name="sw_lbfgs_create")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: n, m
       real(c_double), value :: xmin, xmax
       real(c_float)         :: mask(*)
       integer(c_int), value :: bound_type, freeze_soft
       real(c_double)        :: xinit(*)
       type(c_ptr)           :: s
     end function
     integer(c_int) function sw_lbfgs_destroy(s) bind(C, name="sw_lbfgs_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: s
     end function
     integer(c_int) function sw_lbfgs_step(s, x, f, g, eps, xtol, iflag, myinfo) &
          bind(C, name="sw_lbfgs_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value     :: s
       real(c_double)         :: x(*)
       real(c_double), value  :: f
       real(c_double)         :: g(*)
       real(c_double), value  :: eps, xtol
       integer(c_int)         :: iflag, myinfo
     end function
     integer(c_int) function sw_lbfgs_diag(s, out8) bind(C, name="sw_lbfgs_diag")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: s
       real(c_double)     :: out8(8)
     end function
     integer(c_int) function sw_lbfgs_oc_step(ctx, d, x, f, g, w, diag, st, iflag, myinfo) &
          bind(C, name="sw_lbfgs_oc_step")
       import :: c_int, c_ptr, c_double, sw_lbfgs_oc_desc, sw_lbfgs_oc_state
       type(c_ptr), value      :: ctx
       type(sw_lbfgs_oc_desc)  :: d
       real(c_double)          :: x(*)
       real(c_double), value   :: f
       real(c_double)          :: g(*), w(*), diag(*)
       type(sw_lbfgs_oc_state) :: st
       integer(c_int)          :: iflag, myinfo
     end function
     ! ---- tuning, preconditioner, instrumentation ------------------------------
     integer(c_int) function sw_ctx_set_tuning(ctx, t) bind(C, name="sw_ctx_set_tuning")
       import :: c_int, c_ptr, sw_tuning
       type(c_ptr), value :: ctx
       type(sw_tuning)    :: t
     end function
     integer(c_int) function sw_ctx_get_tuning(ctx, t) bind(C, name="sw_ctx_get_tuning")
       import :: c_int, c_ptr, sw_tuning
       type(c_ptr), value :: ctx
       type(sw_tuning)    :: t
     end function
     integer(c_int) function sw_cnn_create(ctx, nlayers, channels, seed, net) &
          bind(C, name="sw_cnn_create")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value        :: ctx
       integer(c_int), value     :: nlayers
       integer(c_int)            :: channels(*)
       integer(c_int64_t), value :: seed
       type(c_ptr)               :: net
     end function
     integer(c_int) function sw_cnn_destroy(net) bind(C, name="sw_cnn_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: net
     end function
     integer(c_int) function sw_cnn_num_weights(net) bind(C, name="sw_cnn_num_weights")
       import :: c_int, c_ptr
       type(c_ptr), value :: net
     end function
     integer(c_int) function sw_cnn_get_weights(net, w) bind(C, name="sw_cnn_get_weights")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float)      :: w(*)
     end function
     integer(c_int) function sw_cnn_set_weights(net, w) bind(C, name="sw_cnn_set_weights")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: net
       real(c_float)      :: w(*)
     end function
     integer(c_int) function sw_cnn_forward(net, nz, nx, in, out) &
          bind(C, name="sw_cnn_forward")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value    :: net
       integer(c_int), value :: nz, nx
       real(c_float)         :: in(*), out(*)
     end function
     integer(c_int) function sw_cnn_create3d(ctx, nlayers, channels, seed, net) &
          bind(C, name="sw_cnn_create3d")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value        :: ctx
       integer(c_int), value     :: nlayers
       integer(c_int)            :: channels(*)
       integer(c_int64_t), value :: seed
       type(c_ptr)               :: net
     end function
     integer(c_int) function sw_cnn_forward3d(net, nz, nx, ny, in, out) &
          bind(C, name="sw_cnn_forward3d")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value    :: net
       integer(c_int), value :: nz, nx, ny
       real(c_float)         :: in(*), out(*)
     end function
     integer(c_int) function sw_cnn_gradient3d(net, nbatch, nz, nx, ny, in, target, grad, &
          loss) bind(C, name="sw_cnn_gradient3d")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: net
       integer(c_int), value :: nbatch, nz, nx, ny
       real(c_float)         :: in(*), target(*), grad(*)
       real(c_double)        :: loss
     end function
     integer(c_int) function sw_cnn_train_step3d(net, nbatch, nz, nx, ny, in, target, lr, &
          loss) bind(C, name="sw_cnn_train_step3d")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: net
       integer(c_int), value :: nbatch, nz, nx, ny
       real(c_float)         :: in(*), target(*)
       real(c_float), value  :: lr
       real(c_double)        :: loss
     end function
     integer(c_int) function sw_cnn_gradient(net, nbatch, nz, nx, in, target, grad, loss) &
          bind(C, name="sw_cnn_gradient")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: net
       integer(c_int), value :: nbatch, nz, nx
       real(c_float)         :: in(*), target(*), grad(*)
       real(c_double)        :: loss
     end function
     integer(c_int) function sw_cnn_train_step(net, nbatch, nz, nx, in, target, lr, loss) &
          bind(C, name="sw_cnn_train_step")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: net
       integer(c_int), value :: nbatch, nz, nx
       real(c_float)         :: in(*), target(*)
       real(c_float), value  :: lr
       real(c_double)        :: loss
     end function
     integer(c_int) function sw_modeling_noalloc(g, vel, sou, wav, nrec, rec, dat) &
          bind(C, name="sw_modeling_noalloc")
       import :: c_int, c_float, sw_genpar
       type(sw_genpar)       :: g
       real(c_float)         :: vel(*), sou(3), wav(*)
       integer(c_int), value :: nrec
       real(c_float)         :: rec(*), dat(*)
     end function
     integer(c_int) function sw_ctx_get_stats(ctx, st) bind(C, name="sw_ctx_get_stats")
       import :: c_int, c_ptr, sw_stats
       type(c_ptr), value :: ctx
       type(sw_stats)     :: st
     end function
     integer(c_int) function sw_ctx_reset_stats(ctx) bind(C, name="sw_ctx_reset_stats")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function sw_ctx_set_boundary(ctx, mode) bind(C, name="sw_ctx_set_boundary")
       import :: c_int, c_ptr
       type(c_ptr), value    :: ctx
       integer(c_int), value :: mode
     end function
     integer(c_int) function sw_ctx_set_profiling(ctx, on) bind(C, name="sw_ctx_set_profiling")
       import :: c_int, c_ptr
       type(c_ptr), value    :: ctx
       integer(c_int), value :: on
     end function
  end interface
end module swave_iface
