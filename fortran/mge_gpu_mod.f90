! mge_gpu_mod.f90 -- ISO_C_BINDING interface to libmge_gpu.so, the GB300
! multigrid Runge-Kutta cycle, for the unchanged code_mge Fortran driver.
!
! The derived types mirror include/mge_gpu.h field for field (bind(C)); the
! interfaces bind the C entry points; mge_stop turns a nonzero status into
! the stop the reference executes on the same condition.
module mge_gpu_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: MGE_OK = 0, MGE_ENAN = -1, MGE_ENEGPRESS = -2, MGE_EZERORHO = -3
  integer(c_int), parameter :: MGE_EBADCFG = -4, MGE_ENOMEM = -5, MGE_ETIMEOUT = -6, MGE_ECUDA = -7
  integer(c_int), parameter :: MGE_ENOTFOUND = -8
  integer(c_int), parameter :: MGE_EQN_EULER = 0, MGE_EQN_NS = 1
  integer(c_int), parameter :: MGE_DIS_CENTRAL = 0, MGE_DIS_ROE1 = 1, MGE_DIS_ROE2 = 2
  integer(c_int), parameter :: MGE_DISSIP_SCALAR = 0, MGE_DISSIP_MATRIX = 1
  integer(c_int), parameter :: MGE_PREC_FP64 = 0, MGE_PREC_MIXED = 1, MGE_PREC_REFINED = 2
  ! the layout of the types below; mge_abi_version() of the library must match
  integer(c_int), parameter :: MGE_ABI_VERSION = 2
  integer, parameter :: MGE_MAX_STAGE = 8, MGE_MAX_LEVEL = 16, MGE_MAX_CLOUD = 8

  type, bind(C) :: mge_params
    integer(c_int) :: mstage
    real(c_double) :: cstp(MGE_MAX_STAGE), cdis(MGE_MAX_STAGE)
    real(c_double) :: cfl
    integer(c_int) :: vt
    real(c_double) :: vis2, vis4, smoo
    integer(c_int) :: mgtype, eqntype, distype, dissip
    real(c_double) :: gamma, rm, alpha, beta
    real(c_double) :: rho0, p0, c0, ei0, u0, v0, w0, h0
    real(c_double) :: viscl, prlmean, gas_const, limfac, epsentr
    integer(c_int) :: wall_adiabatic, irs_variant, precision, nlevel
    integer(c_int) :: mcyc(MGE_MAX_LEVEL)
    real(c_double) :: conv_drop
    integer(c_int) :: execmode
    real(c_double) :: dtstep
  end type mge_params

  type, bind(C) :: mge_block_desc
    integer(c_int) :: nx, ny, nz
    real(c_double) :: h(3), origin(3), cellvolume
    real(c_double) :: si(3), sj(3), sk(3)
    integer(c_int) :: bctype(6)
    real(c_double) :: facenvec(3, 6)          ! C [6][3]: facenvec(:,face)
    type(c_ptr)    :: blank
    integer(c_int) :: nmir
    type(c_ptr)    :: ccid, scid, faceid, zz, npoint, ijkdex
    type(c_ptr)    :: coef, nvec, qb, area
    integer(c_int) :: parent
    integer(c_int) :: ratio(3), offset(3)
    type(c_ptr)    :: psurf                   ! [nmir][3] z(m)%psurf, or c_null_ptr
  end type mge_block_desc

  type, bind(C) :: mge_forces
    real(c_double) :: force(3), moment(3), cl, cd
  end type mge_forces

  type, bind(C) :: mge_solve_opts
    integer(c_int) :: max_cycles_total
    real(c_double) :: ref_area, moment_center(3)
    integer(c_int) :: use_graph
    real(c_double) :: refine_drop             ! mixed form: FP64 from this residual drop on (0: never)
  end type mge_solve_opts

  interface
    integer(c_int) function mge_abi_version() bind(C, name="mge_abi_version")
      import :: c_int
    end function
    integer(c_int) function mge_init(prm, device, ctx) bind(C, name="mge_init")
      import :: c_int, c_ptr, mge_params
      type(mge_params), intent(in) :: prm
      integer(c_int), value :: device
      type(c_ptr), intent(out) :: ctx
    end function
    subroutine mge_destroy(ctx) bind(C, name="mge_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    type(c_ptr) function mge_last_error(ctx) bind(C, name="mge_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mge_add_block(ctx, desc, level, serial) bind(C, name="mge_add_block")
      import :: c_int, c_ptr, mge_block_desc
      type(c_ptr), value :: ctx
      type(mge_block_desc), intent(in) :: desc
      integer(c_int), value :: level, serial
    end function
    integer(c_int) function mge_commit(ctx) bind(C, name="mge_commit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mge_init_flow(ctx) bind(C, name="mge_init_flow")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mge_upload_state(ctx, level, serial, w) bind(C, name="mge_upload_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
      real(c_double), intent(in) :: w(*)
    end function
    integer(c_int) function mge_download_state(ctx, level, serial, w, p) bind(C, name="mge_download_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
      real(c_double), intent(out) :: w(*), p(*)
    end function
    integer(c_int) function mge_timestep(ctx, level, serial) bind(C, name="mge_timestep")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
    end function
    integer(c_int) function mge_euler(ctx, level, serial, itime, ncyc, mgl, mlvl, lres, lfir) &
        bind(C, name="mge_euler")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial, itime, ncyc, mgl, mlvl, lres, lfir
    end function
    integer(c_int) function mge_movco(ctx, mgl) bind(C, name="mge_movco")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: mgl
    end function
    integer(c_int) function mge_movfin(ctx, mgl, mlvl) bind(C, name="mge_movfin")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: mgl, mlvl
    end function
    integer(c_int) function mge_bc_overlap(ctx, mgl) bind(C, name="mge_bc_overlap")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: mgl
    end function
    integer(c_int) function mge_get_rtrms(ctx, level, serial, ncyc, rt) bind(C, name="mge_get_rtrms")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial, ncyc
      real(c_double), intent(out) :: rt
    end function
    integer(c_int) function mge_cycle(ctx, mlvl, ncyc, max_res) bind(C, name="mge_cycle")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: mlvl, ncyc
      real(c_double), intent(out) :: max_res
    end function
    integer(c_int) function mge_solve(ctx, opts, hist, hist_len, cycles_done, forces) bind(C, name="mge_solve")
      import :: c_int, c_ptr, c_double, mge_solve_opts, mge_forces
      type(c_ptr), value :: ctx
      type(mge_solve_opts), intent(in) :: opts
      real(c_double), intent(out) :: hist(*)
      integer(c_int), value :: hist_len
      integer(c_int), intent(out) :: cycles_done
      type(mge_forces), intent(out) :: forces
    end function
    integer(c_int) function mge_set_precision(ctx, precision) bind(C, name="mge_set_precision")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: precision
    end function
    integer(c_int) function mge_forces_compute(ctx, level, opts, forces) bind(C, name="mge_forces_compute")
      import :: c_int, c_ptr, mge_solve_opts, mge_forces
      type(c_ptr), value :: ctx
      integer(c_int), value :: level
      type(mge_solve_opts), intent(in) :: opts
      type(mge_forces), intent(out) :: forces
    end function
    integer(c_int) function mge_upload_solut(ctx, level, serial, p_tot, solut, count, nval_out) &
        bind(C, name="mge_upload_solut")
      import :: c_int, c_ptr, c_double, c_size_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
      real(c_double), value :: p_tot
      real(c_double), intent(out) :: solut(*)        ! solut(2:il,2:jl,2:kl,1:nval)
      integer(c_size_t), value :: count
      integer(c_int), intent(out) :: nval_out
    end function
    integer(c_int) function mge_write_restart(ctx, path, codes, ncodes) bind(C, name="mge_write_restart")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)  ! NUL-terminated
      integer(c_int), intent(in) :: codes(*)
      integer(c_int), value :: ncodes
    end function
    integer(c_int) function mge_read_restart(ctx, path, codes, ncodes) bind(C, name="mge_read_restart")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), intent(in) :: codes(*)
      integer(c_int), value :: ncodes
    end function
    integer(c_int) function mge_time_advance(ctx, itime_out) bind(C, name="mge_time_advance")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: itime_out
    end function
    ! movsurf.f90:28-35 at solver.f90:117 (approxbc on), per block:
    ! pnew = psurf + disp, normal norv, qb = vel/vel_fs; arrays (3, nmir)
    integer(c_int) function mge_move_surface(ctx, level, serial, disp, norv, vel, vel_fs) &
        bind(C, name="mge_move_surface")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
      real(c_double), intent(in) :: disp(*), norv(*), vel(*)
      real(c_double), value :: vel_fs
    end function
    integer(c_int) function mge_get_surface(ctx, level, serial, pnew) bind(C, name="mge_get_surface")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: level, serial
      real(c_double), intent(out) :: pnew(*)
    end function
    integer(c_int) function mge_residual_norm_noalloc(dw_rho, vdtim, blank, nx, ny, nz, cfl, vt, dtim, &
        norm_out, stream) bind(C, name="mge_residual_norm_noalloc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dw_rho, vdtim, blank, norm_out, stream   ! device pointers
      integer(c_int), value :: nx, ny, nz, vt
      real(c_double), value :: cfl, dtim
    end function
  end interface

contains

  ! turn a nonzero status into the reference's stop
  subroutine mge_stop(rc, ctx, where)
    integer(c_int), intent(in) :: rc
    type(c_ptr), intent(in) :: ctx
    character(len=*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == MGE_OK) return
    call c_f_pointer(mge_last_error(ctx), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    print *, "mge_gpu error ", rc, " in ", where, ": ", msg(1:n)
    stop
  end subroutine mge_stop

end module mge_gpu_mod
