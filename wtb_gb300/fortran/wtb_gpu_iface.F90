! ISO_C_BINDING layer between the WTB Fortran program and libwtb_gb300.so (include/wtb_gpu.h).
!
! module wtb_gpu holds
!   * the bind(C) derived types of the C ABI (wtb_bse_params_t, wtb_timings_t, wtb_temp_params_t), field for
!     field the C structs of include/wtb_gpu.h;
!   * bind(C) interfaces to the entry points (c_wtb_*);
!   * helpers: the process's device context (wtb_gpu_init), the status check that turns a library error into
!     the reference's behaviour (print the message, the reference's STOP text where it has one, and STOP),
!     the COULOMB_POT string -> potential code mapping, the run keys -> wtb_bse_params_t fill, file names as
!     NUL-terminated C strings;
!   * GPU versions of the reference's scalar routines with their argument lists unchanged, so the body of each
!     reference routine can become one call:
!       wtb_gpu_eigsys   <- eigsys   (src/module_hamiltonian.F90:200-320)
!       wtb_gpu_hlm      <- hlm      (src/module_optics.F90:12-108)
!       wtb_gpu_optsp    <- optsp    (src/module_optics.F90:113-167)
!       wtb_gpu_optdiel  <- optdiel  (src/module_optics.F90:171-255)
!       wtb_gpu_v2dk, wtb_gpu_vcoul, wtb_gpu_v3diel, wtb_gpu_v2dt, wtb_gpu_v0dt, wtb_gpu_v2dt2, wtb_gpu_v2drk,
!       wtb_gpu_v2dohono, wtb_gpu_v1dt <- the potentials of module_coulomb (src/module_coulomb.F90:11-442)
! The drop-in replacements of whole modules (module_bse, module_slepc_solver) are in module_bse.F90 and
! module_slepc_solver.F90 beside this file; they use this module.
!
! No Fortran compiler exists in the build image, so these files are not compiled by the project's build; the
! field layout of the bind(C) types is checked against the C header by tests/test_fortran_layer.py.
module wtb_gpu
  use iso_c_binding
  implicit none
  private
  public :: wtb_bse_params_t, wtb_timings_t, wtb_temp_params_t
  public :: wtb_gpu_init, wtb_gpu_ctx, wtb_gpu_check, wtb_coultype_code, wtb_gpu_params, wtb_cstr
  public :: wtb_gpu_set_hr, wtb_gpu_eigsys, wtb_gpu_slepc_solver, wtb_gpu_hlm, wtb_gpu_optsp, wtb_gpu_optdiel
  public :: wtb_gpu_v2dk, wtb_gpu_vcoul, wtb_gpu_v3diel, wtb_gpu_v2dt, wtb_gpu_v0dt, wtb_gpu_v2dt2, &
            wtb_gpu_v2drk, wtb_gpu_v2dohono, wtb_gpu_v1dt
  public :: c_wtb_bsesolver, c_wtb_bsedielraw, c_wtb_bsedielrawpol, c_wtb_spdielraw, c_wtb_spdielrawpol, &
            c_wtb_bsebnds, c_wtb_bsesolvertemp, c_wtb_bsebndstemp, c_wtb_zheev, c_wtb_zheev_vectors, &
            c_wtb_spoptics, c_wtb_spoptics_temp, c_wtb_spoptpolbz, c_wtb_spectrum_loss, c_wtb_bse_backward, &
            c_wtb_dielbse, c_wtb_bseoptprop, c_wtb_bseoptproppol, c_wtb_exciton_lifetime, c_wtb_bse_q_eigenpairs, &
            c_wtb_eigsys_mesh, c_wtb_write_bse_opt_diel, c_wtb_write_sp_optics, c_wtb_write_tm_coef, &
            c_wtb_write_exc_wf, c_wtb_write_exciton_lifetime, c_wtb_write_diel, c_wtb_write_bands_bse, &
            c_wtb_write_bz_act, c_wtb_coulomb_pair

  ! include/wtb_gpu.h: struct wtb_bse_params
  type, bind(C) :: wtb_bse_params_t
    integer(c_int)  :: ngrid(3)
    integer(c_int)  :: nc, nv
    real(c_double)  :: mshift(3)
    integer(c_int)  :: coultype, renorm
    real(c_double)  :: ktol, ediel(3), ez, w_coul, r0, lc, cshift, ebse0, ebsef
    integer(c_int)  :: numbse, nev, precision, op
    real(c_double)  :: tol
    integer(c_int)  :: maxit, block
  end type

  ! include/wtb_gpu.h: struct wtb_timings
  type, bind(C) :: wtb_timings_t
    real(c_double)  :: t_bands_ms, t_build_ms, t_solve_ms, t_optics_ms, t_total_ms
    integer(c_int)  :: iterations, matvec_columns
    real(c_double)  :: max_rel_residual, refine_shift_max
    integer(c_int)  :: kernel_launches
  end type

  ! include/wtb_gpu.h: wtb_temp_params
  type, bind(C) :: wtb_temp_params_t
    real(c_double)  :: temp
    integer(c_int)  :: ta
    real(c_double)  :: st, phavg
    integer(c_int)  :: dtfull, cpol
  end type

  interface
    integer(c_int) function c_wtb_ctx_create(ctx, device) bind(C, name="wtb_ctx_create")
      import :: c_ptr, c_int
      type(c_ptr), intent(out) :: ctx
      integer(c_int), value :: device
    end function
    type(c_ptr) function c_wtb_last_error(ctx) bind(C, name="wtb_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function c_wtb_set_hr(ctx, w, nvec, rvec, ffactor, hop, ihop, rlat, efermi, scs, np) &
        bind(C, name="wtb_set_hr")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: w, nvec, np
      integer(c_int) :: rvec(*), ffactor(*)
      real(c_double) :: hop(*), ihop(*), rlat(*)
      real(c_double), value :: efermi, scs
    end function
    integer(c_int) function c_wtb_eigsys(nthreads, scs, exc, nocp, ffactor, kx, ky, kz, w, nvec, rlat, rvec, &
        hop, ihop, efermi, energias, autovetores) bind(C, name="wtb_eigsys")
      import :: c_int, c_double, c_double_complex
      integer(c_int), value :: nthreads, w, nvec
      real(c_double), value :: scs, exc, kx, ky, kz, efermi
      integer(c_int) :: nocp, ffactor(*), rvec(*)
      real(c_double) :: rlat(*), hop(*), ihop(*), energias(*)
      complex(c_double_complex) :: autovetores(*)
    end function
    integer(c_int) function c_wtb_eigsys_mesh(ctx, nk, kpt, nv, nc, eigv, vector, nocpk) bind(C, name="wtb_eigsys_mesh")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nk, nv, nc
      real(c_double) :: kpt(*)
      type(c_ptr), value :: eigv, vector
      integer(c_int) :: nocpk(*)
    end function
    integer(c_int) function c_wtb_coulomb_pair(p, rlat, kpt1, kpt2, v) bind(C, name="wtb_coulomb_pair")
      import :: c_double, wtb_bse_params_t
      type(wtb_bse_params_t) :: p
      real(c_double) :: rlat(*), kpt1(*), kpt2(*), v
    end function
    integer(c_int) function c_wtb_hlm(kx, ky, kz, ffactor, w, nvec, rlat, rvec, hop, ihop, hx, hy, hz) &
        bind(C, name="wtb_hlm")
      import :: c_int, c_double, c_double_complex
      real(c_double), value :: kx, ky, kz
      integer(c_int), value :: w, nvec
      integer(c_int) :: ffactor(*), rvec(*)
      real(c_double) :: rlat(*), hop(*), ihop(*)
      complex(c_double_complex) :: hx(*), hy(*), hz(*)
    end function
    integer(c_int) function c_wtb_optsp_pair(ev, vv, ec, vc, kx, ky, kz, ffactor, sme, w, nvec, rlat, rvec, hop, &
        ihop, hrx, hry, hrz) bind(C, name="wtb_optsp_pair")
      import :: c_int, c_double, c_double_complex
      real(c_double), value :: ev, ec, kx, ky, kz, sme
      integer(c_int), value :: w, nvec
      complex(c_double_complex) :: vv(*), vc(*), hrx, hry, hrz
      integer(c_int) :: ffactor(*), rvec(*)
      real(c_double) :: rlat(*), hop(*), ihop(*)
    end function
    integer(c_int) function c_wtb_optdiel(rtype, vc, dimse, ngrid, elux, exciton, fosc, sme, rpart, ipart) &
        bind(C, name="wtb_optdiel")
      import :: c_int, c_double
      integer(c_int), value :: rtype, dimse
      real(c_double), value :: vc, elux, sme
      integer(c_int) :: ngrid(*)
      real(c_double) :: exciton(*), fosc(*), rpart, ipart
    end function
    integer(c_int) function c_wtb_slepc_solver(ctx, hx, ex, he, nx, ne) bind(C, name="wtb_slepc_solver")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex) :: hx(*), he(*)
      real(c_double) :: ex(*)
      integer(c_int), value :: nx, ne
    end function
    integer(c_int) function c_wtb_dielbse(ctx, dimse, dimse1, excitonvec, hopt1, hopt2, pair, activity) &
        bind(C, name="wtb_dielbse")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: dimse, dimse1, pair
      complex(c_double_complex) :: excitonvec(*), hopt1(*), hopt2(*)
      real(c_double) :: activity(*)
    end function
    integer(c_int) function c_wtb_bsesolver(ctx, p, ws, acts, he, t) bind(C, name="wtb_bsesolver")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t, wtb_timings_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      real(c_double) :: ws(*), acts(*)
      type(c_ptr), value :: he
      type(wtb_timings_t) :: t
    end function
    integer(c_int) function c_wtb_bsedielraw(ctx, p, dimse, ws, acts, dielf) bind(C, name="wtb_bsedielraw")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: dimse
      real(c_double) :: ws(*), acts(*), dielf(*)
    end function
    integer(c_int) function c_wtb_bsedielrawpol(ctx, p, dimse, ws, acts, dielf) bind(C, name="wtb_bsedielrawpol")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: dimse
      real(c_double) :: ws(*), acts(*), dielf(*)
    end function
    integer(c_int) function c_wtb_spdielraw(ctx, p, dimsp, esp, acts, dielf) bind(C, name="wtb_spdielraw")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: dimsp
      real(c_double) :: esp(*), acts(*), dielf(*)
    end function
    integer(c_int) function c_wtb_spdielrawpol(ctx, p, dimsp, esp, acts, dielf) bind(C, name="wtb_spdielrawpol")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: dimsp
      real(c_double) :: esp(*), acts(*), dielf(*)
    end function
    integer(c_int) function c_wtb_bseoptprop(ctx, numbse, dielf, props) bind(C, name="wtb_bseoptprop")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: numbse
      real(c_double) :: dielf(*), props(*)
    end function
    integer(c_int) function c_wtb_bseoptproppol(ctx, numbse, dielf, props) bind(C, name="wtb_bseoptproppol")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: numbse
      real(c_double) :: dielf(*), props(*)
    end function
    integer(c_int) function c_wtb_exciton_lifetime(ctx, sysdim, ngrid, dim, fosc, pol, lft) &
        bind(C, name="wtb_exciton_lifetime")
      import :: c_ptr, c_int, c_double, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char) :: sysdim(*)
      integer(c_int) :: ngrid(*)
      integer(c_int), value :: dim, pol
      real(c_double) :: fosc(*), lft(*)
    end function
    integer(c_int) function c_wtb_bsebnds(ctx, p, nq, qpath, exk) bind(C, name="wtb_bsebnds")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: nq
      real(c_double) :: qpath(*), exk(*)
    end function
    integer(c_int) function c_wtb_bse_q_eigenpairs(ctx, p, q4, il, nvec, w, z) bind(C, name="wtb_bse_q_eigenpairs")
      import :: c_ptr, c_int, c_double, c_double_complex, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      real(c_double) :: q4(*), w(*)
      integer(c_int), value :: il, nvec
      complex(c_double_complex) :: z(*)
    end function
    integer(c_int) function c_wtb_bsesolvertemp(ctx, p, tp, ws, acts, he, fdeh) bind(C, name="wtb_bsesolvertemp")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t, wtb_temp_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      type(wtb_temp_params_t) :: tp
      real(c_double) :: ws(*), acts(*)
      type(c_ptr), value :: he, fdeh
    end function
    integer(c_int) function c_wtb_bsebndstemp(ctx, p, tp, nq, qpath, exk) bind(C, name="wtb_bsebndstemp")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t, wtb_temp_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      type(wtb_temp_params_t) :: tp
      integer(c_int), value :: nq
      real(c_double) :: qpath(*), exk(*)
    end function
    integer(c_int) function c_wtb_zheev(ctx, n, a, lda, w) bind(C, name="wtb_zheev")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: n, lda
      complex(c_double_complex) :: a(*)
      real(c_double) :: w(*)
    end function
    integer(c_int) function c_wtb_zheev_vectors(ctx, n, a, lda, w, z) bind(C, name="wtb_zheev_vectors")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: n, lda
      complex(c_double_complex) :: a(*), z(*)
      real(c_double) :: w(*)
    end function
    integer(c_int) function c_wtb_spoptics(ctx, p, rec) bind(C, name="wtb_spoptics")
      import :: c_ptr, c_int, c_float, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      real(c_float) :: rec(*)
    end function
    integer(c_int) function c_wtb_spoptics_temp(ctx, p, tp, rec) bind(C, name="wtb_spoptics_temp")
      import :: c_ptr, c_int, c_float, wtb_bse_params_t, wtb_temp_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      type(wtb_temp_params_t) :: tp
      real(c_float) :: rec(*)
    end function
    integer(c_int) function c_wtb_spoptpolbz(ctx, p, act) bind(C, name="wtb_spoptpolbz")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      real(c_double) :: act(*)
    end function
    integer(c_int) function c_wtb_spectrum_loss(ctx, p, dimse, nev, e, fxx, target, l, dl_de, dl_df) &
        bind(C, name="wtb_spectrum_loss")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: dimse, nev
      real(c_double) :: e(*), fxx(*), target(*), l, dl_de(*), dl_df(*)
    end function
    integer(c_int) function c_wtb_bse_backward(ctx, p, dl_de, dl_df, dl_dhop, dl_dihop, dl_dr0, t) &
        bind(C, name="wtb_bse_backward")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t, wtb_timings_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      real(c_double) :: dl_de(*), dl_df(*), dl_dhop(*), dl_dihop(*), dl_dr0
      type(wtb_timings_t) :: t
    end function
    integer(c_int) function c_wtb_write_bse_opt_diel(path, dim, ws, acts, pol) bind(C, name="wtb_write_bse_opt_diel")
      import :: c_int, c_double, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: dim, pol
      real(c_double) :: ws(*), acts(*)
    end function
    integer(c_int) function c_wtb_write_sp_optics(path, dimsp, rec, pol) bind(C, name="wtb_write_sp_optics")
      import :: c_int, c_float, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: dimsp, pol
      real(c_float) :: rec(*)
    end function
    integer(c_int) function c_wtb_write_tm_coef(path, nk, nc, nv, rec, pol) bind(C, name="wtb_write_tm_coef")
      import :: c_int, c_float, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: nk, nc, nv, pol
      real(c_float) :: rec(*)
    end function
    integer(c_int) function c_wtb_write_exc_wf(path, nk, nc, nv, nocpk, kpt, q4, excnum, energy, ewf) &
        bind(C, name="wtb_write_exc_wf")
      import :: c_ptr, c_int, c_double, c_double_complex, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: nk, nc, nv, excnum
      integer(c_int) :: nocpk(*)
      real(c_double) :: kpt(*)
      type(c_ptr), value :: q4
      real(c_double), value :: energy
      complex(c_double_complex) :: ewf(*)
    end function
    integer(c_int) function c_wtb_write_exciton_lifetime(path, dim, energy, lft, pol) &
        bind(C, name="wtb_write_exciton_lifetime")
      import :: c_int, c_double, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: dim, pol
      real(c_double) :: energy(*), lft(*)
    end function
    integer(c_int) function c_wtb_write_diel(path, numbse, dielf) bind(C, name="wtb_write_diel")
      import :: c_int, c_double, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: numbse
      real(c_double) :: dielf(*)
    end function
    integer(c_int) function c_wtb_write_bands_bse(path, nq, dim, qpath, exk) bind(C, name="wtb_write_bands_bse")
      import :: c_int, c_double, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: nq, dim
      real(c_double) :: qpath(*), exk(*)
    end function
    integer(c_int) function c_wtb_write_bz_act(path, nk, kpt, value) bind(C, name="wtb_write_bz_act")
      import :: c_int, c_double, c_char
      character(kind=c_char) :: path(*)
      integer(c_int), value :: nk
      real(c_double) :: kpt(*), value(*)
    end function
  end interface

  type(c_ptr), save :: ctx = c_null_ptr

contains

  ! the process's device context (device 0, or WTB_DEVICE), created on first use
  subroutine wtb_gpu_init(device)
    integer, intent(in) :: device
    if (.not. c_associated(ctx)) call wtb_gpu_check(c_wtb_ctx_create(ctx, int(device, c_int)), 'wtb_ctx_create')
  end subroutine

  type(c_ptr) function wtb_gpu_ctx()
    character(len=16) :: env
    integer :: dev, st
    if (.not. c_associated(ctx)) then
      dev = 0
      call get_environment_variable('WTB_DEVICE', env, status=st)
      if (st == 0) read(env, *, iostat=st) dev
      call wtb_gpu_init(dev)
    end if
    wtb_gpu_ctx = ctx
  end function

  ! a non-zero status: print the library's message (the reference's STOP text where it has one) and STOP
  subroutine wtb_gpu_check(status, where)
    integer(c_int), intent(in) :: status
    character(*), intent(in) :: where
    character(kind=c_char, len=512), pointer :: msg
    integer :: n
    if (status /= 0) then
      if (c_associated(ctx)) then
        call c_f_pointer(c_wtb_last_error(ctx), msg)
        n = index(msg, c_null_char) - 1
        if (n < 0) n = len(msg)
        write(*,*) trim(where)//': '//msg(1:n)
      else
        write(*,*) trim(where)//': library status', status
      end if
      stop
    end if
  end subroutine

  ! COULOMB_POT keys of the reference's select case (src/module_bse.F90:49-72) -> WTB_V* codes
  integer(c_int) function wtb_coultype_code(coultype)
    character(len=*), intent(in) :: coultype
    select case (trim(adjustl(coultype)))
    case ("V2DK")
      wtb_coultype_code = 0
    case ("V3D")
      wtb_coultype_code = 1
    case ("V3DL")
      wtb_coultype_code = 2
    case ("V2DT")
      wtb_coultype_code = 3
    case ("V2DT2")
      wtb_coultype_code = 4
    case ("V2DOH")
      wtb_coultype_code = 5
    case ("V2DRK")
      wtb_coultype_code = 6
    case ("V1DT")
      wtb_coultype_code = 7
    case ("V0DT")
      wtb_coultype_code = 8
    case default
      write(*,*) "Wrong Coulomb Potential"
      stop
    end select
  end function

  ! the run keys of bsesolver and friends -> wtb_bse_params_t.  NEV, PRECISION and OPERATOR are not keys of the
  ! reference's input: they come from the environment (WTB_NEV, default 100 as the reference hard-codes at
  ! src/module_bse.F90:2432; WTB_PRECISION fp64 | fp32 | bf16x3 | bf16x6, default fp64; WTB_OPERATOR
  ! matfree | dense, default matfree; WTB_TOL, default 0 = the library's per-precision target).
  function wtb_gpu_params(ngrid, nc, nv, mshift, coultype, renorm, ktol, ediel, ez, w1, r0, lc, sme, ebse0, &
                          ebsef, numbse) result(p)
    integer, intent(in) :: ngrid(3), nc, nv
    double precision, intent(in) :: mshift(3), ktol, ediel(3), ez, w1, r0, lc, sme, ebse0, ebsef, numbse
    character(len=*), intent(in) :: coultype
    logical, intent(in) :: renorm
    type(wtb_bse_params_t) :: p
    character(len=16) :: env
    integer :: st, nev
    double precision :: tol
    p%ngrid = int(ngrid, c_int)
    p%nc = int(nc, c_int)
    p%nv = int(nv, c_int)
    p%mshift = mshift
    p%coultype = wtb_coultype_code(coultype)
    p%renorm = 0
    if (renorm) p%renorm = 1
    p%ktol = ktol
    p%ediel = ediel
    p%ez = ez
    p%w_coul = w1
    p%r0 = r0
    p%lc = lc
    p%cshift = sme
    p%ebse0 = ebse0
    p%ebsef = ebsef
    p%numbse = int(numbse, c_int)
    nev = 100
    call get_environment_variable('WTB_NEV', env, status=st)
    if (st == 0) read(env, *, iostat=st) nev
    nev = min(nev, ngrid(1)*ngrid(2)*ngrid(3)*nc*nv)
    p%nev = int(nev, c_int)
    p%precision = 0
    call get_environment_variable('WTB_PRECISION', env, status=st)
    if (st == 0) then
      select case (trim(env))
      case ("fp32")
        p%precision = 1
      case ("bf16x3")
        p%precision = 2
      case ("bf16x6")
        p%precision = 3
      end select
    end if
    p%op = 1
    call get_environment_variable('WTB_OPERATOR', env, status=st)
    if (st == 0 .and. trim(env) == "dense") p%op = 0
    tol = 0.d0
    call get_environment_variable('WTB_TOL', env, status=st)
    if (st == 0) read(env, *, iostat=st) tol
    p%tol = tol
    p%maxit = 0
    p%block = 0
  end function

  ! folder // name as a NUL-terminated C string
  function wtb_cstr(folder, name) result(s)
    character(len=*), intent(in) :: folder, name
    character(kind=c_char, len=len_trim(folder)+len(name)+1) :: s
    s = trim(folder)//name//c_null_char
  end function

  ! module_hamiltonian globals -> the context (after hamiltonian_input_read)
  subroutine wtb_gpu_set_hr(w90basis, nvec, rvec, ffactor, hopmatrices, ihopmatrices, rlat, efermi, scs, systype)
    integer :: w90basis, nvec, rvec(nvec,3), ffactor(nvec)
    double precision :: hopmatrices(nvec,w90basis,w90basis), ihopmatrices(nvec,w90basis,w90basis)
    double precision :: rlat(3,3), efermi, scs
    character(len=*) :: systype
    integer(c_int) :: np
    type(c_ptr) :: c
    c = wtb_gpu_ctx()
    np = 0
    if (trim(systype) == "NP") np = 1
    call wtb_gpu_check(c_wtb_set_hr(c, w90basis, nvec, rvec, ffactor, hopmatrices, ihopmatrices, rlat, efermi, scs, &
                       np), 'wtb_set_hr')
  end subroutine

  ! same argument list as eigsys (src/module_hamiltonian.F90:200-201)
  subroutine wtb_gpu_eigsys(nthreads, scs, exc, nocp, ffactor, kx, ky, kz, w90basis, nvec, rlat, rvec, &
                            hopmatrices, ihopmatrices, efermi, energias, autovetores)
    integer :: nthreads, nocp, w90basis, nvec
    integer :: ffactor(*), rvec(nvec,3)
    double precision :: scs, exc, kx, ky, kz, efermi, rlat(3,3)
    double precision :: hopmatrices(nvec,w90basis,w90basis), ihopmatrices(nvec,w90basis,w90basis)
    double precision :: energias(w90basis)
    double complex :: autovetores(w90basis,w90basis)
    integer(c_int) :: st, nocpc
    nocpc = nocp
    st = c_wtb_eigsys(nthreads, scs, exc, nocpc, ffactor, kx, ky, kz, w90basis, nvec, rlat, rvec, hopmatrices, &
                      ihopmatrices, efermi, energias, autovetores)
    if (st /= 0) then
      write(*,*) 'The algorithm failed to compute eigenvalues.'
      stop
    end if
    nocp = nocpc
  end subroutine

  ! same argument list as slepc_solver (src/module_slepc_solver.F90:12)
  subroutine wtb_gpu_slepc_solver(HX, EX, HE, NX, NE)
    integer :: NX, NE
    complex(8) :: HX(NX,NX), HE(NX,NE)
    real(8) :: EX(NE)
    call wtb_gpu_check(c_wtb_slepc_solver(wtb_gpu_ctx(), HX, EX, HE, NX, NE), 'slepc_solver')
  end subroutine

  ! same argument list as hlm (src/module_optics.F90:12)
  subroutine wtb_gpu_hlm(kx, ky, kz, ffactor, w90basis, nvec, rlat, rvec, hopmatrices, ihopmatrices, hx, hy, hz)
    integer :: w90basis, nvec
    integer :: ffactor(nvec), rvec(nvec,3)
    double precision :: kx, ky, kz, rlat(3,3)
    double precision :: hopmatrices(nvec,w90basis,w90basis), ihopmatrices(nvec,w90basis,w90basis)
    double complex :: hx(w90basis,w90basis), hy(w90basis,w90basis), hz(w90basis,w90basis)
    call wtb_gpu_check(c_wtb_hlm(kx, ky, kz, ffactor, w90basis, nvec, rlat, rvec, hopmatrices, ihopmatrices, hx, hy, &
                       hz), 'hlm')
  end subroutine

  ! same argument list as optsp (src/module_optics.F90:113)
  subroutine wtb_gpu_optsp(ev, vv, ec, vc, kx, ky, kz, ffactor, sme, w90basis, nvec, rlat, rvec, hopmatrices, &
                           ihopmatrices, hrx, hry, hrz)
    integer :: w90basis, nvec
    integer :: ffactor(nvec), rvec(nvec,3)
    double precision :: ev, ec, kx, ky, kz, sme, rlat(3,3)
    double complex :: vv(w90basis), vc(w90basis)
    double precision :: hopmatrices(nvec,w90basis,w90basis), ihopmatrices(nvec,w90basis,w90basis)
    double complex :: hrx, hry, hrz
    call wtb_gpu_check(c_wtb_optsp_pair(ev, vv, ec, vc, kx, ky, kz, ffactor, sme, w90basis, nvec, rlat, rvec, &
                       hopmatrices, ihopmatrices, hrx, hry, hrz), 'optsp')
  end subroutine

  ! same argument list as optdiel (src/module_optics.F90:171)
  subroutine wtb_gpu_optdiel(rtype, vc, dimse, ngrid, elux, exciton, fosc, sme, rpart, ipart)
    integer :: rtype, dimse
    integer, dimension(3) :: ngrid
    double precision :: vc, elux, sme, rpart, ipart
    double precision, dimension(dimse) :: exciton, fosc
    call wtb_gpu_check(c_wtb_optdiel(rtype, vc, dimse, ngrid, elux, exciton, fosc, sme, rpart, ipart), 'optdiel')
  end subroutine

  ! one value of potential code ct through wtb_coulomb_pair
  double precision function coulomb1(ct, kpt1, kpt2, rlat, ngrid, tolr, ediel, lc, ez, w, r0)
    integer(c_int), intent(in) :: ct
    double precision :: kpt1(3), kpt2(3), rlat(3,3), tolr, ediel(3), lc, ez, w, r0
    integer :: ngrid(3)
    type(wtb_bse_params_t) :: p
    real(c_double) :: v
    p%ngrid = int(ngrid, c_int)
    p%nc = 1
    p%nv = 1
    p%mshift = 0.d0
    p%coultype = ct
    p%renorm = 0
    p%ktol = tolr
    p%ediel = ediel
    p%ez = ez
    p%w_coul = w
    p%r0 = r0
    p%lc = lc
    p%cshift = 0.d0
    p%ebse0 = 0.d0
    p%ebsef = 0.d0
    p%numbse = 2
    p%nev = 1
    p%precision = 0
    p%op = 1
    p%tol = 0.d0
    p%maxit = 0
    p%block = 0
    call wtb_gpu_check(c_wtb_coulomb_pair(p, rlat, kpt1, kpt2, v), 'coulomb potential')
    coulomb1 = v
  end function

  ! the potentials of module_coulomb, same argument lists (src/module_coulomb.F90:11-442)
  real(8) function wtb_gpu_v2dk(kpt1, kpt2, ediel, rlat, ngrid, lc, tolr)
    double precision, dimension(3) :: kpt1, kpt2, ediel
    double precision :: rlat(3,3), lc, tolr
    integer, dimension(3) :: ngrid
    wtb_gpu_v2dk = coulomb1(0_c_int, kpt1, kpt2, rlat, ngrid, tolr, ediel, lc, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_vcoul(kpt1, kpt2, rlat, ngrid, tolr)
    double precision, dimension(3) :: kpt1, kpt2
    double precision :: rlat(3,3), tolr, ed(3)
    integer, dimension(3) :: ngrid
    ed = 1.d0
    wtb_gpu_vcoul = coulomb1(1_c_int, kpt1, kpt2, rlat, ngrid, tolr, ed, 0.d0, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_v3diel(kpt1, kpt2, ediel, rlat, ngrid, tolr)
    double precision, dimension(3) :: kpt1, kpt2, ediel
    double precision :: rlat(3,3), tolr
    integer, dimension(3) :: ngrid
    wtb_gpu_v3diel = coulomb1(2_c_int, kpt1, kpt2, rlat, ngrid, tolr, ediel, 0.d0, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_v2dt(kpt1, kpt2, ngrid, rlat, tolr)
    double precision, dimension(3) :: kpt1, kpt2
    double precision :: rlat(3,3), tolr, ed(3)
    integer, dimension(3) :: ngrid
    ed = 1.d0
    wtb_gpu_v2dt = coulomb1(3_c_int, kpt1, kpt2, rlat, ngrid, tolr, ed, 0.d0, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_v0dt(kpt1, kpt2, ngrid, rlat, tolr)
    double precision, dimension(3) :: kpt1, kpt2
    double precision :: rlat(3,3), tolr, ed(3)
    integer, dimension(3) :: ngrid
    ed = 1.d0
    wtb_gpu_v0dt = coulomb1(8_c_int, kpt1, kpt2, rlat, ngrid, tolr, ed, 0.d0, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_v2dt2(kpt1, kpt2, ngrid, rlat, lc, tolr)
    double precision, dimension(3) :: kpt1, kpt2
    double precision :: rlat(3,3), lc, tolr, ed(3)
    integer, dimension(3) :: ngrid
    ed = 1.d0
    wtb_gpu_v2dt2 = coulomb1(4_c_int, kpt1, kpt2, rlat, ngrid, tolr, ed, lc, 1.d0, 0.d0, 0.d0)
  end function

  real(8) function wtb_gpu_v2drk(kpt1, kpt2, ngrid, rlat, ediel, lc, ez, w, r0, tolr)
    double precision, dimension(3) :: kpt1, kpt2, ediel
    double precision :: rlat(3,3), lc, ez, w, r0, tolr
    integer, dimension(3) :: ngrid
    wtb_gpu_v2drk = coulomb1(6_c_int, kpt1, kpt2, rlat, ngrid, tolr, ediel, lc, ez, w, r0)
  end function

  real(8) function wtb_gpu_v2dohono(kpt1, kpt2, ngrid, rlat, ediel, w, ez, tolr)
    double precision, dimension(3) :: kpt1, kpt2, ediel
    double precision :: rlat(3,3), w, ez, tolr
    integer, dimension(3) :: ngrid
    wtb_gpu_v2dohono = coulomb1(5_c_int, kpt1, kpt2, rlat, ngrid, tolr, ediel, 0.d0, ez, w, 0.d0)
  end function

  real(8) function wtb_gpu_v1dt(kpt1, kpt2, ngrid, rlat, tolr, lc)
    double precision, dimension(3) :: kpt1, kpt2
    double precision :: rlat(3,3), tolr, lc, ed(3)
    integer, dimension(3) :: ngrid
    ed = 1.d0
    wtb_gpu_v1dt = coulomb1(7_c_int, kpt1, kpt2, rlat, ngrid, tolr, ed, lc, 1.d0, 0.d0, 0.d0)
  end function

end module wtb_gpu
