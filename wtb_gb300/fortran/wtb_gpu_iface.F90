! ISO_C_BINDING layer between the WTB Fortran modules and libwtb_gb300.so (include/wtb_gpu.h).
!
! Each wtb_gpu_* procedure keeps the argument list of the WTB subroutine it replaces, so the body of
! that subroutine can become a single call (see INTEGRATION.md):
!   wtb_gpu_eigsys        <- eigsys        (src/module_hamiltonian.F90:200-320)
!   wtb_gpu_slepc_solver  <- slepc_solver  (src/module_slepc_solver.F90:12-97)
!   wtb_gpu_bsesolver     <- bsesolver     (src/module_bse.F90:2023-2594)
!   wtb_gpu_bsedielraw    <- bsedielraw    (src/module_bse.F90:835-1036)
!   wtb_gpu_bsedielrawpol <- bsedielrawpol (src/module_bse.F90:1043-1199)
!   wtb_gpu_spoptics      <- spoptics      (src/module_bse.F90:4802-5071), records before the writes
!   wtb_gpu_spdielraw     <- spdielraw     (src/module_bse.F90:4090-4308)
!   wtb_gpu_spdielrawpol  <- spdielrawpol  (src/module_bse.F90:4318-4524)
!   wtb_gpu_bsebnds       <- the Q loop of bsebnds (src/module_bse.F90:1206-1566)
!   wtb_gpu_bsesolvertemp <- bsesolvertemp (src/module_bse.F90:2649-3263) before its writes
!   wtb_gpu_bsebndstemp   <- the Q loop of bsebndstemp (src/module_bse.F90:1572-1990)
!   wtb_gpu_zheev         <- ZHEEV('N'/'V', 'U', n, A, lda, W, ...) of the full-spectrum paths
! A non-zero status from the library is turned into the reference's behaviour: print the message
! (the reference's STOP text where it has one) and STOP.
! No Fortran compiler exists in the build image, so this file is not compiled by the project's build.
module wtb_gpu
  use iso_c_binding
  implicit none
  private
  public :: wtb_bse_params_t, wtb_timings_t, wtb_gpu_init, wtb_gpu_eigsys, wtb_gpu_slepc_solver, &
            wtb_gpu_bsesolver, wtb_gpu_bsedielraw, wtb_gpu_set_hr, wtb_gpu_bsedielrawpol, &
            wtb_gpu_spoptics, wtb_gpu_spdielraw, wtb_gpu_spdielrawpol, wtb_gpu_bsebnds, &
            wtb_temp_params_t, wtb_gpu_bsesolvertemp, wtb_gpu_bsebndstemp, wtb_gpu_zheev

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

  type, bind(C) :: wtb_timings_t
    real(c_double)  :: t_bands_ms, t_build_ms, t_solve_ms, t_optics_ms, t_total_ms
    integer(c_int)  :: iterations, matvec_columns
    real(c_double)  :: max_rel_residual, refine_shift_max
    integer(c_int)  :: kernel_launches
  end type

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
    integer(c_int) function c_wtb_slepc_solver(ctx, hx, ex, he, nx, ne) bind(C, name="wtb_slepc_solver")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex) :: hx(*), he(*)
      real(c_double) :: ex(*)
      integer(c_int), value :: nx, ne
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
    integer(c_int) function c_wtb_bsebnds(ctx, p, nq, qpath, exk) bind(C, name="wtb_bsebnds")
      import :: c_ptr, c_int, c_double, wtb_bse_params_t
      type(c_ptr), value :: ctx
      type(wtb_bse_params_t) :: p
      integer(c_int), value :: nq
      real(c_double) :: qpath(*), exk(*)
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
  end interface

  type(c_ptr), save :: ctx = c_null_ptr

contains

  subroutine check(status, where)
    integer(c_int), intent(in) :: status
    character(*), intent(in) :: where
    character(len=512), pointer :: msg
    if (status /= 0) then
      call c_f_pointer(c_wtb_last_error(ctx), msg)
      write(*,*) trim(where)//': '//msg(1:index(msg, c_null_char)-1)
      stop
    end if
  end subroutine

  subroutine wtb_gpu_init(device)
    integer, intent(in) :: device
    if (.not. c_associated(ctx)) call check(c_wtb_ctx_create(ctx, int(device, c_int)), 'wtb_ctx_create')
  end subroutine

  ! module_hamiltonian globals -> device (after hamiltonian_input_read)
  subroutine wtb_gpu_set_hr(w90basis, nvec, rvec, ffactor, hopmatrices, ihopmatrices, rlat, efermi, scs, systype)
    integer :: w90basis, nvec, rvec(nvec,3), ffactor(nvec)
    double precision :: hopmatrices(nvec,w90basis,w90basis), ihopmatrices(nvec,w90basis,w90basis)
    double precision :: rlat(3,3), efermi, scs
    character(len=*) :: systype
    integer(c_int) :: np
    call wtb_gpu_init(0)
    np = 0
    if (systype == "NP") np = 1
    call check(c_wtb_set_hr(ctx, w90basis, nvec, rvec, ffactor, hopmatrices, ihopmatrices, rlat, efermi, scs, np), &
               'wtb_set_hr')
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
    integer(c_int) :: st
    st = c_wtb_eigsys(nthreads, scs, exc, nocp, ffactor, kx, ky, kz, w90basis, nvec, rlat, rvec, hopmatrices, &
                      ihopmatrices, efermi, energias, autovetores)
    if (st /= 0) then
      write(*,*) 'The algorithm failed to compute eigenvalues.'
      stop
    end if
  end subroutine

  ! same argument list as slepc_solver (src/module_slepc_solver.F90:12)
  subroutine wtb_gpu_slepc_solver(HX, EX, HE, NX, NE)
    integer :: NX, NE
    complex(8) :: HX(NX,NX), HE(NX,NE)
    real(8) :: EX(NE)
    call wtb_gpu_init(0)
    call check(c_wtb_slepc_solver(ctx, HX, EX, HE, NX, NE), 'slepc_solver')
  end subroutine

  ! bsesolver body: bands, optics, BSE operator, lowest nev excitons, oscillator strengths, then the
  ! reference's bse_opt_diel.dat in 7F15.4 for every one of the dimbse rows (src/module_bse.F90:2556-2567)
  subroutine wtb_gpu_bsesolver(p, outputfolder, Ws, acts, dimbse)
    type(wtb_bse_params_t) :: p
    character(len=70) :: outputfolder
    integer :: dimbse, i, erro
    double precision :: Ws(dimbse), acts(dimbse,8)
    type(wtb_timings_t) :: t
    call wtb_gpu_init(0)
    call check(c_wtb_bsesolver(ctx, p, Ws, acts, c_null_ptr, t), 'bsesolver')
    open(unit=301, file=trim(outputfolder)//"/bse_opt_diel.dat", status='unknown', iostat=erro)
    if (erro /= 0) stop "Error opening bse_opt_diel output file"
    write(301,*) "#","  ", "exciton energy","  ","xx","  ","yy","  ","zz"," ","xy","  ","xz","  ","yz"
    do i = 1, dimbse
      write(301,"(7F15.4)") Ws(i), acts(i,1), acts(i,2), acts(i,3), acts(i,4), acts(i,5), acts(i,6)
    end do
    close(301)
  end subroutine

  subroutine wtb_gpu_bsedielraw(p, dimse, Ws, acts, dielf)
    type(wtb_bse_params_t) :: p
    integer :: dimse
    double precision :: Ws(dimse), acts(dimse,6), dielf(p%numbse,3,6)
    call wtb_gpu_init(0)
    call check(c_wtb_bsedielraw(ctx, p, dimse, Ws, acts, dielf), 'bsedielraw')
  end subroutine

  ! acts(:,1:5) = xx yy zz sp sm (the columns of bse_opt_diel-pol.dat)
  subroutine wtb_gpu_bsedielrawpol(p, dimse, Ws, acts, dielf)
    type(wtb_bse_params_t) :: p
    integer :: dimse
    double precision :: Ws(dimse), acts(dimse,5), dielf(p%numbse,3,5)
    call wtb_gpu_init(0)
    call check(c_wtb_bsedielrawpol(ctx, p, dimse, Ws, acts, dielf), 'bsedielrawpol')
  end subroutine

  ! vecres(dimsp,15) of spoptics, already sorted as Bubblem(7,15,vecres,dimsp) leaves it; the caller keeps
  ! its writes of sp_optics.dat (columns 7-13) and sp_optics-pol.dat (columns 7-10, 14-15)
  subroutine wtb_gpu_spoptics(p, dimsp, vecres)
    type(wtb_bse_params_t) :: p
    integer :: dimsp
    real :: vecres(dimsp,15)
    call wtb_gpu_init(0)
    call check(c_wtb_spoptics(ctx, p, vecres), 'spoptics')
  end subroutine

  ! qauxv(nq,4) of kpathbse; exk(dimbse,nq) all eigenvalues per Q, ascending (ZHEEV 'N')
  subroutine wtb_gpu_bsebnds(p, nq, qauxv, exk)
    type(wtb_bse_params_t) :: p
    integer :: nq
    double precision :: qauxv(nq,4), exk(*)
    call wtb_gpu_init(0)
    call check(c_wtb_bsebnds(ctx, p, nq, qauxv, exk), 'bsebnds')
  end subroutine

  ! W(dimbse) all exciton energies ascending, acts(dimbse,8) xx yy zz xy xz yz sp sm of dielbseptemp
  subroutine wtb_gpu_bsesolvertemp(p, tp, dimbse, W, acts)
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    integer :: dimbse
    double precision :: W(dimbse), acts(dimbse,8)
    call wtb_gpu_init(0)
    call check(c_wtb_bsesolvertemp(ctx, p, tp, W, acts, c_null_ptr, c_null_ptr), 'bsesolvertemp')
  end subroutine

  subroutine wtb_gpu_bsebndstemp(p, tp, nq, qauxv, exk)
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    integer :: nq
    double precision :: qauxv(nq,4), exk(*)
    call wtb_gpu_init(0)
    call check(c_wtb_bsebndstemp(ctx, p, tp, nq, qauxv, exk), 'bsebndstemp')
  end subroutine

  ! jobz 'N': W only (A is left unchanged); jobz 'V': the eigenvectors overwrite A, as ZHEEV's do
  subroutine wtb_gpu_zheev(jobz, n, A, lda, W)
    character :: jobz
    integer :: n, lda
    complex(8) :: A(lda,n)
    double precision :: W(n)
    complex(8), allocatable :: Z(:,:)
    call wtb_gpu_init(0)
    if (jobz == 'V' .or. jobz == 'v') then
      allocate(Z(n,n))
      call check(c_wtb_zheev_vectors(ctx, n, A, lda, W, Z), 'zheev')
      A(1:n,1:n) = Z
      deallocate(Z)
    else
      call check(c_wtb_zheev(ctx, n, A, lda, W), 'zheev')
    end if
  end subroutine

  subroutine wtb_gpu_spdielraw(p, dimsp, esp, acts, dielf)
    type(wtb_bse_params_t) :: p
    integer :: dimsp
    double precision :: esp(dimsp), acts(dimsp,6), dielf(p%numbse,3,6)
    call wtb_gpu_init(0)
    call check(c_wtb_spdielraw(ctx, p, dimsp, esp, acts, dielf), 'spdielraw')
  end subroutine

  subroutine wtb_gpu_spdielrawpol(p, dimsp, esp, acts, dielf)
    type(wtb_bse_params_t) :: p
    integer :: dimsp
    double precision :: esp(dimsp), acts(dimsp,5), dielf(p%numbse,3,5)
    call wtb_gpu_init(0)
    call check(c_wtb_spdielrawpol(ctx, p, dimsp, esp, acts, dielf), 'spdielrawpol')
  end subroutine

  ! gradient of L = sum_j (spinf eps2_xx(omega_j) - target_j)^2 with respect to H(R) and R_0, through the last
  ! wtb_gpu_bsesolver call (same p): dL_dhop/dL_dihop have the layout of hopmatrices/ihopmatrices
  subroutine wtb_gpu_spectrum_gradient(p, dimbse, Ws, acts, target, loss, dl_dhop, dl_dihop, dl_dr0, nvec, w90basis)
    type(wtb_bse_params_t) :: p
    integer :: dimbse, nvec, w90basis
    double precision :: Ws(dimbse), acts(dimbse,8), target(p%numbse), loss, dl_dr0
    double precision :: dl_dhop(nvec,w90basis,w90basis), dl_dihop(nvec,w90basis,w90basis)
    double precision :: dl_de(p%nev), dl_df(p%nev)
    type(wtb_timings_t) :: t
    call wtb_gpu_init(0)
    call check(c_wtb_spectrum_loss(ctx, p, dimbse, p%nev, Ws, acts(1:p%nev,1), target, loss, dl_de, dl_df), &
               'spectrum_loss')
    call check(c_wtb_bse_backward(ctx, p, dl_de, dl_df, dl_dhop, dl_dihop, dl_dr0, t), 'bse_backward')
  end subroutine

end module wtb_gpu
