! Drop-in replacement of WTB's module_bse (src/module_bse.F90) on the GB300 library: the same module name, the
! same module variables (dimbse, hbse, Ws, HE, ltest, ngkpt, kpt) and every public procedure with its argument
! list unchanged, so main.F90 compiles and runs against it without an edit.  The work of each procedure is one
! or two calls of the C ABI (module wtb_gpu, include/wtb_gpu.h); the files it writes are the reference's, in its
! record layouts, through the library's writers.
!
! Kept from the reference build: MPI_P (messages, the rank test), module_hamiltonian (hamiltonian_input_read and
! the H(R) globals, host Fortran by design), module_kmesh (monhkhorst_pack for the wavefunction files, kpathbse
! for the exciton-band path and its KLABELS-BSE.dat), module_coulomb and module_optics (their names stay visible
! through this module, as the reference's use list makes them).  module_slepc_solver is replaced beside this file.
!
! Run keys that the reference's input does not have come from the environment (see wtb_gpu_params): WTB_NEV
! (default 100, the reference's hard-coded count), WTB_PRECISION (fp64 | fp32 | bf16x3 | bf16x6, default fp64),
! WTB_OPERATOR (matfree | dense), WTB_TOL, WTB_DEVICE.  Only rank 0 drives the GPU and writes files, as only rank
! 0 writes them in the reference; the other ranks return after the call.
module module_bse
   use MPI_P
   use module_slepc_solver
   use module_hamiltonian
   use module_coulomb
   use module_kmesh
   use module_optics
   use wtb_gpu
   implicit none
   integer                            :: dimbse                        ! size of HBSE
   COMPLEX(8),allocatable,target      :: hbse(:,:)                     ! exciton eigenvectors of the last solve
   real(8),allocatable                :: Ws(:)                         ! exciton energies
   complex(8), allocatable            :: HE(:,:)
   logical                            :: ltest
   integer                            :: ngkpt                         ! number of k-points
   real(8),allocatable                :: kpt(:,:)                      ! k-points
  contains

  ! ---------------------------------------------------------------------------------------------- helpers
  ! H(R) of the params file -> the library context
  subroutine stage_hr(params)
    character(len=70) :: params
    call hamiltonian_input_read(200,params)
    call wtb_gpu_set_hr(w90basis, nvec, rvec, ffactor, hopmatrices, ihopmatrices, rlat, efermi, scs, systype)
  end subroutine stage_hr

  ! run keys of the spectrum routines (no potential involved)
  function spec_params(ngrid,nc,nv,renorm,sme,ebse0,ebsef,numbse) result(p)
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    logical :: renorm
    double precision :: sme,ebse0,ebsef,numbse
    type(wtb_bse_params_t) :: p
    double precision :: z3(3), one3(3)
    z3 = 0.d0
    one3 = 1.d0
    p = wtb_gpu_params(ngrid, nc, nv, z3, "V2DRK", renorm, 1.d-3, one3, 1.d0, 0.d0, 0.d0, 1.d0, sme, ebse0, ebsef, numbse)
  end function spec_params

  ! the temperature keys of bsesolvertemp/bsebndstemp (gap correction "FA" none, "VE", "BE")
  function temp_params(st,phavg,ta,temp,dtfull,cpol) result(tp)
    double precision :: st,phavg,temp
    character(len=2) :: ta
    logical :: dtfull,cpol
    type(wtb_temp_params_t) :: tp
    tp%temp = temp
    select case (ta)
    case ("VE")
      tp%ta = 1
    case ("BE")
      tp%ta = 2
    case default
      tp%ta = 0
    end select
    tp%st = st
    tp%phavg = phavg
    tp%dtfull = 0
    if (dtfull) tp%dtfull = 1
    tp%cpol = 0
    if (cpol) tp%cpol = 1
  end function temp_params

  ! rows of bse_opt_diel.dat (ncol = 7) or bse_opt_diel-pol.dat / sp_optics*.dat (ncol = 7 or 6)
  subroutine read_rows(path, nrow, ncol, a)
    character(len=*) :: path
    integer :: nrow, ncol, i, erro
    double precision :: a(nrow, ncol)
    character(len=2) :: aread
    OPEN(UNIT=100, FILE=path, STATUS='old', IOSTAT=erro)
    if (erro/=0) stop "Error opening input file"
    read(100,*) aread
    do i = 1, nrow
      read(100,*) a(i,1:ncol)
    end do
    close(100)
  end subroutine read_rows

  ! (omega, eps1, eps2) of one bse_diel_*.dat / sp_diel*.dat file
  subroutine read_diel(path, n, d)
    character(len=*) :: path
    integer :: n, i, erro
    double precision :: d(n,3)
    character(len=2) :: aread
    OPEN(UNIT=100, FILE=path, STATUS='old', IOSTAT=erro)
    if (erro/=0) stop "Error opening input file"
    read(100,*) aread
    do i = 1, n
      read(100,*) d(i,1), d(i,2), d(i,3)
    end do
    close(100)
  end subroutine read_diel

  ! the five optical-property files (7F15.4 or 6F15.4 rows under the reference's list-directed header) from
  ! props(n, ncomp, 5) = refractive index, extinction, reflectivity, absorption, energy loss
  subroutine write_props(outputfolder, prefix, suffix, n, ncomp, energy, props)
    character(len=70) :: outputfolder
    character(len=*) :: prefix, suffix
    integer :: n, ncomp, i, j, erro
    double precision :: energy(n), props(n, ncomp, 5)
    character(len=24), dimension(5) :: names
    names = [character(len=24) :: "refractive_index", "extinction_coef", "reflectibility", "absorption_coef", &
             "en_loss_func"]
    do j = 1, 5
      OPEN(UNIT=200, FILE=trim(outputfolder)//"/"//prefix//trim(names(j))//suffix//".dat", STATUS='unknown', &
           IOSTAT=erro)
      if (erro/=0) stop "Error opening output file"
      if (ncomp == 6) then
        write(200,*) "#","  ","energy","  ","xx","  ","yy","  ","zz","  ","xy","  ","xz","  ","yz"
        do i = 1, n
          write(200,"(7F15.4)") energy(i), props(i,1,j), props(i,2,j), props(i,3,j), props(i,4,j), props(i,5,j), &
                                props(i,6,j)
        end do
      else
        write(200,*) "#","  ","energy","  ","x","  ","y","  ","z","  ","sp","  ","sm"
        do i = 1, n
          write(200,"(6F15.4)") energy(i), props(i,1,j), props(i,2,j), props(i,3,j), props(i,4,j), props(i,5,j)
        end do
      end if
      close(200)
    end do
  end subroutine write_props

  ! the IPA records and their files (sp_optics.dat, sp_optics-pol.dat, optionally tm_coef.dat, tm_coef-pol.dat)
  subroutine write_ipa(outputfolder, ngrid, nc, nv, dimsp, vecres, tmcoef)
    character(len=70) :: outputfolder
    integer,dimension(3) :: ngrid
    integer :: nc, nv, dimsp
    real(c_float) :: vecres(dimsp,15)
    logical :: tmcoef
    integer(c_int) :: nk
    nk = ngrid(1)*ngrid(2)*ngrid(3)
    call wtb_gpu_check(c_wtb_write_sp_optics(wtb_cstr(outputfolder,"/sp_optics.dat"), dimsp, vecres, 0), 'sp_optics.dat')
    call wtb_gpu_check(c_wtb_write_sp_optics(wtb_cstr(outputfolder,"/sp_optics-pol.dat"), dimsp, vecres, 1), &
                       'sp_optics-pol.dat')
    if (tmcoef) then
      call wtb_gpu_check(c_wtb_write_tm_coef(wtb_cstr(outputfolder,"/tm_coef.dat"), nk, nc, nv, vecres, 0), 'tm_coef.dat')
      call wtb_gpu_check(c_wtb_write_tm_coef(wtb_cstr(outputfolder,"/tm_coef-pol.dat"), nk, nc, nv, vecres, 1), &
                         'tm_coef-pol.dat')
    end if
  end subroutine write_ipa

  ! exc_wf_<n>.dat (excwf2) for the excitons excwf0..excwff of the eigenvector block vecs(dim, ncol), whose column
  ! j holds exciton col0 + j - 1
  subroutine write_wf(outputfolder, ngrid, mshift, nc, nv, col0, ncol, E, vecs, excwf0, excwff)
    character(len=70) :: outputfolder
    integer,dimension(3) :: ngrid
    double precision,dimension(3) :: mshift
    integer :: nc, nv, col0, ncol, excwf0, excwff, i, nk
    double precision :: E(*)
    complex(8) :: vecs(:,:)
    double precision, allocatable :: kk(:,:)
    integer(c_int), allocatable :: nocpk(:)
    character(len=200) :: file1
    nk = ngrid(1)*ngrid(2)*ngrid(3)
    allocate(kk(nk,3), nocpk(nk))
    call monhkhorst_pack(ngrid(1),ngrid(2),ngrid(3),mshift,rlat(1,:),rlat(2,:),rlat(3,:),kk)
    call wtb_gpu_check(c_wtb_eigsys_mesh(wtb_gpu_ctx(), nk, kk, nv, nc, c_null_ptr, c_null_ptr, nocpk), 'eigsys')
    do i = max(excwf0, col0), min(excwff, col0 + ncol - 1)
      write(file1,'(a7,I0,a4)') 'exc_wf_', i, '.dat'
      call wtb_gpu_check(c_wtb_write_exc_wf(trim(outputfolder)//trim(file1)//c_null_char, nk, nc, nv, nocpk, kk, &
                         c_null_ptr, i, E(i - col0 + 1), vecs(:, i - col0 + 1)), 'excwf2')
    end do
    deallocate(kk, nocpk)
  end subroutine write_wf

  ! the Q path of bsebnds/bsebndstemp from the kpathsbse file (nks, npts, nks corner points), by the reference's
  ! kpathbse (which also writes KLABELS-BSE.dat)
  subroutine read_qpath(outputfolder, kpathsbse, nq, qauxv)
    character(len=70) :: outputfolder, kpathsbse
    integer :: nq, nks, nkpts, i, erro
    double precision, allocatable :: qauxv(:,:), ks(:,:)
    OPEN(UNIT=500, FILE=kpathsbse, STATUS='old', IOSTAT=erro)
    if (erro/=0) stop "Error opening kpath input file"
    read(500,*) nks
    read(500,*) nkpts
    allocate(ks(nks,3))
    do i = 1, nks
      read(500,*) ks(i,1), ks(i,2), ks(i,3)
    end do
    close(500)
    nq = (nks/2)*nkpts
    allocate(qauxv(nq,4))
    call kpathbse(outputfolder,rlat(1,:),rlat(2,:),rlat(3,:),nks,ks,nkpts,qauxv)
    deallocate(ks)
  end subroutine read_qpath

  ! ---------------------------------------------------------------------------------------------- the path
  ! matrizelbse (src/module_bse.F90:24-83): one element of the BSE matrix, the potential evaluated on the GPU
  ! (wtb_coulomb_pair) and the two length-w overlaps v_i^* . v_j, c_i^* . c_j as the reference forms them.  The
  ! build loop that calls it is replaced whole by the library (wtb_bsesolver / wtb_bse_build); this function is
  ! kept for callers that evaluate single elements.
  complex(8) function matrizelbse(coultype,tolr,w90basis,ediel,lc,ez,w,r0,ngrid,rlat,est1,ec1,ev1,vbc1 &
                                  ,vbv1,kpt1,est2,ec2,ev2,vbc2,vbv2,kpt2)
    character(len=5) :: coultype
    integer,dimension(3) :: ngrid
    integer :: w90basis
    double precision :: ez,w
    integer, dimension(4) :: est1,est2
    double precision :: ec1,ec2,ev1,ev2
    double precision,dimension(3) :: kpt1,kpt2
    double complex, dimension(w90basis) :: vbc1,vbc2,vbv1,vbv2
    double precision,dimension(3,3) :: rlat
    double precision :: tolr
    double precision,dimension(3) :: ediel
    double precision :: lc
    double precision :: r0
    double precision :: vcoul1
    double complex :: vc,vv
    select case (coultype)
    case("V2DK")
      vcoul1 = wtb_gpu_v2dk(kpt1,kpt2,ediel,rlat,ngrid,lc,tolr)
    case("V3D")
      vcoul1 = wtb_gpu_vcoul(kpt1,kpt2,rlat,ngrid,tolr)
    case("V3DL")
      vcoul1 = wtb_gpu_v3diel(kpt1,kpt2,ediel,rlat,ngrid,tolr)
    case("V2DT")
      vcoul1 = wtb_gpu_v2dt(kpt1,kpt2,ngrid,rlat,tolr)
    case("V2DT2")
      vcoul1 = wtb_gpu_v2dt2(kpt1,kpt2,ngrid,rlat,lc,tolr)
    case("V2DOH")
      vcoul1 = wtb_gpu_v2dohono(kpt1,kpt2,ngrid,rlat,ediel,w,ez,tolr)
    case("V2DRK")
      vcoul1 = wtb_gpu_v2drk(kpt1,kpt2,ngrid,rlat,ediel,lc,ez,w,r0,tolr)
    case("V1DT")
      vcoul1 = wtb_gpu_v1dt(kpt1,kpt2,ngrid,rlat,tolr,lc)
    case("V0DT")
      vcoul1 = wtb_gpu_v0dt(kpt1,kpt2,ngrid,rlat,tolr)
    case default
      if(Process==0) write(*,*) "Wrong Coulomb Potential"
      STOP
    end select
    if (est1(1) .eq. est2(1)) then
      matrizelbse = (ec1-ev1) + vcoul1
    else
      vc = sum(conjg(vbc1) * vbc2)
      vv = sum(conjg(vbv1) * vbv2)
      matrizelbse = vcoul1*vc*vv
    end if
  end function matrizelbse

  ! dielbsep (src/module_bse.F90:171-196): activity(i) = Re[(sum_j A(j,i) h1(j)) (sum_j A(j,i) h2(j))^*], i <= dimse1
  subroutine dielbsep(nthread,dimse,dimse1,excitonvec,hopt1,hopt2,activity)
    integer                       :: dimse,dimse1,nthread
    double precision,dimension(:) :: activity
    double complex,dimension(:)   :: hopt1,hopt2
    double complex,dimension(:,:) :: excitonvec
    double complex, allocatable   :: a(:,:), h1(:), h2(:)
    double precision, allocatable :: act(:)
    allocate(a(dimse,dimse1), h1(dimse), h2(dimse), act(dimse))
    a = excitonvec(1:dimse,1:dimse1)
    h1 = hopt1(1:dimse)
    h2 = hopt2(1:dimse)
    call wtb_gpu_check(c_wtb_dielbse(wtb_gpu_ctx(), dimse, dimse1, a, h1, h2, 1, act), 'dielbsep')
    activity(1:dimse) = act
    deallocate(a, h1, h2, act)
  end subroutine dielbsep

  ! dielbsev (src/module_bse.F90:201-245): activity(i) = |sum_j A(j,i) h(j)|^2, i <= dimse1
  subroutine dielbsev(nthread,dimse,dimse1,excitonvec,hopt,activity)
    integer                   :: dimse,dimse1,nthread
    real(8),dimension(:)      :: activity
    complex(8),dimension(:)   :: hopt
    complex(8),dimension(:,:) :: excitonvec
    double complex, allocatable   :: a(:,:), h1(:)
    double precision, allocatable :: act(:)
    allocate(a(dimse,dimse1), h1(dimse), act(dimse))
    a = excitonvec(1:dimse,1:dimse1)
    h1 = hopt(1:dimse)
    call wtb_gpu_check(c_wtb_dielbse(wtb_gpu_ctx(), dimse, dimse1, a, h1, h1, 0, act), 'dielbsev')
    activity(1:dimse) = act
    deallocate(a, h1, act)
  end subroutine dielbsev

  ! bsesolver (src/module_bse.F90:2023-2594): bands, velocity elements, BSE operator, lowest excitons and their
  ! activities on the GPU (wtb_bsesolver); then the reference's files: log_bse-diel.dat, bse_opt_diel.dat
  ! (7F15.4, every one of the dimbse rows, rows past the solved excitons zero), bse_opt_diel-pol.dat, sp_optics.dat,
  ! sp_optics-pol.dat, tm_coef*.dat (tmcoef) and exc_wf_<n>.dat (bsewf, excitons excwf0..excwff).
  subroutine bsesolver(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,ez,w1,r0,lc,rk,meshtype,bsewf,excwf0,excwff,&
             dtfull,cpol,tmcoef)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params
    character(len=70) :: orbw
    character(len=70) :: kpaths
    character(len=70) :: kpathsbse
    character(len=70) :: outputfolder
    character(len=70) :: calcparms
    character(len=70) :: meshtype
    character(len=5) :: coultype
    double precision,dimension(3) :: ediel
    logical :: bsewf
    integer :: excwf0,excwff
    double precision :: ez,w1,lc,r0
    logical :: cpol,dtfull
    logical :: tmcoef
    type(wtb_bse_params_t) :: p
    type(wtb_timings_t) :: t
    double precision, allocatable :: acts(:,:)
    real(c_float), allocatable :: vecres(:,:)
    type(c_ptr) :: c, hep
    integer :: erro, nev
    integer,dimension(8) :: values

    if (Process /= 0) return
    call MSG('MODULE_BSE: hamiltonian_input_read')
    call stage_hr(params)
    c = wtb_gpu_ctx()
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    ngkpt = ngrid(1)*ngrid(2)*ngrid(3)
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, ez, w1, r0, lc, sme, ebse0, ebsef, &
                       numbse)
    nev = p%nev
    if (allocated(Ws)) deallocate(Ws)
    if (allocated(hbse)) deallocate(hbse)
    allocate(Ws(dimbse), acts(dimbse,8))
    hep = c_null_ptr
    if (bsewf) then
      allocate(hbse(dimbse,nev))
      hep = c_loc(hbse)
    end if
    OPEN(UNIT=300, FILE=trim(outputfolder)//"/log_bse-diel.dat",STATUS='unknown', IOSTAT=erro)
    if (erro/=0) stop "Error opening log_bse-diel output file"
    call date_and_time(VALUES=values)
    write(300,*) 'threads:', nthreads
    write(300,*) 'grid:', ngrid(1), ngrid(2), ngrid(3)
    write(300,*) 'ktol-coulomb:', ktol
    write(300,*) 'kmesh shift:', mshift(1), mshift(2), mshift(3)
    write(300,*) 'conduction bands, nc:', nc, '  ', 'valence bands, nv:', nv
    write(300,*) 'begin', '  ', 'day', values(3), '', values(5), 'hours', values(6), 'min', values(7), 'seg'
    call MSG('MODULE_BSE: BSE on the GPU')
    call wtb_gpu_check(c_wtb_bsesolver(c, p, Ws, acts, hep, t), 'bsesolver')
    write(300,*) 'excitons solved:', nev, ' iterations:', t%iterations, ' max relative residual:', t%max_rel_residual
    write(300,*) 'GPU time (ms): bands', t%t_bands_ms, ' build', t%t_build_ms, ' solve', t%t_solve_ms, &
                 ' optics', t%t_optics_ms
    call date_and_time(VALUES=values)
    write(300,*) 'end', '  ', 'day', values(3), '', values(5), 'hours', values(6), 'min', values(7), 'seg'
    close(300)
    call wtb_gpu_check(c_wtb_write_bse_opt_diel(wtb_cstr(outputfolder,"/bse_opt_diel.dat"), dimbse, Ws, acts, 0), &
                       'bse_opt_diel.dat')
    call wtb_gpu_check(c_wtb_write_bse_opt_diel(wtb_cstr(outputfolder,"/bse_opt_diel-pol.dat"), dimbse, Ws, acts, 1), &
                       'bse_opt_diel-pol.dat')
    allocate(vecres(dimbse,15))
    call wtb_gpu_check(c_wtb_spoptics(c, p, vecres), 'spoptics')
    call write_ipa(outputfolder, ngrid, nc, nv, dimbse, vecres, tmcoef)
    deallocate(vecres)
    if (bsewf) call write_wf(outputfolder, ngrid, mshift, nc, nv, 1, nev, Ws, hbse, excwf0, excwff)
    deallocate(acts)
  end subroutine bsesolver

  ! bsedielraw (src/module_bse.F90:835-1036): bse_opt_diel.dat -> bse_diel_xx/xy/xz/yy/yz/zz.dat
  subroutine bsedielraw(nthreads,outputfolder,renorm,params,ngrid,nc,nv,ebse0,ebsef,numbse,sme)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: ebse0,ebsef,numbse
    double precision :: sme
    character(len=70) :: params
    character(len=70) :: outputfolder
    logical :: renorm
    double precision, allocatable :: rows(:,:), dielf(:,:,:)
    type(wtb_bse_params_t) :: p
    integer :: n, j
    character(len=2), dimension(6) :: comp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start bsedielraw')
    call stage_hr(params)
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    n = int(numbse)
    allocate(rows(dimbse,7), dielf(n,3,6))
    call read_rows(trim(outputfolder)//"/bse_opt_diel.dat", dimbse, 7, rows)
    p = spec_params(ngrid,nc,nv,renorm,sme,ebse0,ebsef,numbse)
    call wtb_gpu_check(c_wtb_bsedielraw(wtb_gpu_ctx(), p, dimbse, rows(:,1), rows(:,2:7), dielf), 'bsedielraw')
    comp = [character(len=2) :: "xx", "yy", "zz", "xy", "xz", "yz"]
    do j = 1, 6
      call wtb_gpu_check(c_wtb_write_diel(wtb_cstr(outputfolder,"/bse_diel_"//comp(j)//".dat"), n, dielf(:,:,j)), &
                         'bse_diel_'//comp(j))
    end do
    deallocate(rows, dielf)
  end subroutine bsedielraw

  ! bsedielrawpol (src/module_bse.F90:1043-1199): bse_opt_diel-pol.dat -> bse_diel-pol_x/y/z/sp/sm.dat
  subroutine bsedielrawpol(nthreads,outputfolder,renorm,params,ngrid,nc,nv,ebse0,ebsef,numbse,sme)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: ebse0,ebsef,numbse
    double precision :: sme
    character(len=70) :: params
    character(len=70) :: outputfolder
    logical :: renorm
    double precision, allocatable :: rows(:,:), dielf(:,:,:)
    type(wtb_bse_params_t) :: p
    integer :: n, j
    character(len=2), dimension(5) :: comp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start bsedielrawpol')
    call stage_hr(params)
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    n = int(numbse)
    allocate(rows(dimbse,6), dielf(n,3,5))
    call read_rows(trim(outputfolder)//"/bse_opt_diel-pol.dat", dimbse, 6, rows)
    p = spec_params(ngrid,nc,nv,renorm,sme,ebse0,ebsef,numbse)
    call wtb_gpu_check(c_wtb_bsedielrawpol(wtb_gpu_ctx(), p, dimbse, rows(:,1), rows(:,2:6), dielf), 'bsedielrawpol')
    comp = [character(len=2) :: "x", "y", "z", "sp", "sm"]
    do j = 1, 5
      call wtb_gpu_check(c_wtb_write_diel(wtb_cstr(outputfolder,"/bse_diel-pol_"//trim(comp(j))//".dat"), n, &
                         dielf(:,:,j)), 'bse_diel-pol_'//trim(comp(j)))
    end do
    deallocate(rows, dielf)
  end subroutine bsedielrawpol

  ! spdielraw (src/module_bse.F90:4090-4308): sp_optics.dat -> sp_diel_*.dat
  subroutine spdielraw(nthreads,outputfolder,renorm,params,ngrid,nc,nv,ebse0,ebsef,numbse,sme)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: ebse0,ebsef,numbse
    double precision :: sme
    character(len=70) :: params
    character(len=70) :: outputfolder
    logical :: renorm
    double precision, allocatable :: rows(:,:), dielf(:,:,:)
    type(wtb_bse_params_t) :: p
    integer :: n, j, dimsp
    character(len=2), dimension(6) :: comp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start spdielraw')
    call stage_hr(params)
    dimsp = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    n = int(numbse)
    allocate(rows(dimsp,7), dielf(n,3,6))
    call read_rows(trim(outputfolder)//"/sp_optics.dat", dimsp, 7, rows)
    p = spec_params(ngrid,nc,nv,renorm,sme,ebse0,ebsef,numbse)
    call wtb_gpu_check(c_wtb_spdielraw(wtb_gpu_ctx(), p, dimsp, rows(:,1), rows(:,2:7), dielf), 'spdielraw')
    comp = [character(len=2) :: "xx", "yy", "zz", "xy", "xz", "yz"]
    do j = 1, 6
      call wtb_gpu_check(c_wtb_write_diel(wtb_cstr(outputfolder,"/sp_diel_"//comp(j)//".dat"), n, dielf(:,:,j)), &
                         'sp_diel_'//comp(j))
    end do
    deallocate(rows, dielf)
  end subroutine spdielraw

  ! spdielrawpol (src/module_bse.F90:4318-4524): sp_optics-pol.dat -> sp_diel-pol_*.dat
  subroutine spdielrawpol(nthreads,outputfolder,renorm,params,ngrid,nc,nv,ebse0,ebsef,numbse,sme)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: ebse0,ebsef,numbse
    double precision :: sme
    character(len=70) :: params
    character(len=70) :: outputfolder
    logical :: renorm
    double precision, allocatable :: rows(:,:), dielf(:,:,:)
    type(wtb_bse_params_t) :: p
    integer :: n, j, dimsp
    character(len=2), dimension(5) :: comp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start spdielrawpol')
    call stage_hr(params)
    dimsp = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    n = int(numbse)
    allocate(rows(dimsp,6), dielf(n,3,5))
    call read_rows(trim(outputfolder)//"/sp_optics-pol.dat", dimsp, 6, rows)
    p = spec_params(ngrid,nc,nv,renorm,sme,ebse0,ebsef,numbse)
    call wtb_gpu_check(c_wtb_spdielrawpol(wtb_gpu_ctx(), p, dimsp, rows(:,1), rows(:,2:6), dielf), 'spdielrawpol')
    comp = [character(len=2) :: "x", "y", "z", "sp", "sm"]
    do j = 1, 5
      call wtb_gpu_check(c_wtb_write_diel(wtb_cstr(outputfolder,"/sp_diel-pol_"//trim(comp(j))//".dat"), n, &
                         dielf(:,:,j)), 'sp_diel-pol_'//trim(comp(j)))
    end do
    deallocate(rows, dielf)
  end subroutine spdielrawpol

  ! bseoptprop (src/module_bse.F90:3766-3931) and friends: the spectra files -> the five property files
  subroutine optprop_files(outputfolder, n, inprefix, comps, ncomp, outprefix, outsuffix)
    character(len=70) :: outputfolder
    integer :: n, ncomp, j
    character(len=*) :: inprefix, outprefix, outsuffix
    character(len=2), dimension(ncomp) :: comps
    double precision, allocatable :: dielf(:,:,:), props(:,:,:)
    if (Process /= 0) return
    allocate(dielf(n,3,ncomp), props(n,ncomp,5))
    do j = 1, ncomp
      call read_diel(trim(outputfolder)//"/"//inprefix//trim(comps(j))//".dat", n, dielf(:,:,j))
    end do
    if (ncomp == 6) then
      call wtb_gpu_check(c_wtb_bseoptprop(wtb_gpu_ctx(), n, dielf, props), 'optprop')
    else
      call wtb_gpu_check(c_wtb_bseoptproppol(wtb_gpu_ctx(), n, dielf, props), 'optproppol')
    end if
    call write_props(outputfolder, outprefix, outsuffix, n, ncomp, dielf(:,1,1), props)
    deallocate(dielf, props)
  end subroutine optprop_files

  subroutine bseoptprop(numbse,outputfolder)
    character(len=70) :: outputfolder
    double precision ::  numbse
    call optprop_files(outputfolder, int(numbse), "bse_diel_", &
                       [character(len=2) :: "xx", "yy", "zz", "xy", "xz", "yz"], 6, "bse_", "")
  end subroutine bseoptprop

  subroutine bseoptproppol(numbse,outputfolder)
    character(len=70) :: outputfolder
    double precision ::  numbse
    call optprop_files(outputfolder, int(numbse), "bse_diel-pol_", &
                       [character(len=2) :: "x", "y", "z", "sp", "sm"], 5, "bse_", "-pol")
  end subroutine bseoptproppol

  subroutine spoptprop(numbse,outputfolder)
    character(len=70) :: outputfolder
    double precision ::  numbse
    call optprop_files(outputfolder, int(numbse), "sp_diel_", &
                       [character(len=2) :: "xx", "yy", "zz", "xy", "xz", "yz"], 6, "sp_", "")
  end subroutine spoptprop

  subroutine spoptproppol(numbse,outputfolder)
    character(len=70) :: outputfolder
    double precision ::  numbse
    call optprop_files(outputfolder, int(numbse), "sp_diel-pol_", &
                       [character(len=2) :: "x", "y", "z", "sp", "sm"], 5, "sp_", "-pol")
  end subroutine spoptproppol

  ! lifetime (src/module_bse.F90:3271-3349): bse_opt_diel.dat -> exciton_lifetime.dat
  subroutine lifetime(sysdim,numbse,ngrid,rlat,nc,nv,outputfolder)
    integer :: nc,nv
    double precision :: numbse
    integer,dimension(3) :: ngrid
    double precision,dimension(3,3) :: rlat
    character(len=70) :: outputfolder
    character(len=5) :: sysdim
    double precision, allocatable :: fosc(:,:), lft(:,:)
    if (Process /= 0) return
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    allocate(fosc(dimbse,7), lft(dimbse,4))
    call read_rows(trim(outputfolder)//"/bse_opt_diel.dat", dimbse, 7, fosc)
    call wtb_gpu_check(c_wtb_exciton_lifetime(wtb_gpu_ctx(), trim(sysdim)//c_null_char, ngrid, dimbse, fosc, 0, lft), &
                       'lifetime')
    call wtb_gpu_check(c_wtb_write_exciton_lifetime(wtb_cstr(outputfolder,"/exciton_lifetime.dat"), dimbse, fosc(:,1), &
                       lft, 0), 'exciton_lifetime.dat')
    deallocate(fosc, lft)
  end subroutine lifetime

  ! lifetimepol (src/module_bse.F90:3353-3432): bse_opt_diel-pol.dat -> exciton_lifetime-pol.dat
  subroutine lifetimepol(sysdim,numbse,ngrid,rlat,nc,nv,outputfolder)
    integer :: nc,nv
    double precision :: numbse
    integer,dimension(3) :: ngrid
    double precision,dimension(3,3) :: rlat
    character(len=70) :: outputfolder
    character(len=5) :: sysdim
    double precision, allocatable :: fosc(:,:), lft(:,:)
    if (Process /= 0) return
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    allocate(fosc(dimbse,6), lft(dimbse,6))
    call read_rows(trim(outputfolder)//"/bse_opt_diel-pol.dat", dimbse, 6, fosc)
    call wtb_gpu_check(c_wtb_exciton_lifetime(wtb_gpu_ctx(), trim(sysdim)//c_null_char, ngrid, dimbse, fosc, 1, lft), &
                       'lifetimepol')
    call wtb_gpu_check(c_wtb_write_exciton_lifetime(wtb_cstr(outputfolder,"/exciton_lifetime-pol.dat"), dimbse, &
                       fosc(:,1), lft, 1), 'exciton_lifetime-pol.dat')
    deallocate(fosc, lft)
  end subroutine lifetimepol

  ! spoptics (src/module_bse.F90:4802-5071): the IPA records, sorted by transition energy, and their files
  subroutine spoptics(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,rk,meshtype,tmcoef)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params, orbw, kpaths, kpathsbse, outputfolder, calcparms, meshtype
    character(len=5) :: coultype
    double precision,dimension(3) :: ediel
    logical :: tmcoef
    type(wtb_bse_params_t) :: p
    real(c_float), allocatable :: vecres(:,:)
    integer :: dimsp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start spoptics')
    call stage_hr(params)
    dimsp = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, 1.d0, 0.d0, 0.d0, 1.d0, sme, ebse0, &
                       ebsef, numbse)
    allocate(vecres(dimsp,15))
    call wtb_gpu_check(c_wtb_spoptics(wtb_gpu_ctx(), p, vecres), 'spoptics')
    call write_ipa(outputfolder, ngrid, nc, nv, dimsp, vecres, tmcoef)
    deallocate(vecres)
  end subroutine spoptics

  ! spoptpolbz (src/module_bse.F90:4532-4797): BZ-resolved activity -> bz_act_x/y/z/sp/sm.dat, dichroism.dat
  subroutine spoptpolbz(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,rk,meshtype)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params, orbw, kpaths, kpathsbse, outputfolder, calcparms, meshtype
    character(len=5) :: coultype
    double precision,dimension(3) :: ediel
    type(wtb_bse_params_t) :: p
    double precision, allocatable :: act(:,:), kk(:,:)
    character(len=12), dimension(6) :: names
    integer :: nk, j
    if (Process /= 0) return
    call MSG('MODULE_BSE: start spoptpolbz')
    call stage_hr(params)
    nk = ngrid(1)*ngrid(2)*ngrid(3)
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, 1.d0, 0.d0, 0.d0, 1.d0, sme, ebse0, &
                       ebsef, numbse)
    allocate(act(nk,6), kk(nk,3))
    call wtb_gpu_check(c_wtb_spoptpolbz(wtb_gpu_ctx(), p, act), 'spoptpolbz')
    call monhkhorst_pack(ngrid(1),ngrid(2),ngrid(3),mshift,rlat(1,:),rlat(2,:),rlat(3,:),kk)
    names = [character(len=12) :: "bz_act_x", "bz_act_y", "bz_act_z", "bz_act_sp", "bz_act_sm", "dichroism"]
    do j = 1, 6
      call wtb_gpu_check(c_wtb_write_bz_act(wtb_cstr(outputfolder,"/"//trim(names(j))//".dat"), nk, kk, act(:,j)), &
                         trim(names(j)))
    end do
    deallocate(act, kk)
  end subroutine spoptpolbz

  ! bsesolvertemp (src/module_bse.F90:2649-3263): every exciton of the (f_v - f_c)-weighted BSE matrix
  subroutine bsesolvertemp(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,ez,w1,r0,lc,rk,meshtype,bsewf,excwf0,excwff,&
             dtfull,cpol,tmcoef,st,phavg,ta,temp)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params, orbw, kpaths, kpathsbse, outputfolder, calcparms, meshtype
    character(len=5) :: coultype
    character(len=2) :: ta
    double precision,dimension(3) :: ediel
    logical :: bsewf
    integer :: excwf0,excwff
    double precision :: ez,w1,lc,r0
    logical :: cpol,dtfull
    logical :: tmcoef
    double precision :: st,phavg,temp
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    double precision, allocatable :: acts(:,:)
    real(c_float), allocatable :: vecres(:,:)
    type(c_ptr) :: hep
    if (Process /= 0) return
    call MSG('MODULE_BSE: start bsesolvertemp')
    call stage_hr(params)
    dimbse = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    ngkpt = ngrid(1)*ngrid(2)*ngrid(3)
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, ez, w1, r0, lc, sme, ebse0, ebsef, &
                       numbse)
    tp = temp_params(st,phavg,ta,temp,dtfull,cpol)
    if (allocated(Ws)) deallocate(Ws)
    if (allocated(hbse)) deallocate(hbse)
    allocate(Ws(dimbse), acts(dimbse,8))
    hep = c_null_ptr
    if (bsewf) then
      allocate(hbse(dimbse,dimbse))
      hep = c_loc(hbse)
    end if
    call wtb_gpu_check(c_wtb_bsesolvertemp(wtb_gpu_ctx(), p, tp, Ws, acts, hep, c_null_ptr), 'bsesolvertemp')
    call wtb_gpu_check(c_wtb_write_bse_opt_diel(wtb_cstr(outputfolder,"/bse_opt_diel.dat"), dimbse, Ws, acts, 0), &
                       'bse_opt_diel.dat')
    call wtb_gpu_check(c_wtb_write_bse_opt_diel(wtb_cstr(outputfolder,"/bse_opt_diel-pol.dat"), dimbse, Ws, acts, 1), &
                       'bse_opt_diel-pol.dat')
    allocate(vecres(dimbse,15))
    call wtb_gpu_check(c_wtb_spoptics_temp(wtb_gpu_ctx(), p, tp, vecres), 'spoptics')
    call write_ipa(outputfolder, ngrid, nc, nv, dimbse, vecres, tmcoef)
    deallocate(vecres)
    if (bsewf) call write_wf(outputfolder, ngrid, mshift, nc, nv, 1, dimbse, Ws, hbse, excwf0, excwff)
    deallocate(acts)
  end subroutine bsesolvertemp

  ! the Q loop shared by bsebnds and bsebndstemp: all eigenvalues per Q -> bands_bse.dat; with bsewf the
  ! eigenvectors excwf0..excwff of every Q -> exc_wf_<n>_<q>.dat (excwfi2)
  subroutine qloop(outputfolder, kpathsbse, p, tp, withtemp, bsewf, excwf0, excwff, ngrid, mshift, nc, nv)
    character(len=70) :: outputfolder, kpathsbse
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    logical :: withtemp, bsewf
    integer :: excwf0, excwff, nc, nv
    integer,dimension(3) :: ngrid
    double precision,dimension(3) :: mshift
    double precision, allocatable :: qauxv(:,:), exk(:,:), w(:), kk(:,:)
    complex(8), allocatable :: z(:,:)
    integer(c_int), allocatable :: nocpk(:)
    integer :: nq, dim, i, i2, nk, nw
    character(len=200) :: file1
    double precision, target :: q4(4)
    dim = ngrid(1)*ngrid(2)*ngrid(3)*nc*nv
    nk = ngrid(1)*ngrid(2)*ngrid(3)
    call read_qpath(outputfolder, kpathsbse, nq, qauxv)
    allocate(exk(dim,nq))
    if (withtemp) then
      call wtb_gpu_check(c_wtb_bsebndstemp(wtb_gpu_ctx(), p, tp, nq, qauxv, exk), 'bsebndstemp')
    else
      call wtb_gpu_check(c_wtb_bsebnds(wtb_gpu_ctx(), p, nq, qauxv, exk), 'bsebnds')
    end if
    call wtb_gpu_check(c_wtb_write_bands_bse(wtb_cstr(outputfolder,"/bands_bse.dat"), nq, dim, qauxv, exk), &
                       'bands_bse.dat')
    if (bsewf .and. .not. withtemp .and. excwff >= excwf0) then
      nw = excwff - excwf0 + 1
      allocate(w(dim), z(dim,nw), kk(nk,3), nocpk(nk))
      call monhkhorst_pack(ngrid(1),ngrid(2),ngrid(3),mshift,rlat(1,:),rlat(2,:),rlat(3,:),kk)
      call wtb_gpu_check(c_wtb_eigsys_mesh(wtb_gpu_ctx(), nk, kk, nv, nc, c_null_ptr, c_null_ptr, nocpk), 'eigsys')
      do i = 1, nq
        q4 = qauxv(i,:)
        call wtb_gpu_check(c_wtb_bse_q_eigenpairs(wtb_gpu_ctx(), p, q4, excwf0, nw, w, z), 'bsebnds eigenpairs')
        do i2 = excwf0, excwff
          write(file1,'(a7,I0,a1,I0,a4)') 'exc_wf_', i2, "_", i, '.dat'
          call wtb_gpu_check(c_wtb_write_exc_wf(trim(outputfolder)//trim(file1)//c_null_char, nk, nc, nv, nocpk, kk, &
                             c_loc(q4), i2, w(i2), z(:, i2 - excwf0 + 1)), 'excwfi2')
        end do
      end do
      deallocate(w, z, kk, nocpk)
    end if
    deallocate(qauxv, exk)
  end subroutine qloop

  ! bsebnds (src/module_bse.F90:1206-1566): exciton band structure along the kpathsbse path
  subroutine bsebnds(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,ez,w1,r0,lc,rk,meshtype,bsewf,excwf0,excwff)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params, orbw, kpaths, kpathsbse, outputfolder, calcparms, meshtype
    character(len=5) :: coultype
    double precision,dimension(3) :: ediel
    logical :: bsewf
    integer :: excwf0,excwff
    double precision :: ez,w1,lc,r0
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start bsebnds')
    call stage_hr(params)
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, ez, w1, r0, lc, sme, ebse0, ebsef, &
                       numbse)
    tp = temp_params(0.d0, 0.d0, "FA", 0.d0, .true., .true.)
    call qloop(outputfolder, kpathsbse, p, tp, .false., bsewf, excwf0, excwff, ngrid, mshift, nc, nv)
  end subroutine bsebnds

  ! bsebndstemp (src/module_bse.F90:1572-2017): bsebnds with the temperature keys
  subroutine bsebndstemp(nthreads,outputfolder,calcparms,ngrid,nc,nv,numdos, &
             ebse0,ebsef,numbse,sme,ktol,params,kpaths,kpathsbse,orbw,ediel, &
             exc,mshift,coultype,ez,w1,r0,lc,rk,meshtype,bsewf,excwf0,excwff,st,phavg,ta,temp)
    integer :: nthreads
    integer,dimension(3) :: ngrid
    integer :: nc,nv
    double precision :: numdos
    double precision :: ebse0,ebsef,numbse
    double precision :: sme,exc,rk
    double precision,dimension(3) :: mshift
    double precision :: ktol
    character(len=70) :: params, orbw, kpaths, kpathsbse, outputfolder, calcparms, meshtype
    character(len=5) :: coultype
    character(len=2) :: ta
    double precision,dimension(3) :: ediel
    logical :: bsewf
    integer :: excwf0,excwff
    double precision :: ez,w1,lc,r0
    double precision :: st,phavg,temp
    type(wtb_bse_params_t) :: p
    type(wtb_temp_params_t) :: tp
    if (Process /= 0) return
    call MSG('MODULE_BSE: start bsebndstemp')
    call stage_hr(params)
    p = wtb_gpu_params(ngrid, nc, nv, mshift, coultype, .false., ktol, ediel, ez, w1, r0, lc, sme, ebse0, ebsef, &
                       numbse)
    tp = temp_params(st,phavg,ta,temp,.true.,.true.)
    call qloop(outputfolder, kpathsbse, p, tp, .true., bsewf, excwf0, excwff, ngrid, mshift, nc, nv)
  end subroutine bsebndstemp

end module module_bse
