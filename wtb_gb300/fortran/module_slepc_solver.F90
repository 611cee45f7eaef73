! Drop-in replacement of WTB's module_slepc_solver (src/module_slepc_solver.F90): the same module name and the
! same public procedures with the same argument lists, so module_bse and main.F90 compile against it unchanged,
! and the program no longer links PETSc/SLEPc.
!
!   slepc_solver(HX,EX,HE,NX,NE)         (:12-97)   lowest NE eigenpairs of the dense Hermitian HX on the GPU
!                                                     (wtb_slepc_solver: FP64 block eigensolver, relative residual
!                                                     1e-8 and 200 iterations as the reference's Krylov-Schur)
!   slepc_check_results(HX,EX,HE,NX,NE)  (:120-148) every component of HX HE(:,q) - EX(q) HE(:,q) against 10 tols,
!                                                     printed by rank 0 as the reference prints it
module module_slepc_solver
  use MPI_P, only: Process
  use wtb_gpu
  implicit none
  real(8), parameter :: tols = 1.d-8   ! the reference's EPS tolerance (src/module_slepc_solver.F90:39)
contains

  subroutine slepc_solver(HX, EX, HE, NX, NE)
    integer    :: NX, NE
    complex(8) :: HX(NX,NX)
    real(8)    :: EX(NE)
    complex(8) :: HE(NX,NE)
    call wtb_gpu_slepc_solver(HX, EX, HE, NX, NE)
  end subroutine slepc_solver

  subroutine slepc_check_results(HX, EX, HE, NX, NE)
    integer    :: NX, NE
    complex(8) :: HX(NX,NX)
    real(8)    :: EX(NE)
    complex(8) :: HE(NX,NE)
    complex(8), allocatable :: r(:)
    integer    :: q
    logical    :: l_one
    allocate(r(NX))
    l_one = .false.
    do q = 1, NE
      if (Process == 0) print *, 'SLEPc check solution q=', q
      r = matmul(HX, HE(:,q)) - EX(q) * HE(:,q)
      if (any(abs(r) > tols * 10)) then
        if (Process == 0) print *, 'SLEPc solution q=', q, ' is wrong'
        l_one = .true.
      end if
    end do
    if (.not. l_one .and. Process == 0) print *, 'SLEPc all solutions are correct'
    deallocate(r)
  end subroutine slepc_check_results

end module module_slepc_solver
