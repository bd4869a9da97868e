!> hrweno_gpu - Fortran (ISO_C_BINDING) binding of the GB300 library, libhrweno_gb300.so.
!>
!> It keeps the reference's type and method names, so that a driver written against HR-WENO
!> changes its `use` lines and the construction of its right-hand side, nothing else:
!>
!>   weno(ncells, k, eps, xedges)        src/hrweno_weno.f90:48-50,54-127
!>   w%reconstruct(v, vl, vr)            src/hrweno_weno.f90:44,129-219
!>   rktvd(p, neq, order)                src/hrweno_tvdode.f90:59-61,69-95  (fu -> descriptor p)
!>   mstvd(p, neq)                       src/hrweno_tvdode.f90:63-65,180-201
!>   ode%integrate(u, t, tout, dt, itask) src/hrweno_tvdode.f90:97-178,203-271
!>   ode%fevals, ode%istate              src/hrweno_tvdode.f90:22-28 (here functions of the handle)
!>
!> The reference stores the right-hand side as a procedure pointer (src/hrweno_tvdode.f90:16,
!> 50-57).  A GPU stage kernel cannot call back into Fortran, so the right-hand side is the
!> problem descriptor hrw_problem (include/hrweno_gpu.h), filled by hrw_problem_init and the
!> fields that differ.  Errors stop the program with the library's message, which keeps the
!> reference's text (`error stop`, src/hrweno_weno.f90:75-77).
!>
!> Each object holds a C handle that owns device memory; %destroy() frees it.  There is no
!> final procedure: Fortran finalizes a constructor's function result once `ode = rktvd(...)`
!> has copied it, which would free the handle just copied.
!>
!> The real kind rk of the arrays, eps and the times follows the reference's hrweno_kinds
!> (src/hrweno_kinds.F90:8-17): REAL64 by default, REAL32 when preprocessed with -DREAL32, which
!> selects the library's REAL32 handles (HRW_F32: everything held and computed in FP32, in the
!> reference's operation order).  The adjoint, which the reference does not have, is REAL64.
module hrweno_gpu
  use, intrinsic :: iso_c_binding
  implicit none
  private
  public :: hrw_problem, hrw_problem_init, weno, rktvd, mstvd, adjoint, hrw_error_text, rk
  public :: HRW_NUMERICS_FAST, HRW_NUMERICS_STRICT, HRW_NUMERICS_MIXED

#ifdef REAL32
  integer, parameter :: rk = c_float
  integer(c_int), parameter :: HRW_RK = 1      ! HRW_F32
#else
  integer, parameter :: rk = c_double
  integer(c_int), parameter :: HRW_RK = 0      ! HRW_F64
#endif
  integer(c_int), parameter :: HRW_MEM_HOST = 0
  integer(c_int32_t), parameter :: HRW_NUMERICS_FAST = 0, HRW_NUMERICS_STRICT = 1, &
                                   HRW_NUMERICS_MIXED = 2

  !> struct hrw_problem of include/hrweno_gpu.h (bind(c) follows the C compiler's padding)
  type, bind(c) :: hrw_problem
    integer(c_int32_t) :: kind, ncells(2), k
    real(c_double)     :: eps
    integer(c_int32_t) :: flux, fn(2)
    real(c_double)     :: coef_a(2), coef_b(2), alpha(2)
    integer(c_int32_t) :: bc(2)
    real(c_double)     :: xmin(2), xmax(2)
    type(c_ptr)        :: width(2), rates
    integer(c_int32_t) :: numerics
    type(c_ptr)        :: xedges(2)
  end type

  interface
    subroutine hrw_problem_init(p) bind(c, name="hrw_problem_init")
      import :: hrw_problem
      type(hrw_problem), intent(out) :: p
    end subroutine
    type(c_ptr) function c_last_error() bind(c, name="hrw_last_error")
      import :: c_ptr
    end function
    integer(c_int) function c_weno_create(n, k, eps, xedges, w) bind(c, name="hrw_weno_create")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: n, k
      real(c_double), value :: eps
      type(c_ptr), value :: xedges
      type(c_ptr), intent(out) :: w
    end function
    integer(c_int) function c_weno_reconstruct(w, dtype, mem, v, vl, vr) &
        bind(c, name="hrw_weno_reconstruct")
      import :: c_int, c_ptr
      type(c_ptr), value :: w
      integer(c_int), value :: dtype, mem
      type(c_ptr), value :: v, vl, vr
    end function
    integer(c_int) function c_weno_destroy(w) bind(c, name="hrw_weno_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: w
    end function
    integer(c_int) function c_rktvd_create(p, neq, order, dtype, ode) bind(c, name="hrw_rktvd_create")
      import :: c_int, c_ptr, hrw_problem
      type(hrw_problem), intent(in) :: p
      integer(c_int), value :: neq, order, dtype
      type(c_ptr), intent(out) :: ode
    end function
    integer(c_int) function c_mstvd_create(p, neq, dtype, ode) bind(c, name="hrw_mstvd_create")
      import :: c_int, c_ptr, hrw_problem
      type(hrw_problem), intent(in) :: p
      integer(c_int), value :: neq, dtype
      type(c_ptr), intent(out) :: ode
    end function
    integer(c_int) function c_integrate(ode, mem, u, t, tout, dt, itask) bind(c, name="hrw_integrate")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ode
      integer(c_int), value :: mem, itask
      type(c_ptr), value :: u
      real(c_double), intent(inout) :: t
      real(c_double), value :: tout, dt
    end function
    integer(c_int) function c_ode_info(ode, fevals, istate, nsteps) bind(c, name="hrw_ode_info")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ode
      integer(c_int), intent(out) :: fevals, istate
      integer(c_int64_t), intent(out) :: nsteps
    end function
    integer(c_int) function c_ode_destroy(ode) bind(c, name="hrw_ode_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ode
    end function
    integer(c_int) function c_adjoint_create(p, nseg, checkpoint_every, adj) &
        bind(c, name="hrw_adjoint_create")
      import :: c_int, c_ptr, hrw_problem
      type(hrw_problem), intent(in) :: p
      integer(c_int), value :: nseg, checkpoint_every
      type(c_ptr), intent(out) :: adj
    end function
    integer(c_int) function c_adjoint_gradient(adj, mem, u0, utarget, dt, nsteps, j, grad) &
        bind(c, name="hrw_adjoint_gradient")
      import :: c_int, c_ptr, c_double, c_int64_t
      type(c_ptr), value :: adj, u0, utarget, grad
      integer(c_int), value :: mem
      real(c_double), value :: dt
      integer(c_int64_t), value :: nsteps
      real(c_double), intent(out) :: j(*)
    end function
    integer(c_int) function c_adjoint_destroy(adj) bind(c, name="hrw_adjoint_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: adj
    end function
  end interface

  !> weno(ncells, k, eps, xedges): WENO reconstruction of order 2k-1 on the GPU
  type :: weno
    type(c_ptr) :: h = c_null_ptr
  contains
    procedure :: reconstruct => weno_reconstruct
    procedure :: destroy => weno_destroy
  end type
  interface weno
    module procedure weno_new
  end interface

  !> rktvd(p, neq, order): TVD Runge-Kutta integrator of the right-hand side described by p
  type :: rktvd
    type(c_ptr) :: h = c_null_ptr
  contains
    procedure :: integrate => ode_integrate
    procedure :: fevals => ode_fevals
    procedure :: istate => ode_istate
    procedure :: destroy => ode_destroy
  end type
  interface rktvd
    module procedure rktvd_new
  end interface

  !> mstvd(p, neq): 5-step 3rd-order TVD multistep integrator (RK3 start)
  type, extends(rktvd) :: mstvd
  end type
  interface mstvd
    module procedure mstvd_new
  end interface

  !> adjoint(p, nseg, checkpoint_every): gradient of 0.5 ||u(T) - target||^2 w.r.t. u0
  !> (no counterpart in the reference)
  type :: adjoint
    type(c_ptr) :: h = c_null_ptr
  contains
    procedure :: gradient => adjoint_gradient
    procedure :: destroy => adjoint_destroy
  end type
  interface adjoint
    module procedure adjoint_new
  end interface

contains

  !> hrw_last_error() as a Fortran string
  function hrw_error_text() result(msg)
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: c(:)
    integer :: n
    call c_f_pointer(c_last_error(), c, [4096])
    n = 0
    do while (c(n + 1) /= c_null_char)
      n = n + 1
    end do
    allocate (character(len=n) :: msg)
    msg = transfer(c(1:n), msg)
  end function

  subroutine check(rc)
    integer(c_int), intent(in) :: rc
    if (rc /= 0) error stop hrw_error_text()
  end subroutine

  function weno_new(ncells, k, eps, xedges) result(self)
    integer, intent(in) :: ncells
    integer, intent(in), optional :: k
    real(rk), intent(in), optional :: eps
    real(rk), intent(in), optional :: xedges(0:)  ! xedges(0:ncells)
    type(weno) :: self
    integer(c_int) :: kk
    real(c_double) :: ee
    real(c_double), allocatable, target :: xe64(:)
    type(c_ptr) :: xe
    kk = 0                                 ! 0 / 0.0: the reference's defaults (3, 1e-6)
    if (present(k)) kk = k
    ee = 0
    if (present(eps)) ee = eps             ! a REAL32 value is exact in FP64
    xe = c_null_ptr
    if (present(xedges)) then              ! the reference's size check (src/hrweno_weno.f90:100-109)
      if (size(xedges) /= ncells + 1) error stop "Invalid input 'xedges': size(xedges) /= ncells + 1."
      xe64 = real(xedges, c_double)        ! the library copies the edges at creation
      xe = c_loc(xe64)
    end if
    call check(c_weno_create(ncells, kk, ee, xe, self%h))
  end function

  subroutine weno_reconstruct(self, v, vl, vr)
    class(weno), intent(in) :: self
    real(rk), intent(in), target, contiguous :: v(:)
    real(rk), intent(out), target, contiguous :: vl(:), vr(:)
    call check(c_weno_reconstruct(self%h, HRW_RK, HRW_MEM_HOST, c_loc(v), c_loc(vl), c_loc(vr)))
  end subroutine

  subroutine weno_destroy(self)
    class(weno), intent(inout) :: self
    if (c_associated(self%h)) call check(c_weno_destroy(self%h))
    self%h = c_null_ptr
  end subroutine

  function rktvd_new(p, neq, order) result(self)
    type(hrw_problem), intent(in) :: p
    integer, intent(in) :: neq, order      ! order 1..3, required as in src/hrweno_tvdode.f90:75
    type(rktvd) :: self
    call check(c_rktvd_create(p, neq, order, HRW_RK, self%h))
  end function

  function mstvd_new(p, neq) result(self)
    type(hrw_problem), intent(in) :: p
    integer, intent(in) :: neq
    type(mstvd) :: self
    call check(c_mstvd_create(p, neq, HRW_RK, self%h))
  end function

  subroutine ode_integrate(self, u, t, tout, dt, itask)
    class(rktvd), intent(inout) :: self
    real(rk), intent(inout), target, contiguous :: u(:)
    real(rk), intent(inout) :: t
    real(rk), intent(in) :: tout, dt
    integer, intent(in), optional :: itask
    integer(c_int) :: it
    real(c_double) :: tt
    it = 1
    if (present(itask)) it = itask
    tt = t                                 ! the library returns an FP32 time exactly for HRW_F32
    call check(c_integrate(self%h, HRW_MEM_HOST, c_loc(u), tt, real(tout, c_double), &
                           real(dt, c_double), it))
    t = real(tt, rk)
  end subroutine

  integer function ode_fevals(self)
    class(rktvd), intent(in) :: self
    integer(c_int) :: fe, st
    integer(c_int64_t) :: ns
    call check(c_ode_info(self%h, fe, st, ns))
    ode_fevals = fe
  end function

  integer function ode_istate(self)
    class(rktvd), intent(in) :: self
    integer(c_int) :: fe, st
    integer(c_int64_t) :: ns
    call check(c_ode_info(self%h, fe, st, ns))
    ode_istate = st
  end function

  subroutine ode_destroy(self)
    class(rktvd), intent(inout) :: self
    if (c_associated(self%h)) call check(c_ode_destroy(self%h))
    self%h = c_null_ptr
  end subroutine

  function adjoint_new(p, nseg, checkpoint_every) result(self)
    type(hrw_problem), intent(in) :: p
    integer, intent(in) :: nseg, checkpoint_every
    type(adjoint) :: self
    call check(c_adjoint_create(p, nseg, checkpoint_every, self%h))
  end function

  subroutine adjoint_gradient(self, u0, utarget, dt, nsteps, j, grad)
    class(adjoint), intent(inout) :: self
    real(c_double), intent(in), target, contiguous :: u0(:), utarget(:)
    real(c_double), intent(in) :: dt
    integer(c_int64_t), intent(in) :: nsteps
    real(c_double), intent(out) :: j(:)
    real(c_double), intent(out), target, contiguous :: grad(:)
    call check(c_adjoint_gradient(self%h, HRW_MEM_HOST, c_loc(u0), c_loc(utarget), dt, nsteps, j, &
                                  c_loc(grad)))
  end subroutine

  subroutine adjoint_destroy(self)
    class(adjoint), intent(inout) :: self
    if (c_associated(self%h)) call check(c_adjoint_destroy(self%h))
    self%h = c_null_ptr
  end subroutine
end module hrweno_gpu
