! Drop-in for module gaussianstuff (src/filters/gaussian.F90): type gaussian on the GB300 library.
! init(n, periodic) -> ierr (gaussian.F90:74-93; filters 104-582); filter1, filter2 and the generic filter3 (REAL and
! CMPLX) with the optional boundary codes (default 0).
module gaussianstuff
    use kind_parameters, only: rkind
    use iso_c_binding
    use pade_gb300_capi
    implicit none
    private
    public :: gaussian

    type gaussian
        private
        type(c_ptr) :: h = c_null_ptr
        integer :: n = 0
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure :: filter1
        procedure :: filter2
        procedure, private :: filter3_real
        procedure, private :: filter3_cmplx
        generic :: filter3 => filter3_real, filter3_cmplx
    end type

contains

    function init(this, n_, periodic_) result(ierr)
        class(gaussian), intent(inout) :: this
        integer, intent(in) :: n_
        logical, intent(in) :: periodic_
        integer :: ierr
        call this%destroy()
        this%n = n_
        ierr = int(pade_gaussian_init(this%h, int(n_, c_int), c_logical(periodic_)))
    end function

    subroutine destroy(this)
        class(gaussian), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine filter1(this, f, ff, na, nb, bc1_, bcn_)
        class(gaussian), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(this%n, na, nb), intent(in), target :: f
        real(rkind), dimension(this%n, na, nb), intent(out), target :: ff
        integer, optional, intent(in) :: bc1_, bcn_
        integer :: bc1, bcn
        bc1 = 0
        bcn = 0
        if (present(bc1_)) bc1 = bc1_
        if (present(bcn_)) bcn = bcn_
        call pade_run(this%h, 0, 1, 0, c_loc(f), c_loc(ff), na, nb, bc1, bcn, this%stream, "gaussian%filter1")
    end subroutine

    subroutine filter2(this, f, ff, na, nb, bc1_, bcn_)
        class(gaussian), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, this%n, nb), intent(in), target :: f
        real(rkind), dimension(na, this%n, nb), intent(out), target :: ff
        integer, optional, intent(in) :: bc1_, bcn_
        integer :: bc1, bcn
        bc1 = 0
        bcn = 0
        if (present(bc1_)) bc1 = bc1_
        if (present(bcn_)) bcn = bcn_
        call pade_run(this%h, 0, 2, 0, c_loc(f), c_loc(ff), na, nb, bc1, bcn, this%stream, "gaussian%filter2")
    end subroutine

    subroutine filter3_real(this, f, ff, na, nb, bc1_, bcn_)
        class(gaussian), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, nb, this%n), intent(in), target :: f
        real(rkind), dimension(na, nb, this%n), intent(out), target :: ff
        integer, optional, intent(in) :: bc1_, bcn_
        integer :: bc1, bcn
        bc1 = 0
        bcn = 0
        if (present(bc1_)) bc1 = bc1_
        if (present(bcn_)) bcn = bcn_
        call pade_run(this%h, 0, 3, 0, c_loc(f), c_loc(ff), na, nb, bc1, bcn, this%stream, "gaussian%filter3_real")
    end subroutine

    subroutine filter3_cmplx(this, f, ff, na, nb, bc1_, bcn_)
        class(gaussian), intent(in) :: this
        integer, intent(in) :: na, nb
        complex(rkind), dimension(na, nb, this%n), intent(in), target :: f
        complex(rkind), dimension(na, nb, this%n), intent(out), target :: ff
        integer, optional, intent(in) :: bc1_, bcn_
        integer :: bc1, bcn
        bc1 = 0
        bcn = 0
        if (present(bc1_)) bc1 = bc1_
        if (present(bcn_)) bcn = bcn_
        call pade_run(this%h, 0, 3, 1, c_loc(f), c_loc(ff), na, nb, bc1, bcn, this%stream, "gaussian%filter3_cmplx")
    end subroutine
end module
