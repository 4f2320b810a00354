! Drop-in for module cd06stuff (src/derivatives/cd06.F90): type cd06 on the GB300 library.
! Procedures and arguments as cd06.F90:90-117 (init 129-201, dd1/dd2/dd3 775-839); the
! periodic second derivatives d2d1..d2d3 complete the reference's unfinished cd06der2.
module cd06stuff
    use kind_parameters, only: rkind
    use iso_c_binding
    use pade_gb300_capi
    implicit none
    private
    public :: cd06

    type cd06
        private
        type(c_ptr) :: h = c_null_ptr
        integer :: n = 0
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure :: GetSize
        procedure :: dd1
        procedure :: dd2
        procedure :: dd3
        procedure :: d2d1
        procedure :: d2d2
        procedure :: d2d3
    end type

contains

    pure function GetSize(this) result(val)
        class(cd06), intent(in) :: this
        integer :: val
        val = this%n
    end function

    function init(this, n_, dx_, periodic_, bc1_, bcn_) result(ierr)
        class(cd06), intent(inout) :: this
        integer, intent(in) :: n_
        real(rkind), intent(in) :: dx_
        logical, intent(in) :: periodic_
        integer, intent(in) :: bc1_, bcn_
        integer :: ierr
        call this%destroy()
        this%n = n_
        ierr = int(pade_cd06_init(this%h, int(n_, c_int), real(dx_, c_double), c_logical(periodic_), &
                                  int(bc1_, c_int), int(bcn_, c_int)))
    end function

    subroutine destroy(this)
        class(cd06), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine dd1(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(this%n, na, nb), intent(in), target :: f
        real(rkind), dimension(this%n, na, nb), intent(out), target :: df
        call pade_run(this%h, 1, 1, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%dd1")
    end subroutine

    subroutine dd2(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, this%n, nb), intent(in), target :: f
        real(rkind), dimension(na, this%n, nb), intent(out), target :: df
        call pade_run(this%h, 1, 2, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%dd2")
    end subroutine

    subroutine dd3(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, nb, this%n), intent(in), target :: f
        real(rkind), dimension(na, nb, this%n), intent(out), target :: df
        call pade_run(this%h, 1, 3, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%dd3")
    end subroutine

    subroutine d2d1(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(this%n, na, nb), intent(in), target :: f
        real(rkind), dimension(this%n, na, nb), intent(out), target :: df
        call pade_run(this%h, 2, 1, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%d2d1")
    end subroutine

    subroutine d2d2(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, this%n, nb), intent(in), target :: f
        real(rkind), dimension(na, this%n, nb), intent(out), target :: df
        call pade_run(this%h, 2, 2, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%d2d2")
    end subroutine

    subroutine d2d3(this, f, df, na, nb)
        class(cd06), intent(in) :: this
        integer, intent(in) :: na, nb
        real(rkind), dimension(na, nb, this%n), intent(in), target :: f
        real(rkind), dimension(na, nb, this%n), intent(out), target :: df
        call pade_run(this%h, 2, 3, 0, c_loc(f), c_loc(df), na, nb, 0, 0, this%stream, "cd06%d2d3")
    end subroutine
end module
