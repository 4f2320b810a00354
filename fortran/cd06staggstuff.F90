! Drop-in for module cd06staggstuff (src/derivatives/cd06stagg.F90): type cd06stagg on the
! GB300 library.  The generic init (init_periodic(nx, dx), init_nonperiodic(nx, dx, isTopEven,
! isBotEven, isTopSided, isBotSided); cd06stagg.F90:170-232) and the generic REAL / CMPLX
! procedures ddz_E2C, ddz_C2E, ddz_C2C, ddz_E2E, d2dz2_C2C, d2dz2_E2E, InterpZ_E2C,
! InterpZ_C2E (cd06stagg.F90:820-1059) on (n1, n2, n) cell and (n1, n2, n + 1) edge arrays.
! As in the reference, init is a subroutine: a failure ends the run (GracefulExit).
module cd06staggstuff
    use kind_parameters, only: rkind
    use iso_c_binding
    use pade_gb300_capi
    implicit none
    private
    public :: cd06stagg

    type cd06stagg
        private
        type(c_ptr) :: h = c_null_ptr
        integer :: n = 0, nE = 0
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure, private :: init_periodic
        procedure, private :: init_nonperiodic
        generic :: init => init_periodic, init_nonperiodic
        procedure :: destroy
        procedure, private :: ddz_E2C_REAL
        procedure, private :: ddz_E2C_CMPLX
        generic :: ddz_E2C => ddz_E2C_REAL, ddz_E2C_CMPLX
        procedure, private :: ddz_C2E_REAL
        procedure, private :: ddz_C2E_CMPLX
        generic :: ddz_C2E => ddz_C2E_REAL, ddz_C2E_CMPLX
        procedure, private :: ddz_C2C_REAL
        procedure, private :: ddz_C2C_CMPLX
        generic :: ddz_C2C => ddz_C2C_REAL, ddz_C2C_CMPLX
        procedure, private :: ddz_E2E_REAL
        procedure, private :: ddz_E2E_CMPLX
        generic :: ddz_E2E => ddz_E2E_REAL, ddz_E2E_CMPLX
        procedure, private :: d2dz2_C2C_REAL
        procedure, private :: d2dz2_C2C_CMPLX
        generic :: d2dz2_C2C => d2dz2_C2C_REAL, d2dz2_C2C_CMPLX
        procedure, private :: d2dz2_E2E_REAL
        procedure, private :: d2dz2_E2E_CMPLX
        generic :: d2dz2_E2E => d2dz2_E2E_REAL, d2dz2_E2E_CMPLX
        procedure, private :: InterpZ_E2C_REAL
        procedure, private :: InterpZ_E2C_CMPLX
        generic :: InterpZ_E2C => InterpZ_E2C_REAL, InterpZ_E2C_CMPLX
        procedure, private :: InterpZ_C2E_REAL
        procedure, private :: InterpZ_C2E_CMPLX
        generic :: InterpZ_C2E => InterpZ_C2E_REAL, InterpZ_C2E_CMPLX
    end type

contains

    subroutine init_periodic(this, nx, dx)
        class(cd06stagg), intent(inout) :: this
        integer, intent(in) :: nx
        real(rkind), intent(in) :: dx
        call this%destroy()
        this%n = nx
        this%nE = nx + 1
        call pade_check(pade_cd06stagg_init_periodic(this%h, int(nx, c_int), real(dx, c_double)), "cd06stagg%init")
    end subroutine

    subroutine init_nonperiodic(this, nx, dx, isTopEven, isBotEven, isTopSided, isBotSided)
        class(cd06stagg), intent(inout) :: this
        integer, intent(in) :: nx
        real(rkind), intent(in) :: dx
        logical, intent(in) :: isTopEven, isBotEven
        logical, intent(in), optional :: isTopSided, isBotSided
        logical :: ts, bs
        ts = .false.
        bs = .false.
        if (present(isTopSided)) ts = isTopSided
        if (present(isBotSided)) bs = isBotSided
        call this%destroy()
        this%n = nx
        this%nE = nx + 1
        call pade_check(pade_cd06stagg_init_nonperiodic(this%h, int(nx, c_int), real(dx, c_double), &
                        c_logical(isTopEven), c_logical(isBotEven), c_logical(ts), c_logical(bs)), "cd06stagg%init")
    end subroutine

    subroutine destroy(this)
        class(cd06stagg), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine ddz_E2C_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 0, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_E2C")
    end subroutine

    subroutine ddz_E2C_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 0, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_E2C")
    end subroutine

    subroutine ddz_C2E_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 1, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_C2E")
    end subroutine

    subroutine ddz_C2E_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 1, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_C2E")
    end subroutine

    subroutine ddz_C2C_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 2, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_C2C")
    end subroutine

    subroutine ddz_C2C_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 2, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_C2C")
    end subroutine

    subroutine ddz_E2E_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 3, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_E2E")
    end subroutine

    subroutine ddz_E2E_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 3, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%ddz_E2E")
    end subroutine

    subroutine d2dz2_C2C_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 4, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%d2dz2_C2C")
    end subroutine

    subroutine d2dz2_C2C_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 4, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%d2dz2_C2C")
    end subroutine

    subroutine d2dz2_E2E_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 5, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%d2dz2_E2E")
    end subroutine

    subroutine d2dz2_E2E_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 5, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%d2dz2_E2E")
    end subroutine

    subroutine InterpZ_E2C_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 6, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%InterpZ_E2C")
    end subroutine

    subroutine InterpZ_E2C_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%nE), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%n), intent(out), target :: fout
        call pade_run(this%h, 6, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%InterpZ_E2C")
    end subroutine

    subroutine InterpZ_C2E_REAL(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        real(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        real(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 7, 3, 0, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%InterpZ_C2E")
    end subroutine

    subroutine InterpZ_C2E_CMPLX(this, fin, fout, n1, n2)
        class(cd06stagg), intent(in) :: this
        integer, intent(in) :: n1, n2
        complex(rkind), dimension(n1, n2, this%n), intent(in), target :: fin
        complex(rkind), dimension(n1, n2, this%nE), intent(out), target :: fout
        call pade_run(this%h, 7, 3, 1, c_loc(fin), c_loc(fout), n1, n2, 0, 0, this%stream, "cd06stagg%InterpZ_C2E")
    end subroutine
end module
