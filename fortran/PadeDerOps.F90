! Drop-in for module PadeDerOps (src/incompressible/PadeDerOps.F90): type Pade6stagg on the
! GB300 library (PadeDerOps.F90:22-53).  init(gpC, sp_gpC, gpE, sp_gpE, dz, scheme,
! isPeriodic, spectC) keeps the decomposition pointers for the array extents (gp%zsz for real,
! sp_gp%zsz for complex fields); the nine non-periodic cd06stagg variants and their selection
! by (bot, top) live in the library (pade_pade6stagg_*).  Scheme fourierColl needs spectral's
! z transforms, which this library does not provide: init then ends with GracefulExit.
module PadeDerOps
    use kind_parameters, only: rkind
    use iso_c_binding
    use decomp_2d, only: decomp_info
    use pade_gb300_capi
    implicit none
    private
    public :: Pade6stagg, fd02, cd06, fourierColl

    integer, parameter :: fd02 = 0
    integer, parameter :: cd06 = 1
    integer, parameter :: fourierColl = 2

    type Pade6stagg
        private
        type(c_ptr) :: h = c_null_ptr
        type(decomp_info), pointer :: gp => null(), sp_gp => null()
        integer, public :: scheme = 1
        real(rkind), public :: dz = 0
        logical, public :: isPeriodic = .false.
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure :: getModifiedWavenumbers
        procedure :: getApproxPoincareConstant
        procedure, private :: ddz_C2E_real
        procedure, private :: ddz_C2E_cmplx
        generic :: ddz_C2E => ddz_C2E_real, ddz_C2E_cmplx
        procedure, private :: ddz_E2C_real
        procedure, private :: ddz_E2C_cmplx
        generic :: ddz_E2C => ddz_E2C_real, ddz_E2C_cmplx
        procedure, private :: interpz_C2E_real
        procedure, private :: interpz_C2E_cmplx
        generic :: interpz_C2E => interpz_C2E_real, interpz_C2E_cmplx
        procedure, private :: interpz_E2C_real
        procedure, private :: interpz_E2C_cmplx
        generic :: interpz_E2C => interpz_E2C_real, interpz_E2C_cmplx
        procedure, private :: d2dz2_C2C_real
        procedure, private :: d2dz2_C2C_cmplx
        generic :: d2dz2_C2C => d2dz2_C2C_real, d2dz2_C2C_cmplx
        procedure, private :: d2dz2_E2E_real
        procedure, private :: d2dz2_E2E_cmplx
        generic :: d2dz2_E2E => d2dz2_E2E_real, d2dz2_E2E_cmplx
    end type

contains

    subroutine init(this, gpC, sp_gpC, gpE, sp_gpE, dz, scheme, isPeriodic, spectC)
        class(Pade6stagg), intent(inout) :: this
        type(decomp_info), intent(in), target :: gpC, sp_gpC, gpE, sp_gpE
        real(rkind), intent(in) :: dz
        integer, intent(in) :: scheme
        logical, intent(in) :: isPeriodic
        class(*), intent(in), target, optional :: spectC
        call this%destroy()
        this%gp => gpC
        this%sp_gp => sp_gpC
        this%scheme = scheme
        this%dz = dz
        this%isPeriodic = isPeriodic
        call pade_check(pade_pade6stagg_init(this%h, int(gpC%zsz(3), c_int), real(dz, c_double), int(scheme, c_int), &
                                             c_logical(isPeriodic)), "Pade6stagg%init")
    end subroutine

    subroutine destroy(this)
        class(Pade6stagg), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_pade6stagg_destroy(this%h)
        this%h = c_null_ptr
        nullify(this%gp, this%sp_gp)
    end subroutine

    subroutine getModifiedWavenumbers(this, k, kp)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(:), intent(in) :: k
        real(rkind), dimension(:), intent(out) :: kp
        call pade_check(pade_pade6stagg_getModifiedWavenumbers(this%h, k, kp, int(size(k), c_int)), &
                        "Pade6stagg%getModifiedWavenumbers")
    end subroutine

    function getApproxPoincareConstant(this) result(const)
        class(Pade6stagg), intent(in) :: this
        real(rkind) :: const
        real(c_double) :: c
        call pade_check(pade_pade6stagg_getApproxPoincareConstant(this%h, c), "Pade6stagg%getApproxPoincareConstant")
        const = c
    end function

    subroutine ddz_C2E_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 0_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%ddz_C2E")
    end subroutine

    subroutine ddz_C2E_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 0_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%ddz_C2E")
    end subroutine

    subroutine ddz_E2C_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 1_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%ddz_E2C")
    end subroutine

    subroutine ddz_E2C_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 1_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%ddz_E2C")
    end subroutine

    subroutine interpz_C2E_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 2_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%interpz_C2E")
    end subroutine

    subroutine interpz_C2E_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 2_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%interpz_C2E")
    end subroutine

    subroutine interpz_E2C_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 3_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%interpz_E2C")
    end subroutine

    subroutine interpz_E2C_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 3_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%interpz_E2C")
    end subroutine

    subroutine d2dz2_C2C_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 4_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%d2dz2_C2C")
    end subroutine

    subroutine d2dz2_C2C_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3)), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 4_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%d2dz2_C2C")
    end subroutine

    subroutine d2dz2_E2E_real(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(in), target :: input
        real(rkind), dimension(this%gp%zsz(1), this%gp%zsz(2), this%gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 5_c_int, 0_c_int, c_loc(input), c_loc(output), &
                        int(this%gp%zsz(1), c_int), int(this%gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%d2dz2_E2E")
    end subroutine

    subroutine d2dz2_E2E_cmplx(this, input, output, bot, top)
        class(Pade6stagg), intent(in) :: this
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(in), target :: input
        complex(rkind), dimension(this%sp_gp%zsz(1), this%sp_gp%zsz(2), this%sp_gp%zsz(3) + 1), intent(out), target :: output
        integer, intent(in) :: bot, top
        call pade_check(pade_pade6stagg_apply(this%h, 5_c_int, 1_c_int, c_loc(input), c_loc(output), &
                        int(this%sp_gp%zsz(1), c_int), int(this%sp_gp%zsz(2), c_int), int(bot, c_int), int(top, c_int), &
                        this%stream), "Pade6stagg%d2dz2_E2E")
    end subroutine
end module
