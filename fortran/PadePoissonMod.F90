! Drop-in for module PadePoissonMod (src/incompressible/PadePoisson.F90): type padepoisson on
! the GB300 library (PadePoisson.F90:60-71): init (130-318) with the reference's argument list,
! PressureProjection (434-624), getPressure (752-898), getPressureAndUpdateRHS (900-1163),
! DivergenceCheck (1165-1246) and destroy.  PeriodicInZ selects the periodic CD06-staggered
! projection, otherwise the walled one (computeStokesPressure adds the wall correction over a
! domain of height Lz).  The spectral object must be this library's spectralMod; derivZ is
! not needed (the library holds its own staggered z operators).
module PadePoissonMod
    use kind_parameters, only: rkind
    use iso_c_binding
    use decomp_2d, only: decomp_info
    use spectralMod, only: spectral
    use PadeDerOps, only: Pade6stagg
    use pade_gb300_capi
    implicit none
    private
    public :: padepoisson

    type padepoisson
        private
        type(c_ptr) :: h = c_null_ptr
        integer :: nx = 0, ny = 0, nz = 0
        logical, public :: PeriodicInZ = .false.
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure :: PressureProjection
        procedure :: DivergenceCheck
        procedure :: getPressure
        procedure :: getPressureAndUpdateRHS
    end type

contains

    subroutine init(this, dx, dy, dz, sp, spE, computeStokesPressure, Lz, storePressure, gpC, derivZ, PeriodicInZ)
        class(padepoisson), intent(inout) :: this
        real(rkind), intent(in) :: dx, dy, dz
        class(spectral), intent(in), target :: sp, spE
        logical, intent(in) :: computeStokesPressure, storePressure
        real(rkind), intent(in), optional :: Lz
        type(decomp_info), intent(in), target :: gpC
        type(Pade6stagg), intent(in), target :: derivZ
        logical, intent(in) :: PeriodicInZ
        real(c_double) :: lz_
        call this%destroy()
        this%nx = sp%nx_r
        this%ny = sp%ny_r
        this%nz = sp%nz_r
        this%PeriodicInZ = PeriodicInZ
        if (PeriodicInZ) then
            call pade_check(pade_poisson_periodic_init(this%h, sp%h, real(dx, c_double), real(dy, c_double), &
                                                       real(dz, c_double)), "padepoisson%init")
        else
            lz_ = real(dz, c_double) * this%nz
            if (present(Lz)) lz_ = real(Lz, c_double)
            call pade_check(pade_poisson_wall_init(this%h, sp%h, real(dx, c_double), real(dy, c_double), &
                            real(dz, c_double), lz_, c_logical(computeStokesPressure)), "padepoisson%init")
        end if
    end subroutine

    subroutine destroy(this)
        class(padepoisson), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_poisson_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine PressureProjection(this, uhat, vhat, what)
        class(padepoisson), intent(inout) :: this
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz), intent(inout), target :: uhat, vhat
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz + 1), intent(inout), target :: what
        call pade_check(pade_poisson_projection(this%h, c_loc(uhat), c_loc(vhat), c_loc(what), this%stream), &
                        "padepoisson%PressureProjection")
    end subroutine

    subroutine getPressure(this, uhat, vhat, what, pressure)
        class(padepoisson), intent(inout) :: this
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz), intent(in), target :: uhat, vhat
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz + 1), intent(in), target :: what
        real(rkind), dimension(this%nx, this%ny, this%nz), intent(inout), target :: pressure
        call pade_check(pade_poisson_get_pressure(this%h, c_loc(uhat), c_loc(vhat), c_loc(what), c_loc(pressure), &
                        this%stream), "padepoisson%getPressure")
    end subroutine

    subroutine getPressureAndUpdateRHS(this, uhat, vhat, what, pressure)
        class(padepoisson), intent(inout) :: this
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz), intent(inout), target :: uhat, vhat
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz + 1), intent(inout), target :: what
        real(rkind), dimension(this%nx, this%ny, this%nz), intent(inout), target :: pressure
        call pade_check(pade_poisson_get_pressure_and_update_rhs(this%h, c_loc(uhat), c_loc(vhat), c_loc(what), &
                        c_loc(pressure), this%stream), "padepoisson%getPressureAndUpdateRHS")
    end subroutine

    subroutine DivergenceCheck(this, uhat, vhat, what, divergence, fixDiv)
        class(padepoisson), intent(inout) :: this
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz), intent(inout), target :: uhat, vhat
        complex(rkind), dimension(this%nx / 2 + 1, this%ny, this%nz + 1), intent(inout), target :: what
        real(rkind), dimension(this%nx, this%ny, this%nz), intent(out), target :: divergence
        logical, optional, intent(in) :: fixDiv
        logical :: fix
        real(c_double) :: maxdiv
        fix = .false.
        if (present(fixDiv)) fix = fixDiv
        call pade_check(pade_poisson_divergence_check(this%h, c_loc(uhat), c_loc(vhat), c_loc(what), &
                        c_loc(divergence), c_logical(fix), maxdiv, this%stream), "padepoisson%DivergenceCheck")
    end subroutine
end module
