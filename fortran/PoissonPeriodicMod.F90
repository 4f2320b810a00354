! Drop-in for module PoissonPeriodicMod (src/utilities/PoissonPeriodic.F90): type
! PoissonPeriodic on the GB300 library (PoissonPeriodic.F90:28-33): init (114-210) with the
! reference's argument list, including the optional modified-wavenumber procedures, the
! generic poisson_solve (in place, out of place; 37-111) and destroy.  The library calls the
! modified-wavenumber procedures during init through C-callable trampolines (module state, so
! inits on several threads at once must be serialised by the caller).
module PoissonPeriodicMod
    use kind_parameters, only: rkind
    use iso_c_binding
    use decomp_2d, only: decomp_info
    use pade_gb300_capi
    implicit none
    private
    public :: PoissonPeriodic

    interface
        subroutine GetModifiedWavenum(kinout)
            import :: rkind
            real(rkind), dimension(:), intent(inout) :: kinout
        end subroutine
    end interface

    type PoissonPeriodic
        private
        type(c_ptr) :: h = c_null_ptr
        integer :: nx_in = 0, ny_in = 0, nz_in = 0
        type(c_ptr), public :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure, private :: poisson_solve_inplace
        procedure, private :: poisson_solve_outofplace
        generic :: poisson_solve => poisson_solve_inplace, poisson_solve_outofplace
    end type

    procedure(GetModifiedWavenum), pointer :: cur_x => null(), cur_y => null(), cur_z => null()

contains

    subroutine tramp(fn, kd, n)
        procedure(GetModifiedWavenum), pointer :: fn
        type(c_ptr), value :: kd
        integer(c_int), value :: n
        real(c_double), pointer :: k(:)
        call c_f_pointer(kd, k, [n])
        call fn(k)
    end subroutine

    subroutine tramp_x(kd, n) bind(C)
        type(c_ptr), value :: kd
        integer(c_int), value :: n
        call tramp(cur_x, kd, n)
    end subroutine
    subroutine tramp_y(kd, n) bind(C)
        type(c_ptr), value :: kd
        integer(c_int), value :: n
        call tramp(cur_y, kd, n)
    end subroutine
    subroutine tramp_z(kd, n) bind(C)
        type(c_ptr), value :: kd
        integer(c_int), value :: n
        call tramp(cur_z, kd, n)
    end subroutine

    subroutine init(this, dx, dy, dz, gp, dir_id, useExhaustiveFFT, Get_ModKx, Get_ModKy, Get_ModKz)
        class(PoissonPeriodic), intent(inout) :: this
        real(rkind), intent(in) :: dx, dy, dz
        class(decomp_info), intent(in), target :: gp
        integer, intent(in) :: dir_id
        logical, intent(in), optional :: useExhaustiveFFT
        procedure(GetModifiedWavenum), optional :: Get_ModKx, Get_ModKy, Get_ModKz
        type(c_funptr) :: fx, fy, fz
        call this%destroy()
        ! one GPU holds the grid: the global extents (the x pencil of gp)
        this%nx_in = gp%xsz(1)
        this%ny_in = gp%xsz(2)
        this%nz_in = gp%xsz(3)
        fx = c_null_funptr
        fy = c_null_funptr
        fz = c_null_funptr
        if (present(Get_ModKx)) then
            cur_x => Get_ModKx
            fx = c_funloc(tramp_x)
        end if
        if (present(Get_ModKy)) then
            cur_y => Get_ModKy
            fy = c_funloc(tramp_y)
        end if
        if (present(Get_ModKz)) then
            cur_z => Get_ModKz
            fz = c_funloc(tramp_z)
        end if
        call pade_check(pade_poisson3d_init(this%h, int(this%nx_in, c_int), int(this%ny_in, c_int), &
                        int(this%nz_in, c_int), real(dx, c_double), real(dy, c_double), real(dz, c_double), &
                        int(dir_id, c_int), fx, fy, fz), "PoissonPeriodic%init")
        nullify(cur_x, cur_y, cur_z)
    end subroutine

    subroutine destroy(this)
        class(PoissonPeriodic), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_poisson3d_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine poisson_solve_inplace(this, rhs)
        class(PoissonPeriodic), intent(inout) :: this
        real(rkind), dimension(this%nx_in, this%ny_in, this%nz_in), intent(inout), target :: rhs
        call pade_check(pade_poisson3d_solve(this%h, c_loc(rhs), c_loc(rhs), this%stream), "PoissonPeriodic%poisson_solve")
    end subroutine

    subroutine poisson_solve_outofplace(this, rhs, f)
        class(PoissonPeriodic), intent(inout) :: this
        real(rkind), dimension(this%nx_in, this%ny_in, this%nz_in), intent(in), target :: rhs
        real(rkind), dimension(this%nx_in, this%ny_in, this%nz_in), intent(out), target :: f
        call pade_check(pade_poisson3d_solve(this%h, c_loc(rhs), c_loc(f), this%stream), "PoissonPeriodic%poisson_solve")
    end subroutine
end module
