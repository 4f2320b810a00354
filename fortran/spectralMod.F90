! Drop-in for the x-y transform part of module spectralMod (src/incompressible/spectral.F90)
! on the GB300 library: init with the reference's argument list (spectral.F90:867-881) for
! the two-periodic case the library provides (dimTransform = 2, pencil "x"), fft
! (spectral.F90:1413-1430) and ifft (1432-1452), plus the fused entries of the library (the
! i k multipliers and the test filter folded into the inverse transform).  One GPU holds the
! whole grid, so the physical (nx, ny, nz) and spectral (nx/2+1, ny, nz) arrays are the
! global ones.  The dealiasing, the z operators and the other procedures of the reference
! type are outside this library (the LES entry pade_les_* runs them on the device).
module spectralMod
    use kind_parameters, only: rkind
    use iso_c_binding
    use exits, only: GracefulExit
    use pade_gb300_capi
    implicit none
    private
    public :: spectral

    type spectral
        type(c_ptr) :: h = c_null_ptr
        integer :: nx_r = 0, ny_r = 0, nz_r = 0, nx_c = 0, ny_c = 0, nz_c = 0
        type(c_ptr) :: stream = c_null_ptr
    contains
        procedure :: init
        procedure :: destroy
        procedure :: fft
        procedure :: ifft
    end type

contains

    subroutine init(this, pencil, nx_g, ny_g, nz_g, dx, dy, dz, scheme, filt, dimTransform, fixOddball, use2decompFFT, &
                    useConsrvD2, createK, exhaustiveFFT, init_periodicInZ, dealiasF)
        class(spectral), intent(inout) :: this
        character(len=1), intent(in) :: pencil
        integer, intent(in) :: nx_g, ny_g, nz_g
        real(rkind), intent(in) :: dx, dy, dz
        character(len=*), intent(in) :: scheme, filt
        integer, intent(in), optional :: dimTransform
        logical, optional :: fixOddball, use2decompFFT, useConsrvD2
        logical, intent(in), optional :: createK, exhaustiveFFT, init_periodicInZ
        real(rkind), intent(in), optional :: dealiasF
        logical :: fix
        if (pencil /= "x") call GracefulExit("spectral%init: only x pencils (one GPU holds the grid)", 1004)
        if (present(dimTransform)) then
            if (dimTransform /= 2) call GracefulExit("spectral%init: two-periodic (dimTransform = 2) transforms only", 1004)
        end if
        fix = .true.
        if (present(fixOddball)) fix = fixOddball
        call this%destroy()
        this%nx_r = nx_g
        this%ny_r = ny_g
        this%nz_r = nz_g
        this%nx_c = nx_g / 2 + 1
        this%ny_c = ny_g
        this%nz_c = nz_g
        call pade_check(pade_spectral_init(this%h, int(nx_g, c_int), int(ny_g, c_int), int(nz_g, c_int), &
                        real(dx, c_double), real(dy, c_double), c_logical(fix)), "spectral%init")
    end subroutine

    subroutine destroy(this)
        class(spectral), intent(inout) :: this
        integer(c_int) :: rc
        if (c_associated(this%h)) rc = pade_spectral_destroy(this%h)
        this%h = c_null_ptr
    end subroutine

    subroutine fft(this, arr_in, arr_out)
        class(spectral), intent(inout) :: this
        real(rkind), dimension(this%nx_r, this%ny_r, this%nz_r), intent(in), target :: arr_in
        complex(rkind), dimension(this%nx_c, this%ny_c, this%nz_c), intent(out), target :: arr_out
        call pade_check(pade_spectral_fft(this%h, c_loc(arr_in), c_loc(arr_out), this%stream), "spectral%fft")
    end subroutine

    subroutine ifft(this, arr_in, arr_out, setOddball)
        class(spectral), intent(inout) :: this
        complex(rkind), dimension(this%nx_c, this%ny_c, this%nz_c), intent(in), target :: arr_in
        real(rkind), dimension(this%nx_r, this%ny_r, this%nz_r), intent(out), target :: arr_out
        logical, intent(in), optional :: setOddball
        logical :: odd
        odd = .false.
        if (present(setOddball)) odd = setOddball
        call pade_check(pade_spectral_ifft(this%h, c_loc(arr_in), c_loc(arr_out), c_logical(odd), this%stream), &
                        "spectral%ifft")
    end subroutine
end module
