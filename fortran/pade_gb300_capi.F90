! ISO_C_BINDING interfaces to libpadeops_gb300 (include/padeops_gb300.h) and the status
! check the shim modules share.
!
! The shim modules (cd06stuff, cd10stuff, cf90stuff, gaussianstuff, cd06staggstuff,
! PadeDerOps, spectralMod, PadePoissonMod, PoissonPeriodicMod) keep the reference's module,
! type and procedure names; each type holds the library handle as type(c_ptr) and each
! procedure forwards to one C entry point.  init functions return the library's status as
! the reference's ierr (0, 2, 3, 7); every other non-zero status ends in the reference's
! GracefulExit with the library's message, as the reference's own checks do.
!
! Arrays pass by address (assumed-size dummies of the bind(C) interfaces), so host arrays
! and device arrays (a CUDA Fortran `device` array, or memory from cudaMalloc seen through
! c_f_pointer) both work: the library stages host arrays and runs device arrays on the
! object's stream (the public `stream` component, null = the legacy default stream).
! Complex(rkind) arrays are interleaved (re, im) pairs, the layout the C side expects.
module pade_gb300_capi
    use iso_c_binding
    implicit none
    public

    integer(c_int), parameter :: PADE_OK = 0

    interface
        function pade_strerror(status) result(msg) bind(C, name="pade_strerror")
            import :: c_int, c_ptr
            integer(c_int), value :: status
            type(c_ptr) :: msg
        end function

        ! ---- cd06 ----
        integer(c_int) function pade_cd06_init(op, n, dx, periodic, bc1, bcn) bind(C, name="pade_cd06_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: op
            integer(c_int), value :: n, periodic, bc1, bcn
            real(c_double), value :: dx
        end function
        integer(c_int) function pade_destroy(op) bind(C, name="pade_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value :: op
        end function
        ! generic operator application (pade_apply): family operation `opcode` along `dir`
        integer(c_int) function pade_apply(op, opcode, dir, is_complex, f, out, na, nb, bc1, bcn, path, stream) &
                bind(C, name="pade_apply")
            import :: c_ptr, c_int
            type(c_ptr), value :: op
            integer(c_int), value :: opcode, dir, is_complex, na, nb, bc1, bcn, path
            type(c_ptr), value :: f, out, stream
        end function
        ! ---- cd10 / cf90 / gaussian / cd06stagg init ----
        integer(c_int) function pade_cd10_init(op, n, dx, periodic, bc1, bcn) bind(C, name="pade_cd10_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: op
            integer(c_int), value :: n, periodic, bc1, bcn
            real(c_double), value :: dx
        end function
        integer(c_int) function pade_cf90_init(op, n, periodic) bind(C, name="pade_cf90_init")
            import :: c_ptr, c_int
            type(c_ptr) :: op
            integer(c_int), value :: n, periodic
        end function
        integer(c_int) function pade_gaussian_init(op, n, periodic) bind(C, name="pade_gaussian_init")
            import :: c_ptr, c_int
            type(c_ptr) :: op
            integer(c_int), value :: n, periodic
        end function
        integer(c_int) function pade_cd06stagg_init_periodic(op, n, dx) bind(C, name="pade_cd06stagg_init_periodic")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: op
            integer(c_int), value :: n
            real(c_double), value :: dx
        end function
        integer(c_int) function pade_cd06stagg_init_nonperiodic(op, n, dx, isTopEven, isBotEven, isTopSided, &
                isBotSided) bind(C, name="pade_cd06stagg_init_nonperiodic")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: op
            integer(c_int), value :: n, isTopEven, isBotEven, isTopSided, isBotSided
            real(c_double), value :: dx
        end function

        ! ---- Pade6stagg ----
        integer(c_int) function pade_pade6stagg_init(p, nz, dz, scheme, isPeriodic) bind(C, name="pade_pade6stagg_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: p
            integer(c_int), value :: nz, scheme, isPeriodic
            real(c_double), value :: dz
        end function
        integer(c_int) function pade_pade6stagg_destroy(p) bind(C, name="pade_pade6stagg_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value :: p
        end function
        integer(c_int) function pade_pade6stagg_apply(p, op, is_complex, fin, fout, n1, n2, bot, top, stream) &
                bind(C, name="pade_pade6stagg_apply")
            import :: c_ptr, c_int
            type(c_ptr), value :: p
            integer(c_int), value :: op, is_complex, n1, n2, bot, top
            type(c_ptr), value :: fin, fout, stream
        end function
        integer(c_int) function pade_pade6stagg_getModifiedWavenumbers(p, k, kp, n) &
                bind(C, name="pade_pade6stagg_getModifiedWavenumbers")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: p
            real(c_double), intent(in) :: k(*)
            real(c_double), intent(out) :: kp(*)
            integer(c_int), value :: n
        end function
        integer(c_int) function pade_pade6stagg_getApproxPoincareConstant(p, c) &
                bind(C, name="pade_pade6stagg_getApproxPoincareConstant")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: p
            real(c_double), intent(out) :: c
        end function

        ! ---- spectral layer and Poisson solvers ----
        integer(c_int) function pade_spectral_init(sp, nx, ny, nz, dx, dy, fix_oddball) bind(C, name="pade_spectral_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: sp
            integer(c_int), value :: nx, ny, nz, fix_oddball
            real(c_double), value :: dx, dy
        end function
        integer(c_int) function pade_spectral_destroy(sp) bind(C, name="pade_spectral_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value :: sp
        end function
        integer(c_int) function pade_spectral_fft(sp, fin, fout, stream) bind(C, name="pade_spectral_fft")
            import :: c_ptr, c_int
            type(c_ptr), value :: sp, fin, fout, stream
        end function
        integer(c_int) function pade_spectral_ifft(sp, fin, fout, set_oddball, stream) bind(C, name="pade_spectral_ifft")
            import :: c_ptr, c_int
            type(c_ptr), value :: sp, fin, fout, stream
            integer(c_int), value :: set_oddball
        end function
        integer(c_int) function pade_poisson_periodic_init(p, sp, dx, dy, dz) bind(C, name="pade_poisson_periodic_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: p
            type(c_ptr), value :: sp
            real(c_double), value :: dx, dy, dz
        end function
        integer(c_int) function pade_poisson_wall_init(p, sp, dx, dy, dz, Lz, stokes) bind(C, name="pade_poisson_wall_init")
            import :: c_ptr, c_int, c_double
            type(c_ptr) :: p
            type(c_ptr), value :: sp
            real(c_double), value :: dx, dy, dz, Lz
            integer(c_int), value :: stokes
        end function
        integer(c_int) function pade_poisson_destroy(p) bind(C, name="pade_poisson_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value :: p
        end function
        integer(c_int) function pade_poisson_projection(p, uhat, vhat, what, stream) bind(C, name="pade_poisson_projection")
            import :: c_ptr, c_int
            type(c_ptr), value :: p, uhat, vhat, what, stream
        end function
        integer(c_int) function pade_poisson_get_pressure(p, uhat, vhat, what, pressure, stream) &
                bind(C, name="pade_poisson_get_pressure")
            import :: c_ptr, c_int
            type(c_ptr), value :: p, uhat, vhat, what, pressure, stream
        end function
        integer(c_int) function pade_poisson_get_pressure_and_update_rhs(p, uhat, vhat, what, pressure, stream) &
                bind(C, name="pade_poisson_get_pressure_and_update_rhs")
            import :: c_ptr, c_int
            type(c_ptr), value :: p, uhat, vhat, what, pressure, stream
        end function
        integer(c_int) function pade_poisson_divergence_check(p, uhat, vhat, what, divergence, fix_div, maxdiv, stream) &
                bind(C, name="pade_poisson_divergence_check")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: p, uhat, vhat, what, divergence, stream
            integer(c_int), value :: fix_div
            real(c_double), intent(out) :: maxdiv
        end function
        integer(c_int) function pade_poisson3d_init(p, nx, ny, nz, dx, dy, dz, dir_id, modkx, modky, modkz) &
                bind(C, name="pade_poisson3d_init")
            import :: c_ptr, c_int, c_double, c_funptr
            type(c_ptr) :: p
            integer(c_int), value :: nx, ny, nz, dir_id
            real(c_double), value :: dx, dy, dz
            type(c_funptr), value :: modkx, modky, modkz
        end function
        integer(c_int) function pade_poisson3d_destroy(p) bind(C, name="pade_poisson3d_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value :: p
        end function
        integer(c_int) function pade_poisson3d_solve(p, rhs, f, stream) bind(C, name="pade_poisson3d_solve")
            import :: c_ptr, c_int
            type(c_ptr), value :: p, rhs, f, stream
        end function
    end interface

contains

    ! The library's message of a status, as a Fortran string
    function pade_message(status) result(msg)
        integer(c_int), intent(in) :: status
        character(len=:), allocatable :: msg
        character(kind=c_char), pointer :: s(:)
        type(c_ptr) :: p
        integer :: n
        p = pade_strerror(status)
        if (.not. c_associated(p)) then
            msg = "unknown status"
            return
        end if
        call c_f_pointer(p, s, [256])
        n = 0
        do while (n < 256)
            if (s(n + 1) == c_null_char) exit
            n = n + 1
        end do
        allocate(character(len=n) :: msg)
        msg = transfer(s(1:n), msg)
    end function

    ! A non-zero status ends the run like the reference's own failures (exits.F90:27-33);
    ! the reference's codes (below 1000) are forwarded as they are
    subroutine pade_check(status, where)
        use exits, only: GracefulExit
        integer(c_int), intent(in) :: status
        character(len=*), intent(in) :: where
        if (status /= PADE_OK) call GracefulExit(where//": "//pade_message(status), int(status))
    end subroutine

    ! One operator application through pade_apply (double-float path, FP64 in and out)
    subroutine pade_run(h, opcode, dir, cplx, f, out, na, nb, bc1, bcn, stream, where)
        type(c_ptr), intent(in) :: h, f, out, stream
        integer, intent(in) :: opcode, dir, cplx, na, nb, bc1, bcn
        character(len=*), intent(in) :: where
        call pade_check(pade_apply(h, int(opcode, c_int), int(dir, c_int), int(cplx, c_int), f, out, int(na, c_int), &
                                   int(nb, c_int), int(bc1, c_int), int(bcn, c_int), 0_c_int, stream), where)
    end subroutine

    pure integer(c_int) function c_logical(l)
        logical, intent(in) :: l
        c_logical = merge(1_c_int, 0_c_int, l)
    end function
end module
