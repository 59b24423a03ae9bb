! Fortran module `fmm` (and the alias module `octree`) with the procedures
! field_direct and field_fmm of the reference library (src/fmm.F90:1338-1400),
! same dummy-argument names and order, implemented on the GB300 library
! through its C ABI (include/fmm_gpu.h).
!
! Differences, all supersets of the reference's interface:
!  * damp_type, damping_factors, is_periodic and box_matrix are optional
!    (the README of the reference documents them as optional; its code makes
!    them required);
!  * an optional `status` argument returns the library status instead of
!    stopping (without it, a failure ends the program with `error stop` and the
!    library's message, as the reference does for an unknown damp type);
!  * `field` is set to the result (the reference adds into it).
!
! Build: compile with any Fortran 2008 compiler and link -lfmm_gb300.
module fmm
    use, intrinsic :: iso_c_binding
    implicit none
    private

    public :: field_direct, field_fmm, release_workspace

    integer, parameter :: ip = c_int32_t
    integer, parameter :: rp = c_double
    integer, parameter :: lp = c_int32_t

    interface
        integer(c_int) function c_field_direct(comm, n, coords, mdim, mp, exw, excl, field_order, field, damp, &
                                               damp_len, dampf, opts) bind(C, name="fmm_field_direct")
            import :: c_int, c_int64_t, c_double, c_int32_t, c_char, c_ptr
            integer(c_int), value :: comm
            integer(c_int64_t), value :: n
            real(c_double), intent(in) :: coords(*)
            integer(c_int), value :: mdim
            real(c_double), intent(in) :: mp(*)
            integer(c_int), value :: exw
            integer(c_int32_t), intent(in) :: excl(*)
            integer(c_int), value :: field_order
            real(c_double), intent(inout) :: field(*)
            character(kind=c_char), intent(in) :: damp(*)
            integer(c_int), value :: damp_len
            type(c_ptr), value :: dampf
            type(c_ptr), value :: opts
        end function

        integer(c_int) function c_field_fmm(comm, n, coords, mdim, mp, exw, excl, theta, ncrit, p, field_order, &
                                            field, damp, damp_len, dampf, is_periodic, box, opts) &
            bind(C, name="fmm_field_fmm")
            import :: c_int, c_int64_t, c_double, c_int32_t, c_char, c_ptr
            integer(c_int), value :: comm
            integer(c_int64_t), value :: n
            real(c_double), intent(in) :: coords(*)
            integer(c_int), value :: mdim
            real(c_double), intent(in) :: mp(*)
            integer(c_int), value :: exw
            integer(c_int32_t), intent(in) :: excl(*)
            real(c_double), value :: theta
            integer(c_int), value :: ncrit, p, field_order
            real(c_double), intent(inout) :: field(*)
            character(kind=c_char), intent(in) :: damp(*)
            integer(c_int), value :: damp_len
            type(c_ptr), value :: dampf
            integer(c_int), value :: is_periodic
            type(c_ptr), value :: box
            type(c_ptr), value :: opts
        end function

        integer(c_int) function c_release_workspace() bind(C, name="fmm_release_workspace")
            import :: c_int
        end function

        type(c_ptr) function c_strerror(status) bind(C, name="fmm_strerror")
            import :: c_int, c_ptr
            integer(c_int), value :: status
        end function
    end interface

contains

    subroutine report(status, what, out_status)
        integer(c_int), intent(in) :: status
        character(len=*), intent(in) :: what
        integer(ip), intent(out), optional :: out_status
        character(kind=c_char), pointer :: msg(:)
        character(len=200) :: text
        integer :: k
        if (present(out_status)) then
            out_status = status
            return
        end if
        if (status == 0) return
        call c_f_pointer(c_strerror(status), msg, [200])
        text = ''
        do k = 1, 200
            if (msg(k) == c_null_char) exit
            text(k:k) = msg(k)
        end do
        error stop "fmm_gb300 " // what // ": " // trim(text)
    end subroutine report

    subroutine field_direct(comm, coordinates, multipoles, exclusions, field_order, field, damp_type, &
                            damping_factors, status)
        integer(ip), intent(in) :: comm
        real(rp), intent(in), target :: coordinates(:, :)
        real(rp), intent(in), target :: multipoles(:, :)
        integer(ip), intent(in) :: exclusions(:, :)
        integer(ip), intent(in) :: field_order
        real(rp), intent(out) :: field(size(coordinates, 1), (field_order + 1) * (field_order + 2) * (field_order + 3) / 6)
        character(len=*), intent(in), optional :: damp_type
        real(rp), intent(in), target, contiguous, optional :: damping_factors(:)
        integer(ip), intent(out), optional :: status
        character(kind=c_char, len=16) :: dt
        integer(c_int) :: st, dl
        type(c_ptr) :: dptr
        dt = ''
        dl = 0
        if (present(damp_type)) then
            dt = trim(damp_type)
            dl = len_trim(damp_type)
        end if
        dptr = c_null_ptr
        if (present(damping_factors)) then
            if (size(damping_factors) > 0) dptr = c_loc(damping_factors(1))
        end if
        st = c_field_direct(int(comm, c_int), int(size(coordinates, 1), c_int64_t), coordinates, &
                            int(size(multipoles, 2), c_int), multipoles, int(size(exclusions, 2), c_int), exclusions, &
                            int(field_order, c_int), field, dt, dl, dptr, c_null_ptr)
        call report(st, "field_direct", status)
    end subroutine field_direct

    subroutine field_fmm(comm, coordinates, multipoles, exclusions, theta, ncrit, expansion_order, field_order, &
                         field, damp_type, damping_factors, is_periodic, box_matrix, status)
        integer(ip), intent(in) :: comm
        real(rp), intent(in), target :: coordinates(:, :)
        real(rp), intent(in), target :: multipoles(:, :)
        integer(ip), intent(in) :: exclusions(:, :)
        real(rp), intent(in) :: theta
        integer(ip), intent(in) :: ncrit
        integer(ip), intent(in) :: expansion_order
        integer(ip), intent(in) :: field_order
        real(rp), intent(out) :: field(size(coordinates, 1), (field_order + 1) * (field_order + 2) * (field_order + 3) / 6)
        character(len=*), intent(in), optional :: damp_type
        real(rp), intent(in), target, contiguous, optional :: damping_factors(:)
        logical(lp), intent(in), optional :: is_periodic
        real(rp), intent(in), target, optional :: box_matrix(3, 3)
        integer(ip), intent(out), optional :: status
        character(kind=c_char, len=16) :: dt
        integer(c_int) :: st, dl, per
        type(c_ptr) :: dptr, bptr
        dt = ''
        dl = 0
        if (present(damp_type)) then
            dt = trim(damp_type)
            dl = len_trim(damp_type)
        end if
        dptr = c_null_ptr
        if (present(damping_factors)) then
            if (size(damping_factors) > 0) dptr = c_loc(damping_factors(1))
        end if
        per = 0
        if (present(is_periodic)) then
            if (is_periodic /= 0) per = 1
        end if
        bptr = c_null_ptr
        if (present(box_matrix)) bptr = c_loc(box_matrix(1, 1))
        st = c_field_fmm(int(comm, c_int), int(size(coordinates, 1), c_int64_t), coordinates, &
                         int(size(multipoles, 2), c_int), multipoles, int(size(exclusions, 2), c_int), exclusions, &
                         real(theta, c_double), int(ncrit, c_int), int(expansion_order, c_int), int(field_order, c_int), &
                         field, dt, dl, dptr, per, bptr, c_null_ptr)
        call report(st, "field_fmm", status)
    end subroutine field_fmm

    ! Frees the device memory the library keeps for this host thread between
    ! calls (it grows to the largest system seen); call it when the FMM is not
    ! needed for a while, e.g. at the end of a run.  Not in the reference,
    ! which frees its tree at the end of every call.
    subroutine release_workspace(status)
        integer(ip), intent(out), optional :: status
        call report(c_release_workspace(), "release_workspace", status)
    end subroutine release_workspace

end module fmm

! The README of the reference calls the module `octree` (`use octree`).
module octree
    use fmm
end module octree
