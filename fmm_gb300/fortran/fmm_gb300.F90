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
    public :: get_boxes, get_multipoles, interpolate_electron_fields

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

        integer(c_int) function c_get_boxes(n, coords, ntgt, tcoords, theta, ncrit, p, sizes, idx, bc, bi, opts) &
            bind(C, name="fmm_get_boxes")
            import :: c_int, c_int64_t, c_double, c_ptr
            integer(c_int64_t), value :: n
            real(c_double), intent(in) :: coords(*)
            integer(c_int64_t), value :: ntgt
            real(c_double), intent(in) :: tcoords(*)
            real(c_double), value :: theta
            integer(c_int), value :: ncrit, p
            integer(c_int64_t), intent(inout) :: sizes(2)
            type(c_ptr), value :: idx, bc, bi, opts
        end function

        integer(c_int) function c_get_multipoles(comm, n, coords, mdim, ndens, mp, ntgt, tcoords, theta, ncrit, p, &
                                                 sizes, idx, bc, bm, opts) bind(C, name="fmm_get_multipoles")
            import :: c_int, c_int64_t, c_double, c_ptr
            integer(c_int), value :: comm
            integer(c_int64_t), value :: n
            real(c_double), intent(in) :: coords(*)
            integer(c_int), value :: mdim, ndens
            real(c_double), intent(in) :: mp(*)
            integer(c_int64_t), value :: ntgt
            real(c_double), intent(in) :: tcoords(*)
            real(c_double), value :: theta
            integer(c_int), value :: ncrit, p
            integer(c_int64_t), intent(inout) :: sizes(2)
            type(c_ptr), value :: idx, bc, bm, opts
        end function

        integer(c_int) function c_interpolate_electron_fields(comm, n, coords, nbox, ndens, lx, bi, theta, ncrit, p, &
                                                              field_order, field, opts) &
            bind(C, name="fmm_interpolate_electron_fields")
            import :: c_int, c_int64_t, c_double, c_int32_t, c_ptr
            integer(c_int), value :: comm
            integer(c_int64_t), value :: n
            real(c_double), intent(in) :: coords(*)
            integer(c_int64_t), value :: nbox
            integer(c_int), value :: ndens
            real(c_double), intent(in) :: lx(*)
            integer(c_int32_t), intent(in) :: bi(*)
            real(c_double), value :: theta
            integer(c_int), value :: ncrit, p, field_order
            real(c_double), intent(inout) :: field(*)
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

    ! QM/MM helpers, replacing get_boxes, get_multipoles and
    ! interpolate_electron_fields (src/fmm.F90:1173-1336) with the same dummy
    ! arguments (allocatable outputs allocated here, 1-based indices).  Within
    ! one near-field leaf, idx_near_field lists particles in ascending index
    ! (the reference: insertion order).  The reference's helpers stop in their
    ! final clean-up; these return.  Optional `status` as for field_fmm.
    subroutine get_boxes(coordinates, target_coordinates, theta, ncrit, expansion_order, idx_near_field, &
                         box_coordinates, box_indices, status)
        real(rp), intent(in), target :: coordinates(:, :)
        real(rp), intent(in) :: target_coordinates(:, :)
        real(rp), intent(in) :: theta
        integer(ip), intent(in) :: ncrit
        integer(ip), intent(in) :: expansion_order
        integer(ip), intent(out), allocatable, target :: idx_near_field(:)
        real(rp), intent(out), allocatable, target :: box_coordinates(:, :)
        integer(ip), intent(out), allocatable, target :: box_indices(:)
        integer(ip), intent(out), optional :: status
        integer(c_int64_t) :: sizes(2)
        integer(c_int) :: st
        sizes = 0
        st = c_get_boxes(int(size(coordinates, 1), c_int64_t), coordinates, int(size(target_coordinates, 1), &
                         c_int64_t), target_coordinates, real(theta, c_double), int(ncrit, c_int), &
                         int(expansion_order, c_int), sizes, c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr)
        if (st /= 0) then
            call report(st, "get_boxes", status)
            return
        end if
        allocate (idx_near_field(max(sizes(1), 1_c_int64_t)), box_coordinates(max(sizes(2), 1_c_int64_t), 3), &
                  box_indices(max(sizes(2), 1_c_int64_t)))
        st = c_get_boxes(int(size(coordinates, 1), c_int64_t), coordinates, int(size(target_coordinates, 1), &
                         c_int64_t), target_coordinates, real(theta, c_double), int(ncrit, c_int), &
                         int(expansion_order, c_int), sizes, c_loc(idx_near_field), c_loc(box_coordinates), &
                         c_loc(box_indices), c_null_ptr)
        call shrink_int(idx_near_field, sizes(1))
        call shrink_real2(box_coordinates, sizes(2))
        call shrink_int(box_indices, sizes(2))
        call report(st, "get_boxes", status)
    end subroutine get_boxes

    subroutine get_multipoles(comm, coordinates, multipoles, target_coordinates, theta, ncrit, expansion_order, &
                              idx_near_field, box_coordinates, box_multipoles, status)
        integer(ip), intent(in) :: comm
        real(rp), intent(in), target :: coordinates(:, :)
        real(rp), intent(in), target :: multipoles(:, :, :)
        real(rp), intent(in) :: target_coordinates(:, :)
        real(rp), intent(in) :: theta
        integer(ip), intent(in) :: ncrit
        integer(ip), intent(in) :: expansion_order
        integer(ip), intent(out), allocatable, target :: idx_near_field(:)
        real(rp), intent(out), allocatable, target :: box_coordinates(:, :)
        real(rp), intent(out), allocatable :: box_multipoles(:, :, :)
        integer(ip), intent(out), optional :: status
        integer(c_int64_t) :: sizes(2)
        integer(c_int) :: st
        integer :: nq
        real(rp), allocatable, target :: tmp(:, :, :)
        nq = (expansion_order + 1) * (expansion_order + 2) * (expansion_order + 3) / 6
        sizes = 0
        st = c_get_multipoles(int(comm, c_int), int(size(coordinates, 1), c_int64_t), coordinates, &
                              int(size(multipoles, 2), c_int), int(size(multipoles, 3), c_int), multipoles, &
                              int(size(target_coordinates, 1), c_int64_t), target_coordinates, real(theta, c_double), &
                              int(ncrit, c_int), int(expansion_order, c_int), sizes, c_null_ptr, c_null_ptr, &
                              c_null_ptr, c_null_ptr)
        if (st /= 0) then
            call report(st, "get_multipoles", status)
            return
        end if
        allocate (idx_near_field(max(sizes(1), 1_c_int64_t)), box_coordinates(max(sizes(2), 1_c_int64_t), 3), &
                  tmp(max(sizes(2), 1_c_int64_t), nq, size(multipoles, 3)))
        st = c_get_multipoles(int(comm, c_int), int(size(coordinates, 1), c_int64_t), coordinates, &
                              int(size(multipoles, 2), c_int), int(size(multipoles, 3), c_int), multipoles, &
                              int(size(target_coordinates, 1), c_int64_t), target_coordinates, real(theta, c_double), &
                              int(ncrit, c_int), int(expansion_order, c_int), sizes, c_loc(idx_near_field), &
                              c_loc(box_coordinates), c_loc(tmp), c_null_ptr)
        call shrink_int(idx_near_field, sizes(1))
        call shrink_real2(box_coordinates, sizes(2))
        allocate (box_multipoles(sizes(2), nq, size(multipoles, 3)))
        box_multipoles = tmp(1:sizes(2), :, :)
        call report(st, "get_multipoles", status)
    end subroutine get_multipoles

    subroutine interpolate_electron_fields(comm, coordinates, local_expansion, box_indices, theta, ncrit, &
                                           expansion_order, field_order, field, status)
        integer(ip), intent(in) :: comm
        real(rp), intent(in), target :: coordinates(:, :)
        real(rp), intent(in) :: local_expansion(:, :, :)
        integer(ip), intent(in) :: box_indices(:)
        real(rp), intent(in) :: theta
        integer(ip), intent(in) :: ncrit
        integer(ip), intent(in) :: expansion_order
        integer(ip), intent(in) :: field_order
        real(rp), intent(out) :: field(size(coordinates, 1), (field_order + 1) * (field_order + 2) * &
                                       (field_order + 3) / 6, size(local_expansion, 3))
        integer(ip), intent(out), optional :: status
        call report(c_interpolate_electron_fields(int(comm, c_int), int(size(coordinates, 1), c_int64_t), &
                                                  coordinates, int(size(local_expansion, 1), c_int64_t), &
                                                  int(size(local_expansion, 3), c_int), local_expansion, &
                                                  box_indices, real(theta, c_double), int(ncrit, c_int), &
                                                  int(expansion_order, c_int), int(field_order, c_int), field, &
                                                  c_null_ptr), "interpolate_electron_fields", status)
    end subroutine interpolate_electron_fields

    ! The outputs were allocated with at least one element; cut to the count.
    subroutine shrink_int(a, m)
        integer(ip), allocatable, intent(inout) :: a(:)
        integer(c_int64_t), intent(in) :: m
        integer(ip), allocatable :: b(:)
        if (size(a, kind=c_int64_t) == m) return
        allocate (b(m))
        b = a(1:m)
        call move_alloc(b, a)
    end subroutine shrink_int

    subroutine shrink_real2(a, m)
        real(rp), allocatable, intent(inout) :: a(:, :)
        integer(c_int64_t), intent(in) :: m
        real(rp), allocatable :: b(:, :)
        if (size(a, 1, kind=c_int64_t) == m) return
        allocate (b(m, size(a, 2)))
        b = a(1:m, :)
        call move_alloc(b, a)
    end subroutine shrink_real2

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
