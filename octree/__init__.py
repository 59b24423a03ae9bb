"""Python module ``octree`` with the reference's f2py call signatures.

The reference builds ``octree`` with f2py from src/fmm.F90 and exports
``octree.fmm.field_fmm`` and ``octree.fmm.field_direct`` (CMakeLists.txt:21-40).
This package offers the same calls, backed by the GB300 library:

    field = octree.fmm.field_fmm(comm, coordinates, multipoles, exclusions,
                                 theta, ncrit, expansion_order, field_order,
                                 damp_type, damping_factors, is_periodic,
                                 box_matrix)
    field = octree.fmm.field_direct(comm, coordinates, multipoles, exclusions,
                                    field_order, damp_type, damping_factors)

Arrays may be in either memory order; they are converted to Fortran order as
f2py does.  A nonzero library status raises RuntimeError (the reference's
``error stop`` ends the process instead).
"""
import fmm_gb300 as _impl


class _Module:
    """Namespace standing in for the f2py module object ``octree.fmm``."""

    @staticmethod
    def field_fmm(comm, coordinates, multipoles, exclusions, theta, ncrit, expansion_order, field_order,
                  damp_type="", damping_factors=None, is_periodic=False, box_matrix=None, options=None):
        return _impl.field_fmm(comm, coordinates, multipoles, exclusions, theta, ncrit, expansion_order,
                               field_order, damp_type, damping_factors, is_periodic, box_matrix, options=options)

    @staticmethod
    def field_direct(comm, coordinates, multipoles, exclusions, field_order, damp_type="", damping_factors=None,
                     options=None):
        return _impl.field_direct(comm, coordinates, multipoles, exclusions, field_order, damp_type,
                                  damping_factors, options=options)


fmm = _Module()

__all__ = ["fmm"]
