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

and the QM/MM helpers get_boxes, get_multipoles and
interpolate_electron_fields (src/fmm.F90:1173-1336; the helpers that return
allocatable arrays return them as a tuple).

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


    @staticmethod
    def interpolate_electron_fields(comm, coordinates, local_expansion, box_indices, theta, ncrit,
                                    expansion_order, field_order):
        return _impl.interpolate_electron_fields(comm, coordinates, local_expansion, box_indices, theta, ncrit,
                                                 expansion_order, field_order)

    @staticmethod
    def get_boxes(coordinates, target_coordinates, theta, ncrit, expansion_order):
        """(idx_near_field, box_coordinates, box_indices), 1-based."""
        return _impl.get_boxes(coordinates, target_coordinates, theta, ncrit, expansion_order)

    @staticmethod
    def get_multipoles(comm, coordinates, multipoles, target_coordinates, theta, ncrit, expansion_order):
        """(idx_near_field, box_coordinates, box_multipoles)."""
        return _impl.get_multipoles(comm, coordinates, multipoles, target_coordinates, theta, ncrit,
                                    expansion_order)


fmm = _Module()

__all__ = ["fmm"]
