"""CPU oracle (test infrastructure only) for the fmm field-evaluation path.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, and only as the checker.  The product library
in ``fmm_gb300`` never imports it.
"""
from .oracle import *  # noqa: F401,F403
