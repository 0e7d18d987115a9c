"""nt2_gb300 -- sm_103a evaluator for NT2's fused elementwise expressions over
nt2::table and its sum/dot reductions.

The product is libnt2gpu.so (C ABI: include/nt2g.h) and the C++ table layer
(nt2_gb300/include/nt2/table.hpp).  This Python package is the binding used
by the tests and the benchmark: ``lib`` (ctypes entry points), ``expr`` (an
NT2-style expression front end that lowers to nt2g programs) and ``build``.
"""
from . import lib  # noqa: F401

__all__ = ["lib"]
