"""GB300-native SimPLIC volume-fraction advection step.

The compute path is ``libsimplic_cuda.so`` (hand-written CUDA for sm_103a
behind the C ABI in include/simplic.h); this package holds its Python
binding (``capi``), the ``solveVofEqu`` mirror (``solve_vof_equ``), the mesh
generators and the pure-advection harness used by tests and bench.py.
Importing the package does not touch CUDA; the binding builds / loads the
library on first use and raises if it cannot.
"""

__all__ = ["capi", "meshgen", "harness", "solve_vof_equ", "build"]
