"""fdtdpic: GB300-native 1D FDTD/PIC time stepping (hand-written sm_103a CUDA via a C ABI).

Host-side entry points:
  fdtdpic.engine.run(grids, precision)      run grids (one launch for all resident grids)
  fdtdpic.grid.grids_from_reference(...)    grids of a reference integrator call
The reference-compatible modules (Solver_Engine, BaseFDTD11, MasterController, ...) live one
directory up and call into this package.
"""
from ._lib import build, lib  # noqa: F401

__all__ = ["build", "lib"]
