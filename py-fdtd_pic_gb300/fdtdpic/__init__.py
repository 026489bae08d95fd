"""fdtdpic: GB300-native 1D FDTD/PIC time stepping (hand-written sm_103a CUDA via a C ABI).

Host-side entry points:
  fdtdpic.engine.run(grids, precision)      run grids (one launch for all resident grids)
  fdtdpic.grid.grids_from_reference(...)    grids of a reference integrator call
  fdtdpic.sweep / fdtdpic.pic / fdtdpic.server  batched sweeps, beam PIC, served requests
The reference-compatible modules (MasterController, Solver_Engine, BaseFDTD11, ...) are in
fdtdpic.compat and call into this package.
"""
from ._lib import build, lib  # noqa: F401

__all__ = ["build", "lib"]
