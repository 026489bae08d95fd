"""Drop-in modules with the reference's script names and call signatures.

fraserac/Py-FDTD_PIC is a flat folder of scripts (``MasterController``, ``Solver_Engine``,
``BaseFDTD11``, ``Environment_Setup``, ``Material_Def``, ``TransformHandler``,
``genericStability``).  This package offers the same module names, classes and functions, with
the time stepping done by the GPU kernels of libfdtdpic.so (``fdtdpic.engine``):

    from fdtdpic.compat import MasterController as MC, Environment_Setup as envDef
    P = MC.Params(*envDef.envSetup(9e9, 0.7, 7000, 8000), False, 0.7, 9e9, 20, LorentzMed=True)
    V = MC.Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
    C_P, C_V = MC.CPML_Params(P.dz), MC.CPML_Variables(P.Nz, P.timeSteps)
    V, P, C_V, C_P, Exs, Hys = MC.Controller(V, P, C_V, C_P)
    R = MC.results(V, P, C_V, C_P, None, RefCo=True)

Putting this folder on ``sys.path`` lets a reference script import the modules by their bare
names (``import Solver_Engine as SE``).  ``Solver_Engine.PRECISION`` selects FP64 (the default,
within 1e-12 of the reference) or FP32 state.
"""
