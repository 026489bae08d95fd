"""The set-up functions of fdtdpic.compat.BaseFDTD11 and of the legacy fdtdpic.compat.BaseFDTD
(host code, numpy) against the reference's own functions run on the same inputs
(tests/golden/stepops.npz, written by make_golden.py from BaseFDTD11.py and BaseFDTD.py):
the CPML set-up chain of boundCondManager (Solver_Engine.py:70-87), the legacy update
coefficients and source, and the host-only history shuffles, bit for bit."""
from types import SimpleNamespace

import numpy as np
import pytest

from helpers import load

CHAIN = ("CPML_ScalingCalc", "CPML_Ex_RC_Define", "CPML_HY_RC_Define", "CPML_Ex_Update_Coef",
         "CPML_Hy_Update_Coef", "denominators")
CV_ARRAYS = ("psi_Ex", "psi_Hy", "beX", "ceX", "bmY", "cmY", "Cb", "C2", "den_Exdz",
             "den_Hydz", "kappa_Ex", "kappa_Hy", "sigma_Ex", "sigma_Hy", "alpha_Ex", "alpha_Hy",
             "eLoss_CPML", "mLoss_CPML", "Ca", "Cc", "C1", "C3")
INT_KEYS = ("Nz", "pmlWidth", "materialFrontEdge", "materialRearEdge", "nzsrc")


def objects(g, tag):
    """V, P, C_V, C_P of the compat classes carrying the fixture's parameters."""
    from fdtdpic.compat import MasterController as MC
    sc = {k[len(tag) + 6:]: g[k][()].item() for k in g.files if k.startswith(tag + "_scal_")}
    P = SimpleNamespace(**{k: (int(v) if k in INT_KEYS else v) for k, v in sc.items()})
    P.timeSteps, P.CPMLXp, P.CPMLXm, P.TFSF = 64, True, True, False
    V = MC.Variables(P.Nz, P.timeSteps, 16, 1)
    for k in ("plasmaFreqE", "omega_0E", "gammaE", "chi3Stat", "alpha3"):
        setattr(V, k, sc[k])
    C_P = SimpleNamespace(**{k: sc[k] for k in ("kappaMax", "sigmaOpt", "alphaMax", "r_scale",
                                                "r_a_scale")})
    C_V = MC.CPML_Variables(P.Nz, P.timeSteps)
    return V, P, C_V, C_P


@pytest.mark.parametrize("tag", ["b11", "b0"])
def test_cpml_setup_chain_equals_reference(tag):
    from fdtdpic.compat import BaseFDTD, BaseFDTD11
    mod = BaseFDTD11 if tag == "b11" else BaseFDTD
    g = load("stepops")
    V, P, C_V, C_P = objects(g, tag)
    mod.FieldInit(V, P)
    V.UpHyMat, V.UpExMat = mod.EmptySpaceCalc(V, P)
    if tag == "b0":
        V.epsilon, V.mu, *_ = mod.Material(V, P)
        UpHy, UpEx = mod.UpdateCoef(V, P)
        np.testing.assert_array_equal(UpHy, g["b0_UpdateCoef_UpHyMat"])
        np.testing.assert_array_equal(UpEx, g["b0_UpdateCoef_UpExMat"])
        for k in ("UpExSelf", "UpHySelf", "UpExHcompsCo", "UpHyEcompsCo"):
            np.testing.assert_array_equal(getattr(V, k), g["b0_Material_" + k], err_msg=k)
        for k in ("UpExMat", "UpHyMat"):
            np.testing.assert_array_equal(getattr(V, k), g["b0_EmptySpaceCalc_" + k], err_msg=k)
        import contextlib
        import io
        with contextlib.redirect_stdout(io.StringIO()):
            Exs, Hys = mod.SmoothTurnOn(V, P)
        np.testing.assert_array_equal(Exs, g["b0_SmoothTurnOn_Exs"])
        np.testing.assert_array_equal(Hys, g["b0_SmoothTurnOn_Hys"])
    mod.CPML_FieldInit(V, P, C_V, C_P)
    for fn in CHAIN:
        getattr(mod, fn)(V, P, C_V, C_P)
        for a in CV_ARRAYS:
            np.testing.assert_array_equal(getattr(C_V, a), g[f"{tag}_{fn}_{a}"],
                                          err_msg=f"{fn} {a}")
    if tag == "b11":
        assert C_V.kappa_Hy is C_V.kappa_Ex  # the reference assigns the objects


def test_host_history_shuffles_equal_reference():
    from fdtdpic.compat import BaseFDTD, BaseFDTD11
    g = load("stepops")
    for tag, mod in (("b11", BaseFDTD11), ("b0", BaseFDTD)):
        V, P, C_V, C_P = objects(g, tag)
        for k in ("polarisationCurr", "tempVarPol", "tempTempVarPol", "tempVarE", "tempTempVarE",
                  "Ex"):
            setattr(V, k, g[f"{tag}_in_{k}"].copy())
        if tag == "b11":
            ex_before = V.Ex
            mod.ADE_TempPolCurr(V, P, C_V, C_P)
            assert V.Ex is not ex_before and V.tempVarHy is V.Hy
        else:
            mod.ADE_TempPolCurr(V, P)
        for k in ("tempTempVarPol", "tempVarPol", "tempTempVarE", "tempVarE"):
            key = f"{tag}_ADE_TempPolCurr_{k}"
            want = g[key] if key in g.files else g[f"{tag}_in_{k}"]
            np.testing.assert_array_equal(getattr(V, k), want, err_msg=f"{tag} {k}")


def test_step_op_layout_and_checks():
    """The ctypes struct matches the library's, and the host check refuses stencils that would
    read outside the arrays."""
    import ctypes
    from fdtdpic import stepops as so
    from fdtdpic._lib import lib
    L = lib()
    so.check_layout(L)
    ptrs = (ctypes.c_void_p * so.N_SLOTS)(*([4096] * so.N_SLOTS))
    ok = so.make_op(so.OP_CURL, 1, 100, 0, -1)
    assert L.fdtdpic_step_op_check(ctypes.byref(ok), ptrs, 100) == 0
    bad = so.make_op(so.OP_CURL, 0, 100, 0, -1)  # reads x[-1]
    assert L.fdtdpic_step_op_check(ctypes.byref(bad), ptrs, 100) != 0
    bad = so.make_op(so.OP_CURL, 1, 100, 1, 0)  # reads x[100]
    assert L.fdtdpic_step_op_check(ctypes.byref(bad), ptrs, 100) != 0
    bad = so.make_op(so.OP_PSI, 1, 101, 0, -1)  # past the arrays
    assert L.fdtdpic_step_op_check(ctypes.byref(bad), ptrs, 100) != 0
    nulls = (ctypes.c_void_p * so.N_SLOTS)(4096, 4096, 4096, 0, 0, 0, 0, 0)
    psi = so.make_op(so.OP_PSI, 1, 50, 0, -1)  # needs six arrays
    assert L.fdtdpic_step_op_check(ctypes.byref(psi), nulls, 100) != 0
    assert L.fdtdpic_step_op_check(ctypes.byref(so.make_op(99, 1, 50)), ptrs, 100) != 0
