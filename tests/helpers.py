"""Shared test helpers: reference-shaped parameter objects from golden fixtures."""
import os
from types import SimpleNamespace

import numpy as np

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RUN_CASES = ["freespace_gauss_tfsf", "kerr_kappa3", "kerr_nz1000", "kerr_sinecont_tfsf",
             "lorentz_nz1000", "lorentz_sinecont_tfsf"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def ref_objects(g):
    """P, V, C_P namespaces carrying the fixture's parameter values (reference attribute names)."""
    P = SimpleNamespace()
    for k in g.files:
        if k.startswith("P_"):
            v = g[k][()]
            setattr(P, k[2:], v.item() if hasattr(v, "item") else v)
    for k in ("Nz", "timeSteps", "materialFrontEdge", "materialRearEdge", "pmlWidth", "nzsrc",
              "x1Loc", "x2Loc", "vidInterval"):
        setattr(P, k, int(getattr(P, k)))
    for k in ("TFSF", "SineCont", "Gaussian", "nonLinMed", "LorentzMed", "CPMLXp", "CPMLXm"):
        setattr(P, k, bool(getattr(P, k)))
    V = SimpleNamespace(plasmaFreqE=float(g["plasmaFreqE_in"]), gammaE=float(g["gammaE"]),
                        omega_0E=float(g["omega_0E"]), chi3Stat=float(g["chi3Stat"]),
                        alpha3=float(g["alpha3"]))
    C_P = SimpleNamespace(kappaMax=float(g["kappaMax"]), r_scale=float(g["r_scale"]),
                          r_a_scale=float(g["r_a_scale"]), sigmaOpt=float(g["sigmaOpt"]),
                          alphaMax=float(g["alphaMax"]))
    return P, V, C_P


def integrator_of(g):
    return str(g["integrator"])


def sources_of(g):
    if bool(g["source_supplied"]):
        return g["Exs"], g["Hys"]
    return None, None
