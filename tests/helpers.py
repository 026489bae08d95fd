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


def compat_objects(g):
    """(V, P, C_V, C_P) of fdtdpic.compat.MasterController built as the fixture's generator
    built the reference's objects (tests/golden/make_golden.py: make_params + setters)."""
    from fdtdpic.compat import MasterController as MC
    C0 = 299792458.0
    sc = lambda k: g["P_" + k][()].item()  # noqa: E731
    nz, steps, dz, f = int(sc("Nz")), int(sc("timeSteps")), sc("dz"), sc("freq_in")
    P = MC.Params(nz, steps, 0, 0, 1.0, 1.0, 1.0, 1.0, int(sc("x1Loc")), int(sc("x2Loc")),
                  int(sc("materialFrontEdge")), int(sc("materialRearEdge")), int(sc("pmlWidth")),
                  int(sc("nzsrc")), C0 / f, dz, sc("delT"), sc("courantNo"), 1.0 / f, 10.0, False,
                  nz * dz, f, 20)
    P.vidInterval = int(sc("vidInterval"))
    for k in ("TFSF", "SineCont", "Gaussian", "nonLinMed", "LorentzMed", "CPMLXp", "CPMLXm"):
        setattr(P, k, bool(sc(k)))
    P.FreeSpace = not (P.nonLinMed or P.LorentzMed)
    P.Periods, P.Amplitude = sc("Periods"), sc("Amplitude")
    P.epsRe, P.muRe = sc("epsRe"), sc("muRe")
    V = MC.Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
    V.plasmaFreqE, V.gammaE = float(g["plasmaFreqE_in"]), float(g["gammaE"])
    V.omega_0E, V.chi3Stat = float(g["omega_0E"]), float(g["chi3Stat"])
    C_P = MC.CPML_Params(P.dz)
    C_P.kappaMax, C_P.alphaMax = float(g["kappaMax"]), float(g["alphaMax"])
    C_V = MC.CPML_Variables(P.Nz, P.timeSteps)
    return V, P, C_V, C_P


def acubic_bound(want, kerr, dx_rel=1e-10):
    """Per-cell bound on the Kerr amplitude A of a whole run against the reference's.  The
    reference's closed form returns x = 2 j cos(k/3) - b/3a with b/3a far larger than the root,
    so last-place differences between two libraries' pow/acos/cos reach the root magnified by
    |b/3a| / |x|: 64 units in the last place of |b/3a|.  The root also carries the run's own
    difference in Dx (d = -(Dx/eps0)^2 feeds it with twice Dx's relative error, and
    x ~ -d / c): dx_rel of |x|."""
    a, b = float(kerr[0]), float(kerr[1])
    shift = abs(b / (3.0 * a)) if a != 0.0 else 0.0
    return 64.0 * np.finfo(float).eps * shift + dx_rel * np.abs(want)
