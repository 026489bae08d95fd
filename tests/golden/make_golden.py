"""Generate the golden fixtures in this folder by running the reference's own Python code.

The reference (fraserac/Py-FDTD_PIC) is a flat folder of scripts.  As shipped it does not
import: it needs numba, matplotlib and pyttsx3 (absent here) and a ``Tests`` package that does
not exist, and ``MasterController`` runs a whole simulation at import time.  This script makes it
runnable without changing a line of it:

* ``numba`` is replaced by an inert module.  ``njit``/``jit`` return the function unchanged and
  ``jitclass(spec)`` returns a subclass whose ``__setattr__`` applies the declared scalar type of
  each field (``dict(spec)``: the last duplicate wins, as numba's ordered spec does).  A field
  declared ``float32`` therefore holds the float32-rounded value, which then enters float64
  arithmetic, exactly as reading a float32 jitclass member does inside numba.  Arrays are stored
  by reference (no copy), as jitclass members are.
* ``matplotlib``, ``pyttsx3`` and ``Tests.Integration_Tester`` become empty modules,
  ``Tests.genericStability`` is the reference's own ``genericStability.py``.
* ``MasterController.py`` is not imported; its four state classes and their specs are taken out
  of the file with ``ast`` and executed under the jitclass stand-in.
* ``BaseFDTD11.Nonlin_Cubic_Solver`` calls ``CubicEquationSolver.CubicSolver(a,b,c,d)`` and then
  ``solve(CS)``; ``CubicSolver`` does not exist.  The intended callee is ``solve(a,b,c,d)``
  (``CubicEquationSolver.py:29``), so ``CubicSolver`` packs its four arguments and ``solve``
  unpacks them.  Nothing else in the reference is patched.

Run from the repository root with the reference checkout named by ``PYFDTD_REFERENCE``:
``PYFDTD_REFERENCE=<checkout> python tests/golden/make_golden.py`` (about two minutes;
a mode argument writes one fixture alone: ``variants`` -> ``variants.npz``, ``stepops`` ->
``stepops.npz``; ``time`` times the reference's own Kerr integrator instead).  It writes
``*.npz`` beside this file.  The fixtures are committed; tests only read them.
"""
from __future__ import annotations

import ast
import contextlib
import importlib.util
import io
import os
import sys
import types
import warnings

import numpy as np
import scipy
import scipy.constants

REF = os.environ.get("PYFDTD_REFERENCE")
OUT = os.path.dirname(os.path.abspath(__file__))

sys.dont_write_bytecode = True


# ---------------------------------------------------------------------------------------------
# inert stand-ins for the reference's missing imports
# ---------------------------------------------------------------------------------------------
class _NbScalar:
    def __init__(self, name, cast):
        self.name, self.cast = name, cast
        self.dtype = np.dtype("bool" if name == "boolean" else name)  # usable as a numpy dtype

    def __getitem__(self, idx):  # float64[:] / complex128[:, :]
        return _NbArray(self)

    def __repr__(self):
        return self.name


class _NbArray:
    def __init__(self, dtype):
        self.dtype = dtype


def _f32(v):
    return float(np.float32(np.real(v)))


def _f64(v):
    return float(np.real(v)) if np.iscomplexobj(v) else float(v)


_TYPES = {
    "int32": _NbScalar("int32", int),
    "int64": _NbScalar("int64", int),
    "float32": _NbScalar("float32", _f32),
    "float64": _NbScalar("float64", _f64),
    "boolean": _NbScalar("boolean", bool),
    "complex128": _NbScalar("complex128", complex),
}


def _decorator_factory(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


def _jitclass(spec):
    declared = dict(spec)

    def deco(cls):
        def __setattr__(self, name, value):
            t = declared.get(name)
            if isinstance(t, _NbScalar):
                value = t.cast(value)
            object.__setattr__(self, name, value)

        return type(cls.__name__, (cls,), {"__setattr__": __setattr__})

    return deco


def _install_stubs():
    nb = types.ModuleType("numba")
    nb.njit = nb.jit = _decorator_factory
    nb.prange = range
    nb.guvectorize = nb.vectorize = _decorator_factory
    for k, v in _TYPES.items():
        setattr(nb, k, v)
    exp = types.ModuleType("numba.experimental")
    exp.jitclass = _jitclass
    nb.experimental = exp
    typed = types.ModuleType("numba.typed")
    typed.Dict = dict
    nb.typed = typed
    nbtypes = types.ModuleType("numba.types")
    nbtypes.DictType = lambda *a: None
    nbtypes.List = list
    nbtypes.string = str
    nbtypes.optional = lambda *a: None
    nb.types = nbtypes
    sys.modules.update({"numba": nb, "numba.experimental": exp, "numba.typed": typed,
                        "numba.types": nbtypes})

    mpl = types.ModuleType("matplotlib")
    pylab = types.ModuleType("matplotlib.pylab")
    pyplot = types.ModuleType("matplotlib.pyplot")
    animation = types.ModuleType("matplotlib.animation")
    mpl.pylab, mpl.pyplot, mpl.animation = pylab, pyplot, animation
    sys.modules.update({"matplotlib": mpl, "matplotlib.pylab": pylab, "matplotlib.pyplot": pyplot,
                        "matplotlib.animation": animation})
    sys.modules["pyttsx3"] = types.ModuleType("pyttsx3")

    tests_pkg = types.ModuleType("Tests")
    tests_pkg.__path__ = []
    integ = types.ModuleType("Tests.Integration_Tester")
    integ.testerFuncVector = lambda *a, **k: {}
    sys.modules.update({"Tests": tests_pkg, "Tests.Integration_Tester": integ})

    sys.path.insert(0, REF)
    spec = importlib.util.spec_from_file_location("Tests.genericStability",
                                                  os.path.join(REF, "genericStability.py"))
    gstab = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gstab)
    sys.modules["Tests.genericStability"] = gstab
    tests_pkg.genericStability = gstab

    import CubicEquationSolver as ces  # the reference's vendored solver

    raw_solve = ces.solve

    def solve(*args):
        if len(args) == 1:
            args = tuple(args[0])
        return raw_solve(*args)

    ces.CubicSolver = lambda a, b, c, d: (a, b, c, d)
    ces.solve = solve
    return raw_solve


def _load_state_classes():
    """Execute MasterController's spec lists and four jitclasses, nothing else."""
    src = open(os.path.join(REF, "MasterController.py")).read()
    tree = ast.parse(src)
    keep = []
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(
                isinstance(t, ast.Name) and t.id in ("specV", "specP", "specCP", "specCV")
                for t in node.targets):
            keep.append(node)
        elif isinstance(node, ast.ClassDef) and node.name in (
                "Variables", "Params", "CPML_Params", "CPML_Variables"):
            keep.append(node)
    mod = ast.Module(body=keep, type_ignores=[])
    ns = {"np": np, "sci": scipy, "jclass": _jitclass}
    ns.update(_TYPES)
    exec(compile(mod, "MasterController.py", "exec"), ns)
    return ns["Variables"], ns["Params"], ns["CPML_Params"], ns["CPML_Variables"]


# ---------------------------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------------------------
C0 = 299792458.0


def gauss_sine(n_steps, f, dt, t0=200.0, sigma=60.0, amp=1.0):
    """Gaussian-modulated sine, the soft source of the 1000-cell workload."""
    n = np.arange(n_steps, dtype=np.float64)
    return amp * np.exp(-0.5 * ((n - t0) / sigma) ** 2) * np.sin(2.0 * np.pi * f * (n - t0) * dt)


def make_params(Params, *, Nz, steps, dz, sc, front, rear, pml, nzsrc, x1, x2, freq_in):
    dt = sc * dz / C0
    P = Params(Nz, steps, 0, 0, 1.0, 1.0, 1.0, 1.0, x1, x2, front, rear, pml, nzsrc,
               C0 / freq_in, dz, dt, sc, 1.0 / freq_in, 10.0, False, Nz * dz, freq_in, 20)
    P.vidInterval = 50
    return P


def lorentz(V, d_eps, f0, gamma):
    w0 = 2.0 * np.pi * f0
    V.omega_0E = w0
    V.plasmaFreqE = np.sqrt(d_eps) * w0
    V.gammaE = gamma


def run_case(mods, integrator, P, V_setup, source=None, extra_probes=(), keep_history=True):
    Variables, Params, CPML_Params, CPML_Variables = mods["classes"]
    SE, B11 = mods["SE"], mods["B11"]
    V = Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
    V_setup(V)
    C_P = CPML_Params(P.dz)
    C_V = CPML_Variables(P.Nz, P.timeSteps)
    pf_in = V.plasmaFreqE

    trace = {c: [] for c in extra_probes}
    orig_probe = SE.probeSim
    orig_source = SE.SourceManager

    def probe(V_, P_, C_V_, C_P_, counts, *a, **k):
        for c in extra_probes:
            trace[c].append(V_.Ex[c])
        return orig_probe(V_, P_, C_V_, C_P_, counts, *a, **k)

    SE.probeSim = probe
    if source is not None:
        SE.SourceManager = lambda V_, P_, C_V_, C_P_: (source[0].copy(), source[1].copy())
    try:
        with contextlib.redirect_stdout(io.StringIO()), warnings.catch_warnings():
            warnings.simplefilter("ignore")
            fin_be = int(P.timeSteps * 0.7)
            st_af = int(P.timeSteps * 0.05)
            V.x1ColBe = np.zeros(P.timeSteps)
            V.x1ColAf = np.zeros(P.timeSteps)
            out = getattr(SE, integrator)(V, P, C_V, C_P, fin_be, st_af)
    finally:
        SE.probeSim = orig_probe
        SE.SourceManager = orig_source
    Ex, Hy, Exs, Hys, psiE, psiH, be, af = out
    res = dict(
        Ex=np.asarray(Ex, float), Hy=np.asarray(Hy, float), Exs=np.asarray(Exs, float),
        Hys=np.asarray(Hys, float), psi_Ex=np.asarray(psiE, float), psi_Hy=np.asarray(psiH, float),
        x1ColBe=np.asarray(be, float), x1ColAf=np.asarray(af, float),
        Dx=np.asarray(V.Dx, float), polarisationCurr=np.asarray(V.polarisationCurr, float),
        Acubic=np.asarray(V.Acubic, float), Port1=np.asarray(V.Port1, float),
        Port2=np.asarray(V.Port2, float), Ex_History=np.asarray(V.Ex_History, float),
        plasmaFreqE_in=pf_in, plasmaFreqE_out=V.plasmaFreqE,
        omega_0E=V.omega_0E, gammaE=V.gammaE, chi3Stat=V.chi3Stat, alpha3=V.alpha3,
        beX=C_V.beX.copy(), ceX=C_V.ceX.copy(), bmY=C_V.bmY.copy(), cmY=C_V.cmY.copy(),
        Cb=C_V.Cb.copy(), C2=C_V.C2.copy(), den_Exdz=C_V.den_Exdz.copy(),
        den_Hydz=C_V.den_Hydz.copy(), kappaMax=C_P.kappaMax, alphaMax=C_P.alphaMax,
        sigmaOpt=C_P.sigmaOpt, r_scale=C_P.r_scale, r_a_scale=C_P.r_a_scale,
    )
    for c in extra_probes:
        res[f"probe_{c}"] = np.asarray(trace[c], float)
    if not keep_history:
        del res["Ex_History"]
    scal = dict(Nz=P.Nz, timeSteps=P.timeSteps, dz=P.dz, delT=P.delT, courantNo=P.courantNo,
                materialFrontEdge=P.materialFrontEdge, materialRearEdge=P.materialRearEdge,
                pmlWidth=P.pmlWidth, nzsrc=P.nzsrc, x1Loc=P.x1Loc, x2Loc=P.x2Loc,
                freq_in=P.freq_in, permit_0=P.permit_0, permea_0=P.permea_0, CharImp=P.CharImp,
                c0=P.c0, TFSF=P.TFSF, SineCont=P.SineCont, Gaussian=P.Gaussian,
                nonLinMed=P.nonLinMed, LorentzMed=P.LorentzMed, period=P.period,
                Periods=P.Periods, Amplitude=P.Amplitude, vidInterval=P.vidInterval,
                CPMLXp=P.CPMLXp, CPMLXm=P.CPMLXm, epsRe=P.epsRe, muRe=P.muRe)
    res.update({f"P_{k}": v for k, v in scal.items()})
    res["integrator"] = integrator
    res["source_supplied"] = source is not None
    return res


def cubic_cases(raw_solve):
    """Known answers of the reference's solve() (CubicEquationSolver.py:29-90)."""
    rng = np.random.Generator(np.random.PCG64(20261203))
    coeffs = [(1, -6, 11, -6), (1, -3, 3, -1), (0, 0, 2, -4), (0, 1, 0, -4), (2, 0, 0, -16),
              (4.9e-7, 2e-3, 4, -1), (1, 0, 0, 8), (1, 1, 1, -1), (3, -2, 5, -7),
              (1, -2, 1, -1e-9), (1, -3, 3, -1 + 1e-12), (4.9e-5, 0.0128, 21.0, -20.0),
              (4.9e-5, -0.0128, 21.0, -20.0), (4.9e-9, 1.3e-4, 5.0, -3.0)]
    # Kerr-like polynomials: a=(a3 chi3)^2, b=2 Re(a3 eps chi3), c=|eps|^2, d=-|D/eps0|^2
    for _ in range(60):
        chi3 = 10 ** rng.uniform(-4, -1)
        a3 = float(np.float32(0.7))
        re_eps = rng.uniform(-6, 8)
        im_eps = rng.uniform(-2, 0)
        d = -(10 ** rng.uniform(-6, 2))
        coeffs.append(((a3 * chi3) ** 2, 2 * a3 * re_eps * chi3, re_eps ** 2 + im_eps ** 2, d))
    roots_re, roots_im, n_roots, cplx = [], [], [], []
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for co in coeffs:
            for as_complex in (False, True):
                args = [np.complex128(x) for x in co] if as_complex else [float(x) for x in co]
                r = np.asarray(raw_solve(*args), dtype=complex)
                pad = np.zeros(3, complex)
                pad[:len(r)] = r
                roots_re.append(pad.real)
                roots_im.append(pad.imag)
                n_roots.append(len(r))
                cplx.append(as_complex)
    co = np.repeat(np.array(coeffs, float), 2, axis=0)
    return dict(coeffs=co, roots_re=np.array(roots_re), roots_im=np.array(roots_im),
                n_roots=np.array(n_roots), complex_input=np.array(cplx))


def env_cases():
    import Environment_Setup as envDef
    import Material_Def as matDef
    out = {}
    rows_in, rows_out = [], []
    for args in [(9e9, 0.7, 7000, 8000, True), (9e9, 0.7, 7000, 8000, False),
                 (3e9, 0.5, 400, 600, False), (5e9, 0.3, 300, 900, True),
                 (1e10, 0.2, 1000, 1001, False)]:
        f, dom, lo, hi, nl = args
        with contextlib.redirect_stdout(io.StringIO()):
            r = envDef.envSetup(f, dom, lo, hi, nonLinMed=nl)
        rows_in.append(args)
        rows_out.append([float(x) for x in r])
    out["env_in"] = np.array(rows_in, float)
    out["env_out"] = np.array(rows_out, float)
    rows_in, rows_out = [], []
    for args in [(3e9, 0.5, 400, 800), (1e9, 0.5, 400, 800), (2.4e9, 1.0, 500, 900)]:
        with contextlib.redirect_stdout(io.StringIO()):
            r = matDef.matSetup(None, None, None, None, *args)
        rows_in.append(args)
        rows_out.append([float(x) for x in r])
    out["mat_in"] = np.array(rows_in, float)
    out["mat_out"] = np.array(rows_out, float)
    return out


def stab_cases():
    gstab = sys.modules["Tests.genericStability"]
    ins, outs = [], []
    for args in [(4096, 1000, 0.015, 1e9, 0.5 * 0.015 / C0, np.sqrt(2) * 2 * np.pi * 1.5e9,
                  2 * np.pi * 1.5e9, 2 * np.pi * 0.1e9),
                 (19250, 11555, 9.5172e-5, 9e9, 3.0159e-13, np.sqrt(1.5 * (2 * np.pi * 20e9) ** 2),
                  2 * np.pi * 20e9, 2 * np.pi * 20e9 * 0.1),
                 (8192, 4000, 0.015, 1e9, 0.5 * 0.015 / C0, np.sqrt(3.0) * 2 * np.pi * 0.9e9,
                  2 * np.pi * 0.9e9, 2 * np.pi * 0.1e9)]:
        with contextlib.redirect_stdout(io.StringIO()), warnings.catch_warnings():
            warnings.simplefilter("ignore")
            r = gstab.spatialStab(*args)
        ins.append(args)
        outs.append([float(np.real(x)) for x in r])
    return dict(stab_in=np.array(ins, float), stab_out=np.array(outs, float))


VARIANT_CASES = [  # (tag, Nz, materialFrontEdge, materialRearEdge)
    ("v60", 60, 20, 45), ("v200", 200, 80, 150), ("v6", 6, 1, 5), ("v8", 8, 2, 7),
    ("v10", 10, 3, 9)]


def variant_cases(mods):
    """The per-step functions no integrator calls (BaseFDTD11.py:543-607, 769-788), each run
    once on seeded arrays of Nz+1 cells.  Grids of 6-10 cells make MUR1DEx's two loops overlap.
    ADE_JxUpdate reads V.omega_0, which Variables lacks: the first call's AttributeError is
    recorded, then the attribute is set and the call repeated."""
    Variables, Params = mods["classes"][:2]
    B11 = mods["B11"]
    rng = np.random.Generator(np.random.PCG64(20261204))
    out = {}
    for tag, Nz, front, rear in VARIANT_CASES:
        P = make_params(Params, Nz=Nz, steps=16, dz=1e-3, sc=0.95, front=front, rear=rear,
                        pml=1, nzsrc=1, x1=1, x2=1, freq_in=9e9)
        V = Variables(Nz, 16, 4, 1)
        n = Nz + 1
        w0 = 2 * np.pi * rng.uniform(5e9, 20e9)
        V.omega_0E = w0
        V.plasmaFreqE = np.sqrt(rng.uniform(1.2, 3.0)) * w0
        V.gammaE = w0 * rng.uniform(0.01, 0.2)
        V.chi1Stat = rng.uniform(0.05, 0.5)
        V.chi3Stat = rng.uniform(1e-4, 1e-2)
        V.alpha3 = rng.uniform(0.3, 0.9)
        V.nonLin3gammaE = 0.0 if tag == "v60" else 2 * np.pi * rng.uniform(1e8, 1e9)
        V.nonLin3Omega_0E = 2 * np.pi * rng.uniform(1e9, 1e10)
        rec = dict(Nz=Nz, front=front, rear=rear, c0=P.c0, delT=P.delT, dz=P.dz,
                   permit_0=P.permit_0, omega_0E=V.omega_0E, plasmaFreqE=V.plasmaFreqE,
                   gammaE=V.gammaE, chi1Stat=V.chi1Stat, chi3Stat=V.chi3Stat, alpha3=V.alpha3,
                   nonLin3gammaE=V.nonLin3gammaE, nonLin3Omega_0E=V.nonLin3Omega_0E)
        # MUR1DEx
        V.Ex = rng.standard_normal(n)
        V.tempTempVarE = rng.standard_normal(n)
        rec.update(mur_Ex_in=V.Ex.copy(), mur_E2=V.tempTempVarE.copy())
        rec["mur_Ex_out"] = np.asarray(B11.MUR1DEx(V, P, None, None), float).copy()
        # ADE_JxUpdate
        scale = P.permit_0
        V.Jx = rng.standard_normal(n)
        V.polarisationCurr = scale * rng.standard_normal(n)
        V.tempVarPol = scale * rng.standard_normal(n)
        V.tempTempVarPol = scale * rng.standard_normal(n)
        rec.update(jx_in=V.Jx.copy(), jx_pc=V.polarisationCurr.copy(), jx_p1=V.tempVarPol.copy(),
                   jx_p2=V.tempTempVarPol.copy())
        try:
            B11.ADE_JxUpdate(V, P, None, None)
            rec["jx_raises"] = False
        except AttributeError:
            rec["jx_raises"] = True
        V.omega_0 = 2 * np.pi * rng.uniform(1e9, 1e10)
        rec["omega_0"] = V.omega_0
        rec["jx_out"] = np.asarray(B11.ADE_JxUpdate(V, P, None, None), float).copy()
        # Varin: Pbar3 (entered at zero: the reference stops in the debugger otherwise), then
        # J and P, then G and Q
        V.Pbar3 = np.zeros(n)
        V.Ex = rng.standard_normal(n)
        V.Qx3 = rng.standard_normal(n) ** 2
        rec.update(pbar_Ex=V.Ex.copy(), pbar_Q=V.Qx3.copy())
        rec["pbar_out"] = np.asarray(B11.ADE_NonLin_Pol_Ex_Pbar(V, P), float).copy()
        V.Jx = rng.standard_normal(n)
        V.polarisationCurr = scale * rng.standard_normal(n)
        rec.update(jp_J=V.Jx.copy(), jp_P=V.polarisationCurr.copy())
        J, Pc = B11.ADE_Lin_Curr_And_Pol_Varin(V, P)
        rec.update(jp_J_out=np.asarray(J, float).copy(), jp_P_out=np.asarray(Pc, float).copy())
        V.Gx3 = rng.standard_normal(n)
        rec.update(qg_G=V.Gx3.copy(), qg_Q=V.Qx3.copy(), qg_Ex=V.Ex.copy())
        G, Q, _ = B11.ADE_Nonlin_Q_and_G(V, P)
        rec.update(qg_G_out=np.asarray(G, float).copy(), qg_Q_out=np.asarray(Q, float).copy())
        for k, v in rec.items():
            out[f"{tag}_{k}"] = v
    return out


# arrays of Variables / CPML_Variables that the per-step functions read or write
_V_ARRAYS = ("Ex", "Hy", "Dx", "Jx", "polarisationCurr", "tempVarPol", "tempTempVarPol",
             "tempVarE", "tempTempVarE", "Acubic", "UpExMat", "UpHyMat", "UpExSelf", "UpHySelf",
             "UpExHcompsCo", "UpHyEcompsCo")
_CV_ARRAYS = ("psi_Ex", "psi_Hy", "beX", "ceX", "bmY", "cmY", "Cb", "C2", "den_Exdz",
              "den_Hydz", "kappa_Ex", "kappa_Hy", "sigma_Ex", "sigma_Hy", "alpha_Ex", "alpha_Hy",
              "eLoss_CPML", "mLoss_CPML", "Ca", "Cc", "C1", "C3")


def stepop_cases(mods):
    """The per-step functions of BaseFDTD11 that the integrators call (and the set-up chain of
    boundCondManager), and the legacy BaseFDTD module's functions: each called once on seeded
    state, recorded as ``<module>_<function>_<array>`` for every array it changed, with the
    state it started from as ``<module>_in_<array>`` (every function starts from that state)."""
    import BaseFDTD as B0
    Variables, Params, CPML_Params, CPML_Variables = mods["classes"]
    B11 = mods["B11"]
    rng = np.random.Generator(np.random.PCG64(20261205))
    out = {}
    for tag, mod in (("b11", B11), ("b0", B0)):
        P = make_params(Params, Nz=300, steps=64, dz=0.015, sc=0.5, front=100, rear=200, pml=20,
                        nzsrc=60, x1=30, x2=270, freq_in=1e9)
        P.nonLinMed, P.FreeSpace, P.TFSF = True, False, False
        P.epsRe, P.muRe = 2.0, 1.0
        P.eHcompsCo, P.eSelfCo, P.hEcompsCo, P.hSelfCo = 0.8, 0.99, 1.1, 0.98
        V = Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
        lorentz(V, 2.0, 1.5e9, 2 * np.pi * 0.1e9)
        V.chi3Stat = 1e-2
        C_P = CPML_Params(P.dz)
        C_V = CPML_Variables(P.Nz, P.timeSteps)
        with contextlib.redirect_stdout(io.StringIO()):
            mod.FieldInit(V, P)
            V.UpHyMat, V.UpExMat = mod.EmptySpaceCalc(V, P)
            if tag == "b0":
                V.epsilon, V.mu, *_ = mod.Material(V, P)
                UpHy, UpEx = mod.UpdateCoef(V, P)
                out.update(b0_UpdateCoef_UpHyMat=np.asarray(UpHy).copy(),
                           b0_UpdateCoef_UpExMat=np.asarray(UpEx).copy(),
                           b0_Material_UpExSelf=V.UpExSelf.copy(),
                           b0_Material_UpHySelf=V.UpHySelf.copy(),
                           b0_Material_UpExHcompsCo=V.UpExHcompsCo.copy(),
                           b0_Material_UpHyEcompsCo=V.UpHyEcompsCo.copy(),
                           b0_EmptySpaceCalc_UpExMat=V.UpExMat.copy(),
                           b0_EmptySpaceCalc_UpHyMat=V.UpHyMat.copy())
                Exs, Hys = mod.SmoothTurnOn(V, P)
                out.update(b0_SmoothTurnOn_Exs=np.asarray(Exs, float).copy(),
                           b0_SmoothTurnOn_Hys=np.asarray(Hys, float).copy())
            mod.CPML_FieldInit(V, P, C_V, C_P)
            # the set-up chain in boundCondManager's order, each function's arrays recorded
            for fn in ("CPML_ScalingCalc", "CPML_Ex_RC_Define", "CPML_HY_RC_Define",
                       "CPML_Ex_Update_Coef", "CPML_Hy_Update_Coef", "denominators"):
                getattr(mod, fn)(V, P, C_V, C_P)
                for a in _CV_ARRAYS:
                    out[f"{tag}_{fn}_{a}"] = np.asarray(getattr(C_V, a), float).copy()
        scal = dict(Nz=P.Nz, pmlWidth=P.pmlWidth, materialFrontEdge=P.materialFrontEdge,
                    materialRearEdge=P.materialRearEdge, nzsrc=P.nzsrc, delT=P.delT, dz=P.dz,
                    permit_0=P.permit_0, permea_0=P.permea_0, courantNo=P.courantNo,
                    CharImp=P.CharImp, freq_in=P.freq_in, c0=P.c0, epsRe=P.epsRe, muRe=P.muRe,
                    eHcompsCo=P.eHcompsCo, eSelfCo=P.eSelfCo, hEcompsCo=P.hEcompsCo,
                    hSelfCo=P.hSelfCo, kappaMax=C_P.kappaMax, sigmaOpt=C_P.sigmaOpt,
                    alphaMax=C_P.alphaMax, r_scale=C_P.r_scale, r_a_scale=C_P.r_a_scale,
                    plasmaFreqE=V.plasmaFreqE, omega_0E=V.omega_0E, gammaE=V.gammaE,
                    chi3Stat=V.chi3Stat, alpha3=V.alpha3)
        for k, v in scal.items():
            out[f"{tag}_scal_{k}"] = v
        # seeded state (fields of unit scale, Dx so that about half the slab passes the cubic's
        # |d| > 1e-8 gate), recorded as the start of every per-step call
        n = P.Nz + 1
        e0 = P.permit_0
        state = dict(Ex=rng.standard_normal(n), Hy=rng.standard_normal(n) / 377.0,
                     Dx=e0 * 1e-4 * rng.standard_normal(n) * (rng.random(n) < 0.5) +
                     e0 * 1e-5 * rng.standard_normal(n),
                     Jx=1e-3 * rng.standard_normal(n), polarisationCurr=e0 * rng.standard_normal(n),
                     tempVarPol=e0 * rng.standard_normal(n),
                     tempTempVarPol=e0 * rng.standard_normal(n),
                     tempVarE=rng.standard_normal(n), tempTempVarE=rng.standard_normal(n),
                     Acubic=1e-3 * rng.random(n), UpHySelf=1 + 0.01 * rng.standard_normal(n),
                     UpExSelf=1 + 0.01 * rng.standard_normal(n),
                     psi_Ex=1e-3 * rng.standard_normal(n), psi_Hy=1e-3 * rng.standard_normal(n))
        for k, v in state.items():
            out[f"{tag}_in_{k}"] = v.copy()
        for k in ("UpExMat", "UpHyMat", "UpExHcompsCo", "UpHyEcompsCo"):
            out[f"{tag}_in_{k}"] = np.asarray(getattr(V, k), float).copy()
        for k in _CV_ARRAYS:
            if k not in state:
                out[f"{tag}_in_{k}"] = np.asarray(getattr(C_V, k), float).copy()

        def fresh():
            for k in _V_ARRAYS:
                src = out.get(f"{tag}_in_{k}")
                if src is not None:
                    setattr(V, k, src.copy())
            for k in _CV_ARRAYS:
                src = out.get(f"{tag}_in_{k}")
                if src is not None:
                    setattr(C_V, k, src.copy())

        if tag == "b11":
            calls = [("ADE_ExUpdate", lambda: mod.ADE_ExUpdate(V, P, C_V, C_P, 0)),
                     ("CPML_Psi_e_Update", lambda: mod.CPML_Psi_e_Update(V, P, C_V, C_P)),
                     ("CPML_Psi_m_Update", lambda: mod.CPML_Psi_m_Update(V, P, C_V, C_P)),
                     ("ADE_DxUpdate", lambda: mod.ADE_DxUpdate(V, P, C_V, C_P)),
                     ("AcubicFinder", lambda: mod.AcubicFinder(V, P)),
                     ("NonLinExUpdate", lambda: mod.NonLinExUpdate(V, P)),
                     ("ADE_HyUpdate", lambda: mod.ADE_HyUpdate(V, P, C_V, C_P)),
                     ("ADE_PolarisationCurrent_Ex",
                      lambda: mod.ADE_PolarisationCurrent_Ex(V, P, C_V, C_P, 0)),
                     ("ADE_ExCreate", lambda: mod.ADE_ExCreate(V, P, C_V, C_P)),
                     ("ADE_TempPolCurr", lambda: mod.ADE_TempPolCurr(V, P, C_V, C_P))]
        else:
            calls = [("CPML_Psi_e_Update", lambda: mod.CPML_Psi_e_Update(V, P, C_V, C_P)),
                     ("CPML_Psi_m_Update", lambda: mod.CPML_Psi_m_Update(V, P, C_V, C_P)),
                     ("CPML_HyUpdate", lambda: mod.CPML_HyUpdate(V, P, C_V, C_P)),
                     ("CPML_ExUpdate", lambda: mod.CPML_ExUpdate(V, P, C_V, C_P)),
                     ("ADE_TempPolCurr", lambda: mod.ADE_TempPolCurr(V, P)),
                     ("ADE_PolarisationCurrent_Ex",
                      lambda: mod.ADE_PolarisationCurrent_Ex(V, P, C_V, C_P)),
                     ("ADE_HyUpdate", lambda: mod.ADE_HyUpdate(V, P, C_V, C_P)),
                     ("ADE_ExUpdate", lambda: mod.ADE_ExUpdate(V, P, C_V, C_P)),
                     ("ADE_ExCreate", lambda: mod.ADE_ExCreate(V, P, C_V, C_P)),
                     ("ADE_DxUpdate", lambda: mod.ADE_DxUpdate(V, P, C_V, C_P))]
        for fn, call in calls:
            fresh()
            with contextlib.redirect_stdout(io.StringIO()), warnings.catch_warnings():
                warnings.simplefilter("ignore")
                call()
            for k in _V_ARRAYS:
                a = np.asarray(getattr(V, k), float)
                src = out.get(f"{tag}_in_{k}")
                if src is not None and not np.array_equal(a, src):
                    out[f"{tag}_{fn}_{k}"] = a.copy()
            for k in _CV_ARRAYS:
                a = np.asarray(getattr(C_V, k), float)
                src = out.get(f"{tag}_in_{k}")
                if src is not None and not np.array_equal(a, src):
                    out[f"{tag}_{fn}_{k}"] = a.copy()
            if fn == "AcubicFinder":
                out["b11_AcubicFinder_cubPoly"] = np.asarray(V.cubPoly).copy()
    return out


def _no_debugger(*args, **kwargs):
    raise RuntimeError("the reference reached breakpoint() (a state its checks stop on)")


def time_reference(mods, n_steps=1024):
    """Wall time of the reference's own IntegratorNL1D (plain Python here) on the 1000-cell Kerr
    workload; prints its Mcell-steps/s (the CPU form of the reference's path)."""
    import time
    Params = mods["classes"][1]
    P = make_params(Params, Nz=1000, steps=n_steps, dz=0.015, sc=0.5, front=400, rear=600,
                    pml=20, nzsrc=100, x1=50, x2=950, freq_in=1e9)
    P.nonLinMed, P.FreeSpace, P.TFSF = True, False, False
    src = gauss_sine(P.timeSteps, 1e9, P.delT)

    def cfg0(V):
        lorentz(V, 2.0, 1.5e9, 2 * np.pi * 0.1e9)
        V.chi3Stat = 1e-2

    t0 = time.perf_counter()
    run_case(mods, "IntegratorNL1D", P, cfg0, source=(src, np.zeros_like(src)),
             keep_history=False)
    t = time.perf_counter() - t0
    print(f"reference IntegratorNL1D, Nz=1000, {n_steps} steps: {t:.2f} s, "
          f"{1001 * n_steps / t / 1e6:.3f} Mcell-steps/s")


def main(only=None):
    if not REF or not os.path.isdir(REF):
        sys.exit("set PYFDTD_REFERENCE to the reference checkout (fraserac/Py-FDTD_PIC)")
    sys.breakpointhook = _no_debugger
    raw_solve = _install_stubs()
    import BaseFDTD11 as B11
    import Solver_Engine as SE
    mods = dict(classes=_load_state_classes(), SE=SE, B11=B11)
    if only == "time":
        time_reference(mods)
        return
    Variables, Params, CPML_Params, CPML_Variables = mods["classes"]
    meta = dict(numpy=np.__version__, scipy=scipy.__version__,
                eps0=scipy.constants.epsilon_0, mu0=scipy.constants.mu_0)

    if only == "stepops" or only is None:
        np.savez_compressed(os.path.join(OUT, "stepops.npz"), **stepop_cases(mods), **meta)
        print("stepops done", flush=True)
        if only == "stepops":
            return
    if only == "variants" or only is None:
        np.savez_compressed(os.path.join(OUT, "variants.npz"), **variant_cases(mods), **meta)
        print("variants done", flush=True)
        if only == "variants":
            return
    np.savez_compressed(os.path.join(OUT, "cubic_solve.npz"), **cubic_cases(raw_solve), **meta)
    np.savez_compressed(os.path.join(OUT, "setup.npz"), **env_cases(), **stab_cases(), **meta)

    # 1) the 1000-cell Kerr workload: Nz=1000, dz=15 mm, Sc=0.5, 4096 steps, slab 400-599,
    #    Lorentz eps (d_eps=2, f0=1.5 GHz, gamma=2 pi 0.1 GHz) entering the cubic, chi3=1e-2,
    #    soft Gaussian-modulated 1 GHz source at cell 100, PML 20, extra probes at 50 and 950.
    def cfg0(V):
        lorentz(V, 2.0, 1.5e9, 2 * np.pi * 0.1e9)
        V.chi3Stat = 1e-2

    dz, sc, f = 0.015, 0.5, 1e9
    P = make_params(Params, Nz=1000, steps=4096, dz=dz, sc=sc, front=400, rear=600, pml=20,
                    nzsrc=100, x1=50, x2=950, freq_in=f)
    P.nonLinMed, P.FreeSpace, P.TFSF = True, False, False
    src = gauss_sine(P.timeSteps, f, P.delT)
    r = run_case(mods, "IntegratorNL1D", P, cfg0, source=(src, np.zeros_like(src)),
                 extra_probes=(50, 950), keep_history=False)
    np.savez_compressed(os.path.join(OUT, "kerr_nz1000.npz"), **r, **meta)
    print("kerr_nz1000 done", flush=True)

    # 2) the same grid in the Lorentz (two-pass) integrator, probes x1Loc=50, x2Loc=950
    P = make_params(Params, Nz=1000, steps=4096, dz=dz, sc=sc, front=400, rear=600, pml=20,
                    nzsrc=100, x1=50, x2=950, freq_in=f)
    P.LorentzMed, P.FreeSpace, P.TFSF = True, False, False
    r = run_case(mods, "IntegratorLinLor1D", P, cfg0, source=(src, np.zeros_like(src)),
                 keep_history=False)
    np.savez_compressed(os.path.join(OUT, "lorentz_nz1000.npz"), **r, **meta)
    print("lorentz_nz1000 done", flush=True)

    # 3) the reference's own source path: SineCont with the 0.8 f pump and TF/SF, Kerr slab,
    #    Sc=0.95 (float32), small grid
    P = make_params(Params, Nz=600, steps=900, dz=1e-3, sc=0.95, front=300, rear=480, pml=40,
                    nzsrc=150, x1=280, x2=60, freq_in=9e9)
    P.nonLinMed, P.FreeSpace, P.TFSF, P.SineCont, P.Periods = True, False, True, True, 1000

    def nl_default(V):
        V.chi3Stat = 1e-3

    r = run_case(mods, "IntegratorNL1D", P, nl_default)
    np.savez_compressed(os.path.join(OUT, "kerr_sinecont_tfsf.npz"), **r, **meta)
    print("kerr_sinecont_tfsf done", flush=True)

    # 4) Lorentz two-pass with SineCont + TF/SF (the reference's sweep setting), small grid
    P = make_params(Params, Nz=500, steps=700, dz=1e-3, sc=0.95, front=260, rear=499, pml=30,
                    nzsrc=120, x1=240, x2=60, freq_in=9e9)
    P.LorentzMed, P.FreeSpace, P.TFSF, P.SineCont, P.Periods = True, False, True, True, 1000
    r = run_case(mods, "IntegratorLinLor1D", P, lambda V: None)
    np.savez_compressed(os.path.join(OUT, "lorentz_sinecont_tfsf.npz"), **r, **meta)
    print("lorentz_sinecont_tfsf done", flush=True)

    # 5) free space (two passes, sech-modulated Gaussian source with TF/SF)
    P = make_params(Params, Nz=400, steps=600, dz=1e-3, sc=0.95, front=250, rear=330, pml=25,
                    nzsrc=100, x1=230, x2=50, freq_in=9e9)
    P.FreeSpace, P.TFSF, P.Gaussian = True, True, True
    r = run_case(mods, "IntegratorFreeSpace1D", P, lambda V: None)
    np.savez_compressed(os.path.join(OUT, "freespace_gauss_tfsf.npz"), **r, **meta)
    print("freespace_gauss_tfsf done", flush=True)

    # 6) CPML set-up with a stretched kappa (kappaMax=3) so the den_Exdz/den_Hydz index walk
    #    (BaseFDTD11.py:333-357) is visible; Kerr integrator, short run
    P = make_params(Params, Nz=300, steps=200, dz=1e-3, sc=0.95, front=150, rear=220, pml=16,
                    nzsrc=60, x1=140, x2=30, freq_in=9e9)
    P.nonLinMed, P.FreeSpace, P.TFSF, P.SineCont = True, False, True, True
    orig = CPML_Params.__init__

    def kappa3(self, dz_):
        orig(self, dz_)
        self.kappaMax = 3
        self.alphaMax = 0.02

    CPML_Params.__init__ = kappa3
    try:
        r = run_case(mods, "IntegratorNL1D", P, nl_default)
    finally:
        CPML_Params.__init__ = orig
    np.savez_compressed(os.path.join(OUT, "kerr_kappa3.npz"), **r, **meta)
    print("kerr_kappa3 done", flush=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
