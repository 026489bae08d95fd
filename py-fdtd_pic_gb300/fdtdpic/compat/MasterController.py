"""State classes, ``Controller``, ``results`` and ``LoopedSim`` of MasterController.py.

The four state classes keep the reference's constructor signatures, members and defaults
(MasterController.py:82-440), including the scalar members' declared types (float32 members
such as ``courantNo``, ``alpha3``, ``kappaMax`` and ``alphaMax`` hold float32-rounded values).
``Controller`` dispatches to the GPU integrators of :mod:`Solver_Engine` exactly as the
reference does (:451-469).  ``LoopedSim(loop=True)`` prepares its 20 frequency points in the
reference's order on the host, then steps all of them in one batched GPU launch.

Not carried over: plotting (``plotter``, the figures inside ``RefTester``), the report
template and ``VideoMaker``; ``LoopedSim`` returns its data instead of plotting it.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.constants as _const

from . import BaseFDTD11
from . import Environment_Setup as envDef
from . import Solver_Engine as SE
from . import TransformHandler as transH
from ._typed import typed


class Reporter:
    """Collects named timings/values (MasterController.py:57-78)."""

    def __init__(self):
        self.dict1 = {"": ""}

    def printer(self, item="", name="", show=False):
        self.dict1[name] = item
        if show:
            print(item)


_V_TYPES = dict(Nz="i32", timeSteps="f32", plasmaFreqE="f64", gammaE="f64", omega_0E="f64",
                test="i32", tempTempTest="i32", attenAmnt="i32", alpha3="f32",
                nonLin3gammaE="f64", nonLin3Omega_0E="f64", chi1Stat="f64", chi3Stat="f64")


@typed(_V_TYPES)
class Variables:
    """Fields, probes and material constants that change during a run (:146-214)."""

    def __init__(self, Nz, timeSteps, interval, attenAmnt):
        n = Nz + 1
        rows = int(timeSteps / interval)
        for name in ("UpHyMat", "UpExMat", "UpExHcompsCo", "UpExSelf", "UpHySelf",
                     "UpHyEcompsCo", "epsilon", "mu"):
            setattr(self, name, np.ones(n))
        for name in ("Ex", "Hy", "Dx", "Jx", "polarisationCurr", "tempVarPol", "tempTempVarPol",
                     "tempVarE", "tempTempVarE", "tempVarHy", "tempTempVarHy", "tempVarJx",
                     "tempTempVarJx", "tempVarDx", "tempTempVarDx", "tempTest", "Gx3", "Qx3",
                     "Pbar3", "JxKerr", "JxRaman", "Acubic"):
            setattr(self, name, np.zeros(n))
        for name in ("Ex_History", "Hy_History", "Jx_History", "polCurr_History", "Dx_History",
                     "Psi_e_History"):
            setattr(self, name, np.zeros((rows, n)))
        for name in ("x1ColBe", "x1ColAf", "x1Jx", "x1Hy", "x1ExOld", "x1JxOld", "x1HyOld",
                     "Port1", "Port2"):
            setattr(self, name, np.zeros(timeSteps))
        self.plasmaFreqE = np.sqrt((1.5) * (2 * np.pi * 20e9) ** 2)
        self.gammaE = 2 * np.pi * 20e9 * 0.1
        self.omega_0E = 2 * np.pi * 20e9
        self.test = 5
        self.tempTempTest = 0
        self.attenAmnt = attenAmnt
        self.x1Atten = np.zeros((attenAmnt, timeSteps))
        self.alpha3 = 0.7
        self.nonLin3gammaE = 0
        self.nonLin3Omega_0E = 6e9
        self.chi1Stat = np.sqrt(1.2) - 1
        self.chi3Stat = 1e-3
        self.cubPoly = np.zeros((n, 4), dtype=np.complex128)
        self.roots = np.zeros(4, dtype=np.complex128)

    def __str__(self):
        return "Contains data that will change during sim"


# The reference's spec lists declare some members twice; the later declaration is the one
# that holds (timeSteps int32, period/eLoss/... float64, lamMin float64).
_P_TYPES = dict(
    Nz="i32", timeSteps="i32", eLoss="f64", mLoss="f64", eSelfCo="f64", eHcompsCo="f64",
    hSelfCo="f64", hEcompsCo="f64", x1Loc="i32", x2Loc="i32", materialFrontEdge="i32",
    materialRearEdge="i32", pmlWidth="i32", nzsrc="i32", lamMin="f64", dz="f64", delT="f64",
    courantNo="f32", period="f64", domainSize="i32", freq_in="f64", permit_0="f64",
    permea_0="f64", CharImp="f64", c0="f64", Nlam="f64", MORmode="bool", delayMOR="i32",
    CPMLXp="bool", CPMLXm="bool", TFSF="bool", SineCont="bool", Gaussian="bool", Ricker="bool",
    Amplitude="f32", Periods="f32", LorentzMed="bool", nonLinMed="bool", FreeSpace="bool",
    epsRe="f32", muRe="f32", vidMake="bool", vidInterval="i32", atten="bool", julia="bool",
    testMode="bool")


@typed(_P_TYPES)
class Params:
    """Run constants (:288-339); positional arguments as envSetup's 20-tuple plus MORmode,
    domainSize, freq_in, delayMOR."""

    def __init__(self, Nz, timeSteps, eLoss, mLoss, eSelfCo, eHcompsCo, hSelfCo, hEcompsCo,
                 x1Loc, x2Loc, materialFrontEdge, materialRearEdge, pmlWidth, nzsrc, lamMin, dz,
                 delT, courantNo, period, Nlam, MORmode, domainSize, freq_in, delayMOR,
                 LorentzMed=False, nonLinMed=False, SineCont=False, Gaussian=False, TFSF=False):
        self.permit_0 = _const.epsilon_0
        self.permea_0 = _const.mu_0
        self.CharImp = 376.730313668
        self.c0 = 299792458.0
        self.freq_in = freq_in
        self.lamMin = lamMin
        self.Nlam = Nlam
        self.dz = dz
        self.delT = delT
        self.courantNo = courantNo
        self.materialFrontEdge = materialFrontEdge
        self.materialRearEdge = materialRearEdge
        self.Nz = Nz
        self.timeSteps = timeSteps
        self.x1Loc = x1Loc
        self.x2Loc = x2Loc
        self.nzsrc = nzsrc
        self.period = period
        self.eLoss = eLoss
        self.eSelfCo = eSelfCo
        self.eHcompsCo = eHcompsCo
        self.mLoss = mLoss
        self.hSelfCo = hSelfCo
        self.hEcompsCo = hEcompsCo
        self.pmlWidth = pmlWidth
        self.domainSize = domainSize
        self.MORmode = MORmode
        self.delayMOR = delayMOR
        self.CPMLXp = True
        self.CPMLXm = True
        self.TFSF = TFSF
        self.SineCont = SineCont
        self.Gaussian = Gaussian
        self.Ricker = False
        self.Amplitude = 1.0
        self.Periods = 1.0
        self.LorentzMed = LorentzMed
        self.nonLinMed = nonLinMed
        self.FreeSpace = True
        self.epsRe = 1.0
        self.muRe = 1.0
        self.vidMake = True
        self.vidInterval = 50
        self.atten = False
        self.julia = False
        self.testMode = False

    def __str__(self):
        return "Class containing all values that remain constant throughout a sim"


@typed(dict(kappaMax="f32", r_scale="f32", r_a_scale="f32", sigmaEMax="f64", sigmaHMax="f64",
            sigmaOpt="f64", alphaMax="f32"))
class CPML_Params:
    """CPML grading constants (:351-366)."""

    def __init__(self, dz):
        self.kappaMax = 1
        self.r_scale = 4
        self.r_a_scale = 1
        self.sigmaEMax = 0.5 * (0.8 * (1) / (dz * (_const.mu_0 / _const.epsilon_0) ** 0.5))
        self.sigmaHMax = self.sigmaEMax
        self.sigmaOpt = self.sigmaEMax
        self.alphaMax = 0.05

    def __repr__(self):
        return f"{self.__class__.__name__}"

    def __str__(self):
        return "Class containing all CPML values that remain constant throughout a sim"


@typed(dict(Nz="i32"))
class CPML_Variables:
    """CPML profiles, coefficients and auxiliary fields (:402-440)."""

    def __init__(self, Nz, timeSteps):
        n = Nz + 1
        self.kappa_Ex = np.zeros(n)
        self.kappa_Hy = np.zeros(n)
        self.psi_Ex = np.zeros(n)
        self.psi_Ex_Probe = np.zeros(timeSteps)
        self.psi_Hy = np.zeros(n)
        self.psi_Hy_Probe = np.zeros(timeSteps)
        for name in ("alpha_Ex", "alpha_Hy", "sigma_Ex", "sigma_Hy", "beX", "bmY", "ceX", "cmY",
                     "Ca", "Cb", "Cc", "C1", "C2", "C3", "eLoss_CPML", "mLoss_CPML", "den_Hydz",
                     "den_Exdz", "tempTempVarPsiEx", "tempVarPsiEx", "tempTempVarPsiHy",
                     "tempVarPsiHy"):
            setattr(self, name, np.zeros(n))
        self.psi_Ex_Old = np.zeros(timeSteps)
        self.psi_Hy_Old = np.zeros(timeSteps)

    def __repr__(self):
        return f"{self.__class__.__name__}"

    def __str__(self):
        return "Class containing all CPML values that vary throughout a sim"


def _windows(P):
    return int(P.timeSteps * 0.7), int(P.timeSteps * 0.05)


def Controller(V, P, C_V, C_P):
    """Run the integrator P selects (LorentzMed, then FreeSpace, then nonLinMed) on the GPU;
    returns (V, P, C_V, C_P, Exs, Hys) as the reference's Controller (:451-469)."""
    fin_be, st_af = _windows(P)
    V.x1ColBe = np.zeros(P.timeSteps)
    V.x1ColAf = np.zeros(P.timeSteps)
    out = None
    if P.LorentzMed:
        out = SE.IntegratorLinLor1D(V, P, C_V, C_P, fin_be, st_af)
    elif P.FreeSpace:
        out = SE.IntegratorFreeSpace1D(V, P, C_V, C_P, fin_be, st_af)
    elif P.nonLinMed:
        out = SE.IntegratorNL1D(V, P, C_V, C_P, fin_be, st_af)
    if out is None:
        # the reference reaches its return with Exs unbound
        raise UnboundLocalError("Controller: no integrator selected (LorentzMed, FreeSpace and "
                                "nonLinMed are all False)")
    V.Ex, V.Hy, Exs, Hys, C_V.psi_Ex, C_V.psi_Hy, V.x1ColBe, V.x1ColAf = out
    return V, P, C_V, C_P, Exs, Hys


def Controller_batch(runs):
    """Controller for many (V, P, C_V, C_P) at once: host set-up of each run in order, then
    one batched GPU launch for all of them.  Returns a list of (V, P, C_V, C_P, Exs, Hys)."""
    jobs = []
    for V, P, C_V, C_P in runs:
        fin_be, st_af = _windows(P)
        V.x1ColBe = np.zeros(P.timeSteps)
        V.x1ColAf = np.zeros(P.timeSteps)
        jobs.append(SE.prepare(_integrator_name(P), V, P, C_V, C_P, fin_be, st_af))
    SE.run_prepared(jobs)
    out = []
    for (V, P, C_V, C_P), job in zip(runs, jobs):
        r = SE.finish_prepared(job)
        V.Ex, V.Hy, Exs, Hys, C_V.psi_Ex, C_V.psi_Hy, V.x1ColBe, V.x1ColAf = r
        out.append((V, P, C_V, C_P, Exs, Hys))
    return out


def results(V, P, C_V, C_P, time_Vec, RefCo=False, FFT=False, AnalRefCo=False,
            attenRead=False):
    """Reflection measures of a finished run (:472-505): RefCo -> peak-bin spectral ratio of
    x1ColAf to x1ColBe (spectra on the GPU); AnalRefCo -> Fresnel reflection of the slab."""
    if attenRead:
        _, _, val = transH.RefTester(V, P, V.x1ColBe, 1)
        att = np.zeros(len(V.x1Atten))
        for i in range(len(V.x1Atten)):
            att[i] = transH.RefTester(V, P, V.x1Atten[i], 1, mul=True) / val
        return att
    if RefCo:
        _, _, val = transH.RefTester(V, P, V.x1ColBe, 1)
        _, _, val2 = transH.RefTester(V, P, V.x1ColAf, 1)
        return val2 / val
    if AnalRefCo:
        return BaseFDTD11.AnalyticalReflectionE(V, P)
    return "results ran to end"


def _integrator_name(P):
    if P.LorentzMed:
        return "IntegratorLinLor1D"
    if P.FreeSpace:
        return "IntegratorFreeSpace1D"
    if P.nonLinMed:
        return "IntegratorNL1D"
    raise UnboundLocalError("Controller: no integrator selected")


def LoopedSim(Rep, V, P, C_V, C_P, MORmode, domainSize, lowLimTim, highLimTim,
              stringparamSweep="Input frequency sweep", loop=False, Low=3e9, Interval=1e8,
              RefCoBool=True):
    """Frequency sweep (:530-600).

    loop=True: 20 points.  Each point is set up on the host in the reference's order --
    envSetup sees the previous point's V (whose plasmaFreqE its integrator rescaled) and P
    (whose freq_in was then advanced by Interval) -- and the analytical reflection is taken
    before freq_in advances, as the reference takes it.  The 20 runs are then stepped in ONE
    batched GPU launch and their measured reflections taken from the probe traces.
    Returns (dataRange, measured R, analytical R) in place of the reference's plot.

    loop=False: one Controller run; returns (V, P, C_V, C_P, measured R, analytical R), the
    reflections only for the Lorentz integrator (as the reference prints them)."""
    if loop:
        points = 20
        dataRange = np.arange(Low, points * Interval + Low, Interval)
        ref = np.zeros(points)
        anal = np.zeros(points)
        if stringparamSweep != "Input frequency sweep":
            return dataRange, ref, anal
        states, jobs = [], []
        for i in range(points):
            setup = envDef.envSetup(P.freq_in, domainSize, lowLimTim, highLimTim, VExists=True,
                                    V=V, P=P)
            P = Params(*setup, P.MORmode, domainSize, P.freq_in, 20, LorentzMed=P.LorentzMed,
                       SineCont=P.SineCont, Gaussian=P.Gaussian, TFSF=P.TFSF)
            V = Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
            C_P = CPML_Params(P.dz)
            C_V = CPML_Variables(P.Nz, P.timeSteps)
            fin_be, st_af = _windows(P)
            V.x1ColBe = np.zeros(P.timeSteps)
            V.x1ColAf = np.zeros(P.timeSteps)
            jobs.append(SE.prepare(_integrator_name(P), V, P, C_V, C_P, fin_be, st_af))
            states.append((V, P, C_V, C_P))
            anal[i] = results(V, P, C_V, C_P, None, AnalRefCo=True)
            P.freq_in = P.freq_in + Interval
        SE.run_prepared(jobs)
        for i, ((V_i, P_i, C_V_i, C_P_i), job) in enumerate(zip(states, jobs)):
            r = SE.finish_prepared(job)
            V_i.Ex, V_i.Hy, _, _, C_V_i.psi_Ex, C_V_i.psi_Hy, V_i.x1ColBe, V_i.x1ColAf = r
            t = np.arange(0, len(V_i.x1ColBe)) * P_i.delT
            ref[i] = results(V_i, P_i, C_V_i, C_P_i, t, RefCo=True)
        return dataRange, ref, anal
    tic = time.perf_counter()
    toc = time.perf_counter()
    if Rep is not None:
        Rep.printer(str(toc - tic), "matSetupTime")
    V, P, C_V, C_P, Exs, Hys = Controller(V, P, C_V, C_P)
    t = np.arange(0, len(V.x1ColBe)) * P.delT
    ref = np.zeros(1)
    anal = np.zeros(1)
    if not P.FreeSpace and P.LorentzMed:
        ref[0] = results(V, P, C_V, C_P, t, RefCo=True)
        anal[0] = results(V, P, C_V, C_P, t, AnalRefCo=True)
    return V, P, C_V, C_P, ref, anal
