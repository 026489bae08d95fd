"""CPU oracle for the 1D FDTD/PIC hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this
module, and only as the checker.  The product (``py-fdtd_pic_gb300``) never imports it.

It restates, in numpy, the reference's one-off set-up path and drives the FP64 C stepping loop in
``fdtd_oracle.c`` (built here with gcc, ``-O2 -ffp-contract=off``):

* ``EmptySpaceCalc`` / ``Material`` / ``UpdateCoef``      BaseFDTD11.py:124-182
* ``CPML_FieldInit`` ... ``denominators``                BaseFDTD11.py:196-357 (the Hy arrays alias
  the Ex arrays, ``Cb``/``C2`` stay 0 at index Nz+1-pml, ``den_*dz`` use the reference's index walk)
* ``spatialStab``                                         genericStability.py:12-62
* ``SmoothTurnOn`` / ``Gaussian`` / ``SourceManager`` / ``Sig_Mod``
                                                          BaseFDTD11.py:86-120, Solver_Engine.py:89-140
* ``IntegratorNL1D`` / ``IntegratorLinLor1D`` / ``IntegratorFreeSpace1D``
                                                          Solver_Engine.py:142-371
* ``envSetup`` / ``matSetup``                             Environment_Setup.py:19-166, Material_Def.py:21-120
* the uncalled per-step variants ``MUR1DEx``, ``ADE_JxUpdate``, ``ADE_NonLin_Pol_Ex_Pbar``,
  ``ADE_Lin_Curr_And_Pol_Varin``, ``ADE_Nonlin_Q_and_G``  BaseFDTD11.py:543-607, 769-788

Scalars the reference stores in float32 jitclass fields (``courantNo``, ``alpha3``, ``kappaMax``,
``r_scale``, ``r_a_scale``, ``alphaMax``, ``epsRe``, ``muRe``, ``Amplitude``, ``Periods``;
MasterController.py:129,234-279,341-347) are rounded with :func:`f32` by whoever builds the
parameter set (``jitclass_f32_casts=False`` in :func:`reference_params` skips the rounding).

Parity is pinned: ``tests/golden/*.npz`` are outputs of the reference's own integrators
(``tests/golden/make_golden.py``), and the oracle reproduces them to ~1e-14 relative L2.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import sys
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libfdtd_oracle.so")

FREESPACE, LINLOR, KERR = 0, 1, 2
C0 = 299792458.0
CHAR_IMP = 376.730313668


def f32(x: float) -> float:
    """Round to float32 and back, as a float32 jitclass field does."""
    return float(np.float32(x))


# -------------------------------------------------------------------------------------------
# build + load
# -------------------------------------------------------------------------------------------
def build(force: bool = False) -> str:
    src = os.path.join(HERE, "fdtd_oracle.c")
    srcs = [src, os.path.join(HERE, "pic_oracle.c")]
    srcs = [s for s in srcs if os.path.exists(s)]
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", tmp] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        d, i = ctypes.c_double, ctypes.c_int
        P = ctypes.c_void_p
        _lib.or_cubic_root0.restype = d
        _lib.or_cubic_root0.argtypes = [d, d, d, d]
        _lib.or_cubic_solve.restype = None
        _lib.or_cubic_solve.argtypes = [d, d, d, d, P, P, P]
        _lib.or_run_pass.restype = i
        _lib.or_run_pass.argtypes = ([i] * 13 + [P, P, P, P, P, d] + [P] * 9 + [i, P, i, i, P]
                                     + [i, i, P])
        _lib.or_pic_step.restype = i
        _lib.or_pic_step.argtypes = [i, P, P, P, P, P, P, P, P, P, i, P, i]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# -------------------------------------------------------------------------------------------
# cubic
# -------------------------------------------------------------------------------------------
def cubic_solve(a, b, c, d):
    """All roots of CubicEquationSolver.solve for real coefficients (C restatement)."""
    re = np.zeros(3)
    im = np.zeros(3)
    n = ctypes.c_int()
    lib().or_cubic_solve(a, b, c, d, _p(re), _p(im), ctypes.byref(n))
    return (re + 1j * im)[: n.value]


def cubic_solve_py(a, b, c, d):
    """Pure-Python restatement of CubicEquationSolver.solve (CubicEquationSolver.py:29-90)."""
    if a == 0 and b == 0:
        return np.array([(-d * 1.0) / c])
    if a == 0:
        D = c * c - 4.0 * b * d
        if D >= 0:
            D = math.sqrt(D)
            return np.array([(-c + D) / (2.0 * b), (-c - D) / (2.0 * b)])
        D = math.sqrt(-D)
        return np.array([(-c + D * 1j) / (2.0 * b), (-c - D * 1j) / (2.0 * b)])
    f = ((3.0 * c / a) - ((b ** 2.0) / (a ** 2.0))) / 3.0
    g = (((2.0 * (b ** 3.0)) / (a ** 3.0)) - ((9.0 * b * c) / (a ** 2.0)) + (27.0 * d / a)) / 27.0
    h = (g ** 2.0) / 4.0 + (f ** 3.0) / 27.0
    if f == 0 and g == 0 and h == 0:
        x = (d / (1.0 * a)) ** (1 / 3.0) * -1 if (d / a) >= 0 else (-d / (1.0 * a)) ** (1 / 3.0)
        return np.array([x, x, x])
    if h <= 0:
        i = math.sqrt(((g ** 2.0) / 4.0) - h)
        j = i ** (1 / 3.0)
        k = math.acos(-(g / (2 * i)))
        L = j * -1
        M = math.cos(k / 3.0)
        N = math.sqrt(3) * math.sin(k / 3.0)
        P = (b / (3.0 * a)) * -1
        return np.array([2 * j * math.cos(k / 3.0) - (b / (3.0 * a)), L * (M + N) + P,
                         L * (M - N) + P])
    R = -(g / 2.0) + math.sqrt(h)
    S = R ** (1 / 3.0) if R >= 0 else (-R) ** (1 / 3.0) * -1
    T = -(g / 2.0) - math.sqrt(h)
    U = T ** (1 / 3.0) if T >= 0 else (-T) ** (1 / 3.0) * -1
    x1 = (S + U) - (b / (3.0 * a))
    x2 = -(S + U) / 2 - (b / (3.0 * a)) + (S - U) * math.sqrt(3) * 0.5j
    x3 = -(S + U) / 2 - (b / (3.0 * a)) - (S - U) * math.sqrt(3) * 0.5j
    return np.array([x1, x2, x3])


# -------------------------------------------------------------------------------------------
# parameter set (attribute names of the reference's Params / Variables / CPML_Params)
# -------------------------------------------------------------------------------------------
@dataclass
class RefParams:
    Nz: int
    timeSteps: int
    dz: float
    delT: float
    courantNo: float
    materialFrontEdge: int
    materialRearEdge: int
    pmlWidth: int
    nzsrc: int
    x1Loc: int = 0
    x2Loc: int = 0
    freq_in: float = 1e9
    permit_0: float = 8.8541878188e-12
    permea_0: float = 1.25663706127e-06
    CharImp: float = CHAR_IMP
    c0: float = C0
    TFSF: bool = False
    SineCont: bool = False
    Gaussian: bool = False
    nonLinMed: bool = False
    LorentzMed: bool = False
    FreeSpace: bool = True
    CPMLXp: bool = True
    CPMLXm: bool = True
    vidInterval: int = 50
    period: float = 1e-9
    Periods: float = 1.0
    Amplitude: float = 1.0
    epsRe: float = 1.0
    muRe: float = 1.0
    # Variables
    plasmaFreqE: float = math.sqrt(1.5 * (2 * math.pi * 20e9) ** 2)
    gammaE: float = 2 * math.pi * 20e9 * 0.1
    omega_0E: float = 2 * math.pi * 20e9
    chi3Stat: float = 1e-3
    alpha3: float = f32(0.7)
    # CPML_Params
    kappaMax: float = 1.0
    r_scale: float = 4.0
    r_a_scale: float = 1.0
    sigmaOpt: float = 0.0
    alphaMax: float = f32(0.05)


def params_from_golden(g) -> RefParams:
    """Parameter set of a golden fixture (tests/golden/*.npz)."""
    kw = {}
    for k in RefParams.__dataclass_fields__:
        if f"P_{k}" in g:
            v = g[f"P_{k}"][()]
            kw[k] = v.item() if hasattr(v, "item") else v
    kw.update(plasmaFreqE=float(g["plasmaFreqE_in"]), gammaE=float(g["gammaE"]),
              omega_0E=float(g["omega_0E"]), chi3Stat=float(g["chi3Stat"]),
              alpha3=float(g["alpha3"]), kappaMax=float(g["kappaMax"]),
              r_scale=float(g["r_scale"]), r_a_scale=float(g["r_a_scale"]),
              sigmaOpt=float(g["sigmaOpt"]), alphaMax=float(g["alphaMax"]))
    for b in ("TFSF", "SineCont", "Gaussian", "nonLinMed", "LorentzMed", "CPMLXp", "CPMLXm"):
        kw[b] = bool(kw.get(b, False))
    for i in ("Nz", "timeSteps", "materialFrontEdge", "materialRearEdge", "pmlWidth", "nzsrc",
              "x1Loc", "x2Loc", "vidInterval"):
        kw[i] = int(kw[i])
    kw["FreeSpace"] = not (kw["nonLinMed"] or kw["LorentzMed"])
    return RefParams(**kw)


def sigma_opt(dz, eps0, mu0):
    """CPML_Params.sigmaEMax/sigmaOpt (MasterController.py:356-358)."""
    return 0.5 * (0.8 * (1) / (dz * (mu0 / eps0) ** 0.5))


# -------------------------------------------------------------------------------------------
# set-up restatement
# -------------------------------------------------------------------------------------------
def empty_space(P: RefParams):
    """EmptySpaceCalc (BaseFDTD11.py:124-132): UpHyMat, UpExMat."""
    n = P.Nz + 1
    upHy = np.ones(n) * ((1 / P.CharImp) * P.courantNo)
    upEx = np.ones(n) * (P.CharImp * P.courantNo)
    return upHy, upEx


def material_update_coef(P: RefParams):
    """Material + UpdateCoef (BaseFDTD11.py:136-182): the free-space integrator's coefficients."""
    eps = np.ones(P.Nz)
    mu = np.ones(P.Nz)
    eps[P.materialFrontEdge:P.materialRearEdge] = P.epsRe
    mu[P.materialFrontEdge:P.materialRearEdge] = P.muRe
    upHy = np.ones(P.Nz + 1) * ((1 / P.CharImp) * P.courantNo)
    upEx = np.ones(P.Nz + 1) * (P.CharImp * P.courantNo)
    for k in range(P.materialFrontEdge, P.materialRearEdge):
        upEx[k] = upEx[k] / eps[k]
        upHy[k] = upHy[k] / mu[k]
    return upHy, upEx


def cpml_coefficients(P: RefParams, upEx, upExH=None):
    """boundCondManager's chain (Solver_Engine.py:70-87; BaseFDTD11.py:196-357).

    Returns dict with beX ceX bmY cmY Cb C2 den_Exdz den_Hydz (each Nz+1)."""
    n = P.Nz + 1
    pml = P.pmlWidth
    if upExH is None:
        upExH = np.ones(n)
    kappa = np.ones(n)
    sigma = np.zeros(n)
    alpha = np.zeros(n)
    out = {k: np.zeros(n) for k in ("beX", "ceX", "bmY", "cmY", "Cb", "C2")}
    out["den_Exdz"] = np.ones(n)
    out["den_Hydz"] = np.ones(n)
    if not (P.CPMLXp or P.CPMLXm):
        return out
    nz = np.arange(0, pml, 1)
    kn = 1 + (P.kappaMax - 1) * ((pml - nz) / (pml)) ** P.r_scale
    sn = P.sigmaOpt * ((pml - nz) / (pml)) ** P.r_scale
    an = P.alphaMax * ((nz + 1) / (pml)) ** P.r_a_scale
    kappa[:pml] = kn
    kappa[n - pml:n] = kn[::-1]
    sigma[:pml] = sn
    sigma[n - pml:n] = sn[::-1]
    alpha[:pml] = an
    alpha[n - pml:n] = an[::-1]
    dt, e0, dz = P.delT, P.permit_0, P.dz
    for sl in (slice(None, pml), slice(n - pml, None)):
        out["beX"][sl] = np.exp(-((sigma[sl] * dt / (kappa[sl] * e0)) + ((alpha[sl] * dt) / e0)))
        out["ceX"][sl] = (out["beX"][sl] - 1) * sigma[sl] / (
            (sigma[sl] * kappa[sl] + alpha[sl] * kappa[sl] * kappa[sl]))
        out["bmY"][sl] = np.exp(-((sigma[sl] * dt / (kappa[sl] * e0)) + ((alpha[sl] * dt) / e0)))
        out["cmY"][sl] = (out["bmY"][sl] - 1) * sigma[sl] / (
            (sigma[sl] * kappa[sl] + alpha[sl] * kappa[sl] * kappa[sl]) * dz)
    for k in list(range(0, pml)) + list(range(n - 1, n - pml, -1)):
        out["Cb"][k] = upExH[k] * upEx[k]
        out["C2"][k] = dt / P.permea_0
    jj = pml
    for j in range(n):
        if j <= pml and P.CPMLXm:
            out["den_Hydz"][j] = 1 / kappa[j]
        elif j >= n - pml and P.CPMLXp:
            out["den_Hydz"][j] = 1 / kappa[jj]
            jj -= 1
        else:
            out["den_Hydz"][j] = 1 / (1)
    jj = pml - 1
    for j in range(n):
        if j <= pml and P.CPMLXm:
            out["den_Exdz"][j] = 1 / kappa[j]
        elif j >= n - pml and P.CPMLXp:
            out["den_Exdz"][j] = 1 / kappa[jj]
            jj -= 1
        else:
            out["den_Exdz"][j] = 1 / (1)
    return out


class StabilityExit(SystemExit):
    pass


def spatial_stab(fullTime, fullSpace, spaceStep, frequency, timeStep, plasmaFreq, resonantFreq,
                 gamma):
    """genericStability.spatialStab (genericStability.py:12-62).

    Returns (lamCont, lamDisc, diff, pf, fix); raises StabilityExit where the reference exits."""
    fS = fullSpace
    sp = spaceStep
    los = (np.pi) / 2
    frq = frequency
    rad = 2 * np.pi * frq
    twoPi = rad / frq
    c0 = C0
    tim = timeStep
    if rad * tim > np.pi / 2 and frq <= 5e9:
        raise StabilityExit("unstable timestep")
    sw = np.sinc(np.pi * frq * tim)
    pf = plasmaFreq
    rf = resonantFreq
    es = (pf ** 2) / (rf ** 2) - 1
    gam = gamma
    sqN = (rad ** 2 * sw ** 2 - es * rf ** 2 * np.cos(rad * tim) + 1.0j * gam * rad * sw)
    sqD = (rad ** 2 * sw ** 2 - rf ** 2 * np.cos(rad * tim) + 1.0j * gam * rad * sw)
    arg = (rad / c0) * (sp / 2) * sw * np.sqrt(sqN / sqD)
    ans = (2 / sp) * np.arcsin(arg)
    kNum = abs(ans)
    epsNum = (((pf)) ** 2)
    epsDom = (rf ** 2 - (rad ** 2) - 1j * gam * rad)
    epsilon = 1 + (epsNum / epsDom)
    refr = np.sqrt(abs(np.real(epsilon)))
    matAdjNum = c0 * tim * np.sin((kNum * refr * sp) / 2)
    matAdjDen = refr * sp * np.sin((kNum * c0 * tim) / 2)
    fix = matAdjNum / matAdjDen
    pf = np.sqrt(abs(fix)) * pf
    lamCont = c0 / frq
    lamDisc = (twoPi) / kNum
    diff = abs(lamCont - lamDisc)
    if kNum * sp > los:
        raise StabilityExit("unstable, wave is not resolved")
    if kNum * sp * fS < (5 * lamDisc):
        raise StabilityExit("unstable because domain too small")
    return lamCont, lamDisc, diff, pf, fix


def smooth_turn_on(P: RefParams, tempfreq=0.0):
    """SmoothTurnOn (BaseFDTD11.py:104-120)."""
    frq = tempfreq if tempfreq != 0 else P.freq_in
    ppw = P.c0 / (frq * P.dz)
    Exs, Hys = [], []
    for timer in range(P.timeSteps):
        if timer * P.delT < P.period * P.Periods:
            Exs.append(float(np.sin(2.0 * np.pi / ppw * (P.courantNo * timer))))
            Hys.append(float(np.sin(2.0 * np.pi / ppw * (P.courantNo * (timer + 1)))))
        else:
            Exs.append(0)
            Hys.append(0)
    return Exs, Hys


def gaussian_source(P: RefParams):
    """Gaussian (BaseFDTD11.py:86-96)."""
    t = np.arange(P.timeSteps)
    fc = 200
    tau = fc * 2.2
    gaussArg = ((t - tau) * (t - tau)) / (fc * fc) * np.cos(2 * np.pi * P.freq_in * (t - tau))
    out = np.exp(-gaussArg) * 2
    return P.Amplitude * out / P.courantNo


def source_manager(P: RefParams):
    """SourceManager (Solver_Engine.py:89-124)."""
    if P.SineCont:
        Exs, Hys1 = smooth_turn_on(P)
        Exp, Hyp1 = np.zeros(P.timeSteps), np.zeros(P.timeSteps)
        if P.nonLinMed:
            Exp, Hyp1 = smooth_turn_on(P, tempfreq=P.freq_in * 0.8)
            Exp = np.asarray(Exp) * P.courantNo
            Hyp1 = np.asarray(Hyp1) * P.courantNo
            Exp *= 0.1
            Hyp1 *= 0.01
        Exs = np.asarray(Exs) * P.courantNo + Exp
        Hys1 = np.asarray(Hys1) * P.courantNo + Hyp1
        if P.TFSF:
            Hys1 = Hys1 * (1 / P.CharImp)
        return Exs, Hys1
    if P.Gaussian:
        Exs = gaussian_source(P)
        Hys = np.zeros(len(Exs))
        if P.TFSF:
            Hys = gaussian_source(P)
        return Exs, Hys
    return np.zeros(0), np.zeros(0)


def sig_mod(P: RefParams, sig, AmpCarr=1, AmpMod=1, tau=14.6e-10):
    """Sig_Mod with SechArr (Solver_Engine.py:126-140)."""
    trang = np.arange(len(sig)) * (P.delT)
    omega_mod = 2 * np.pi * (1 / tau)
    a = omega_mod * trang
    a = np.where(a > 50, 50, a)
    return (AmpMod + sig) * (1 / np.cosh(a))


def gauss_sine(n_steps, f, dt, t0=200.0, sigma=60.0, amp=1.0):
    """Gaussian-modulated sine soft source of the synthetic workloads (no reference counterpart)."""
    n = np.arange(n_steps, dtype=np.float64)
    return amp * np.exp(-0.5 * ((n - t0) / sigma) ** 2) * np.sin(2.0 * np.pi * f * (n - t0) * dt)


# -------------------------------------------------------------------------------------------
# integrators
# -------------------------------------------------------------------------------------------
@dataclass
class OracleResult:
    Ex: np.ndarray
    Hy: np.ndarray
    Exs: np.ndarray
    Hys: np.ndarray
    psi_Ex: np.ndarray
    psi_Hy: np.ndarray
    x1ColBe: np.ndarray
    x1ColAf: np.ndarray
    Dx: np.ndarray
    polarisationCurr: np.ndarray
    Acubic: np.ndarray
    Port1: np.ndarray
    Port2: np.ndarray
    Ex_History: np.ndarray
    plasmaFreqE: float
    coef: dict = field(default_factory=dict)
    probes: np.ndarray | None = None


def _kerr_scalars(P: RefParams, pf):
    """AcubicFinder's coefficients (BaseFDTD11.py:804-810) and NonLinExUpdate's denominator
    pieces (:863-869)."""
    epsNum = (pf * pf)
    epsDom = (P.omega_0E * P.omega_0E - (2 * np.pi * P.freq_in * 2 * np.pi * P.freq_in)
              + 1j * P.gammaE * 2 * np.pi * P.freq_in)
    epsilon = 1 + epsNum / epsDom
    cub = (P.alpha3 * P.chi3Stat) ** 2
    qua = 2 * np.real(P.alpha3 * epsilon * P.chi3Stat)
    one = np.abs(epsilon) ** 2
    e0r = P.permit_0 * np.real(np.sqrt(1.2))
    e0chi = P.permit_0 * P.chi3Stat
    return float(cub), float(qua), float(one), float(e0r), float(e0chi)


def _lorentz_scalars(P: RefParams, pf):
    """ADE_PolarisationCurrent_Ex's A, B, C (BaseFDTD11.py:620-626)."""
    D = (1 / P.delT ** 2) + (P.gammaE / (2 * P.delT))
    A = ((2 / P.delT ** 2) - P.omega_0E ** 2) / D
    B = ((P.gammaE / (2 * P.delT)) - 1 / P.delT ** 2) / D
    C = (P.permit_0 * pf ** 2) / D
    return A, B, C


def _run(mode, pol_active, P: RefParams, coef, scal, scal2, Exs, Hys, st, probe_cells, lo, hi,
         probe_out, hist):
    n = P.Nz + 1
    arrs = [np.ascontiguousarray(coef[k], dtype=np.float64) for k in
            ("upEx", "upHy", "den_Exdz", "den_Hydz", "beX", "ceX", "Cb", "bmY", "cmY", "C2")]
    ptrs = (ctypes.c_void_p * 10)(*[a.ctypes.data for a in arrs])
    sc = np.ascontiguousarray(scal, dtype=np.float64)
    sc2 = np.ascontiguousarray(scal2, dtype=np.float64)
    Exs = np.ascontiguousarray(Exs, dtype=np.float64)
    Hys = np.ascontiguousarray(Hys if len(Hys) else np.zeros(P.timeSteps), dtype=np.float64)
    pc = np.ascontiguousarray(probe_cells, dtype=np.int32)
    hist_rows = 0 if hist is None else hist.shape[0]
    rc = lib().or_run_pass(
        mode, pol_active, P.Nz, 0, P.timeSteps, P.pmlWidth, int(P.CPMLXm), int(P.CPMLXp),
        P.materialFrontEdge, P.materialRearEdge, P.nzsrc, int(P.TFSF), 0,
        ptrs, _p(sc), _p(sc2), _p(Exs), _p(Hys), P.courantNo,
        _p(st["Ex"]), _p(st["Hy"]), _p(st["Dx"]), _p(st["P"]), _p(st["Pprev"]), _p(st["psiE"]),
        _p(st["psiH"]), _p(st["A"]), _p(st["Jx"]),
        len(pc), _p(pc), lo, hi, _p(probe_out), P.vidInterval, hist_rows, _p(hist))
    if rc != 0:
        raise ValueError("oracle stepping rejected its arguments")
    return n


def _fresh_state(n):
    return {k: np.zeros(n) for k in ("Ex", "Hy", "Dx", "P", "Pprev", "psiE", "psiH", "A", "Jx")}


def integrate(P: RefParams, mode=None, Exs=None, Hys=None, extra_probes=(), n_steps=None):
    """Run the reference integrator selected by ``mode`` (default from the P flags) and return
    an :class:`OracleResult`.  ``Exs``/``Hys`` replace SourceManager's arrays when given."""
    if mode is None:
        mode = KERR if P.nonLinMed else (LINLOR if P.LorentzMed else FREESPACE)
    T = P.timeSteps
    n = P.Nz + 1
    hist = np.zeros((int(T / P.vidInterval), n))
    x1ColBe, x1ColAf = np.zeros(T), np.zeros(T)
    Port1, Port2 = np.zeros(T), np.zeros(T)
    fin_be, st_af = int(T * 0.7), int(T * 0.05)
    pf = P.plasmaFreqE
    extra = np.zeros((T, max(1, len(extra_probes))))
    user_src = Exs is not None
    if mode == KERR:
        upHy, upEx = empty_space(P)
        coef = cpml_coefficients(P, upEx)
        coef.update(upEx=upEx, upHy=upHy)
        pf = spatial_stab(T, P.Nz, P.dz, P.freq_in, P.delT, pf, P.omega_0E, P.gammaE)[3]
        if not user_src:
            Exs, Hys = source_manager(P)
        cub, qua, one, e0r, e0chi = _kerr_scalars(P, pf)
        scal = [P.delT / (P.dz), P.permit_0, 0.0, 0.0, 0.0, cub, qua, one]
        st = _fresh_state(n)
        cells = [P.materialFrontEdge, P.materialRearEdge] + list(extra_probes)
        pr = np.zeros((T, len(cells)))
        _run(KERR, 0, P, coef, scal, [e0r, e0chi], Exs, Hys, st, cells, 0, T - 1, pr, hist)
        Port1, Port2 = pr[:, 0].copy(), pr[:, 1].copy()
        extra = pr[:, 2:]
    else:
        for i in (0, 1):
            if mode == FREESPACE:
                upHy, upEx = material_update_coef(P)
            else:
                upHy, upEx = empty_space(P)
            coef = cpml_coefficients(P, upEx)
            coef.update(upEx=upEx, upHy=upHy)
            if mode == LINLOR:
                pf = spatial_stab(T, P.Nz, P.dz, P.freq_in, P.delT, pf, P.omega_0E, P.gammaE)[3]
            if not user_src:
                Exs, Hys = source_manager(P)
                if mode == FREESPACE:
                    tauIn = 1 / (P.freq_in / 5)
                    Exs = sig_mod(P, Exs, tau=tauIn)
                    Hys = sig_mod(P, Hys, AmpMod=1 / P.CharImp, tau=tauIn)
            A, B, C = _lorentz_scalars(P, pf)
            scal = [P.delT / (P.dz), P.permit_0, A, B, C, 0.0, 0.0, 0.0]
            st = _fresh_state(n)
            if i == 0:
                pr = np.zeros((T, 1))
                _run(mode, 0, P, coef, scal, [0.0, 0.0], Exs, Hys, st, [P.x1Loc], 0,
                     min(fin_be, T - 1), pr, None)
                x1ColBe = pr[:, 0].copy()
            else:
                pr = np.zeros((T, 1))
                _run(mode, 1, P, coef, scal, [0.0, 0.0], Exs, Hys, st, [P.x2Loc], st_af, T - 1,
                     pr, hist)
                x1ColAf = pr[:, 0].copy()
    return OracleResult(Ex=st["Ex"], Hy=st["Hy"], Exs=np.asarray(Exs), Hys=np.asarray(Hys),
                        psi_Ex=st["psiE"], psi_Hy=st["psiH"], x1ColBe=x1ColBe, x1ColAf=x1ColAf,
                        Dx=st["Dx"], polarisationCurr=st["P"], Acubic=st["A"], Port1=Port1,
                        Port2=Port2, Ex_History=hist, plasmaFreqE=float(pf), coef=coef,
                        probes=extra)


# -------------------------------------------------------------------------------------------
# envSetup / matSetup
# -------------------------------------------------------------------------------------------
def env_setup(newFreq_in, domainSize, minim=400, maxim=600, nonLinMed=False):
    """envSetup with VExists=False (Environment_Setup.py:19-166); 20-tuple."""
    freq_in = newFreq_in
    c0 = C0
    lamMin = (c0 / freq_in)
    Nlam = 400
    if nonLinMed:
        Nlam = 350
    dz = lamMin / Nlam
    delT = (dz / c0) * 0.95
    if nonLinMed:
        delT *= 1
    period = 1 / freq_in
    courantNo = (c0 * delT) / dz
    if courantNo > 3 or courantNo < 0:
        raise StabilityExit("courantNo is unstable")
    pmlWidth = 6 * int(lamMin / dz)
    if pmlWidth >= 12000:
        raise StabilityExit("pmlWidth too big")
    dimen = 1
    nonInt = False
    Nz = int((domainSize) / dz) + 2 * dimen * pmlWidth
    if minim == maxim:
        minim -= 1
    N = minim
    timeSteps = None
    for N in range(minim, maxim):
        check = (freq_in * N) / (1 / delT)
        if int(check) - check == 0:
            timeSteps = N
            break
        elif N == maxim - 1:
            nonInt = True
    if nonInt:
        checkNear = (freq_in * minim) / (1 / delT)
        N = 0
        for N in range(minim, maxim):
            dummyCheck = (freq_in * N) / (1 / delT)
            if int(dummyCheck) - dummyCheck < int(checkNear) - checkNear:
                checkNear = dummyCheck
    if N >= minim:
        timeSteps = N
    else:
        timeSteps = minim
    timeSteps += int(timeSteps * (Nlam / 200))
    if timeSteps >= 2 ** 15:
        raise StabilityExit("timeSteps too large")
    nzsrcFromPml = int(0.05 / dz)
    if nzsrcFromPml >= Nz * 0.65:
        raise StabilityExit("src is too far into domain")
    nzsrc = nzsrcFromPml + pmlWidth
    if nzsrc - 10 <= pmlWidth:
        raise StabilityExit("The probe for fft is in the PML region")
    MaterialDistFromPml = int(0.1 / dz)
    materialFrontEdge = MaterialDistFromPml + pmlWidth
    materialRearEdge = Nz - 1
    if materialRearEdge - materialFrontEdge < 10:
        raise StabilityExit("width is too small or negative")
    if MaterialDistFromPml >= domainSize / dz:
        raise StabilityExit("Material starts in CPML region")
    if materialFrontEdge <= nzsrc:
        raise StabilityExit("Source is inside material")
    x1Loc = materialFrontEdge - 20
    x2Loc = nzsrc - 100
    eLoss = 0
    mLoss = 0
    return (Nz, timeSteps, eLoss, mLoss, (1 - eLoss) / (1 + eLoss), 1 / (1 + eLoss),
            (1 - mLoss) / (1 + mLoss), 1 / (1 + mLoss), x1Loc, x2Loc, materialFrontEdge,
            materialRearEdge, pmlWidth, nzsrc, lamMin, dz, delT, courantNo, period, Nlam)


def mat_setup(newFreq_in, domainSize, minim=400, maxim=800):
    """matSetup (Material_Def.py:21-120); 19-tuple."""
    freq_in = newFreq_in
    c0 = C0
    lamMin = (c0 / freq_in) * 0.1
    Nlam = 20
    dz = lamMin / Nlam
    delT = 0.99 / (c0 * (1 / dz))
    period = 1 / freq_in
    courantNo = (c0 * delT) / dz
    if courantNo > 1 or courantNo < 0:
        raise StabilityExit("courantNo is unstable")
    pmlWidth = 150
    domainSize = 600
    dimen = 1
    nonInt = False
    Nz = domainSize + 2 * dimen * pmlWidth
    N = minim
    for N in range(minim, maxim):
        check = (freq_in * N) / (1 / delT)
        if int(check) - check == 0:
            break
        elif N == maxim - 1:
            nonInt = True
    if nonInt:
        checkNear = (freq_in * minim) / (1 / delT)
        for N in range(minim, maxim):
            dummyCheck = (freq_in * N) / (1 / delT)
            if int(dummyCheck) - dummyCheck < int(checkNear) - checkNear:
                checkNear = dummyCheck
    timeSteps = N
    if timeSteps >= 10000:
        raise StabilityExit("timeSteps too large")
    nzsrcFromPml = 100
    nzsrc = nzsrcFromPml + pmlWidth
    materialFrontEdge = 300 + pmlWidth
    materialRearEdge = Nz - pmlWidth - 1
    x1Loc = nzsrc + int((materialFrontEdge - nzsrc) / 2)
    x2Loc = nzsrc - (nzsrcFromPml + 10) + 50
    eLoss = 0
    mLoss = 0
    return (Nz, timeSteps, eLoss, mLoss, (1 - eLoss) / (1 + eLoss), 1 / (1 + eLoss),
            (1 - mLoss) / (1 + mLoss), 1 / (1 + mLoss), x1Loc, x2Loc, materialFrontEdge,
            materialRearEdge, pmlWidth, nzsrc, lamMin, dz, delT, courantNo, period)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))


# -------------------------------------------------------------------------------------------
# electron-beam PIC (no reference counterpart; model stated in pic_oracle.c)
# -------------------------------------------------------------------------------------------
Q_E = -1.602176634e-19  # electron charge [C]
M_E = 9.1093837139e-31  # electron mass [kg]


def pic_constants(dz, dt, weight, mu0, q=Q_E, m=M_E):
    """(kE, kH, sc, kJ, kJz) of the Boris step in normalised momentum u/c."""
    return dict(kE=q * dt / (2.0 * m * C0), kH=-q * mu0 * dt / (2.0 * m), sc=C0 * dt / dz,
                kJ=q * weight * C0, kJz=q * weight * dz / dt)


def beam(n_part, clo, chi, v_mean=0.3, v_spread=0.003, seed=20261203):
    """Seeded beam: zeta ~ U[clo, chi) (cells), vz ~ N(v_mean c, v_spread c), vx = 0.
    Returned sorted by position as (cell int32, frac, ux, uz) with u = gamma v / c."""
    rng = np.random.Generator(np.random.PCG64(seed))
    zeta = clo + (chi - clo) * rng.random(n_part)
    vz = rng.normal(v_mean, v_spread, n_part)
    uz = vz / np.sqrt(1.0 - vz * vz)
    order = np.argsort(zeta, kind="stable")
    zeta, uz = zeta[order], uz[order]
    cell = np.floor(zeta).astype(np.int32)
    return cell, zeta - cell, np.zeros(n_part), uz.copy()


def _pass_setup(P: RefParams, mode, pf):
    if mode == FREESPACE:
        upHy, upEx = material_update_coef(P)
    else:
        upHy, upEx = empty_space(P)
    coef = cpml_coefficients(P, upEx)
    coef.update(upEx=upEx, upHy=upHy)
    cub, qua, one, e0r, e0chi = _kerr_scalars(P, pf)
    A, B, C = _lorentz_scalars(P, pf)
    scal = [P.delT / (P.dz), P.permit_0, A, B, C, cub, qua, one]
    return coef, scal, [e0r, e0chi]


def integrate_pic(P: RefParams, mode, Exs, Hys, cell, frac, ux, uz, consts, clo, chi, n_steps=None,
                  probe_cells=(50, 950), n_threads=1, apply_stab=True):
    """One FDTD pass (Kerr, Lorentz with polarisation on, or free space) coupled to the beam:
    each step pushes/deposits, then runs the field step with Jx.  Particle arrays are updated
    in place.  Returns a dict of fields, last-step Jx/Jz and probe traces."""
    T = P.timeSteps if n_steps is None else n_steps
    n = P.Nz + 1
    pf = P.plasmaFreqE
    if apply_stab and mode != FREESPACE:
        pf = spatial_stab(P.timeSteps, P.Nz, P.dz, P.freq_in, P.delT, pf, P.omega_0E,
                          P.gammaE)[3]
    coef, scal, scal2 = _pass_setup(P, mode, pf)
    st = _fresh_state(n)
    Hyp = np.zeros(n)
    Jz = np.zeros(n)
    cells = np.ascontiguousarray(probe_cells, np.int32)
    pr = np.zeros((P.timeSteps, len(cells)))
    pscal = np.array([clo, chi, consts["kE"], consts["kH"], consts["sc"], consts["kJ"],
                      consts["kJz"]], np.float64)
    arrs = [np.ascontiguousarray(coef[k], dtype=np.float64) for k in
            ("upEx", "upHy", "den_Exdz", "den_Hydz", "beX", "ceX", "Cb", "bmY", "cmY", "C2")]
    ptrs = (ctypes.c_void_p * 10)(*[a.ctypes.data for a in arrs])
    sc_ = np.ascontiguousarray(scal, np.float64)
    sc2 = np.ascontiguousarray(scal2, np.float64)
    Exs = np.ascontiguousarray(Exs, np.float64)
    Hys = np.ascontiguousarray(Hys if len(Hys) else np.zeros(P.timeSteps), np.float64)
    L = lib()
    lost = 0
    for t in range(T):
        hy_now = st["Hy"].copy()
        lost += L.or_pic_step(len(cell), _p(cell), _p(frac), _p(ux), _p(uz), _p(st["Ex"]), _p(st["Hy"]),
                              _p(Hyp), _p(st["Jx"]), _p(Jz), P.Nz, _p(pscal), n_threads)
        rc = L.or_run_pass(mode, 1, P.Nz, t, 1, P.pmlWidth, int(P.CPMLXm), int(P.CPMLXp),
                           P.materialFrontEdge, P.materialRearEdge, P.nzsrc, int(P.TFSF), 1,
                           ptrs, _p(sc_), _p(sc2), _p(Exs), _p(Hys), P.courantNo,
                           _p(st["Ex"]), _p(st["Hy"]), _p(st["Dx"]), _p(st["P"]),
                           _p(st["Pprev"]), _p(st["psiE"]), _p(st["psiH"]), _p(st["A"]),
                           _p(st["Jx"]), len(cells), _p(cells), 0, P.timeSteps - 1, _p(pr),
                           0, 0, None)
        if rc != 0:
            raise ValueError("oracle stepping rejected its arguments")
        Hyp = hy_now
    return dict(Ex=st["Ex"], Hy=st["Hy"], Dx=st["Dx"], P=st["P"], Acubic=st["A"],
                psi_Ex=st["psiE"], psi_Hy=st["psiH"], Jx=st["Jx"], Jz=Jz, Hyp=Hyp,
                probes=pr[:T], lost=lost, plasmaFreqE=float(pf))


# ---- the reference's uncalled per-step variants (one grid's arrays, updated in place) ---------
# Scalar Python arithmetic in the reference's operation order (left to right); the cell loops
# are vectorised where cells are independent (numpy's elementwise products and sums round one
# by one, as the reference's scalar ones do).


def mur1d_ex(ex, e2, Nz, c0, dt, dz):
    """MUR1DEx (BaseFDTD11.py:769-788): the two loops in the reference's order."""
    m = (c0 * dt - dz) / (c0 * dt + dz)
    for k in range(1, 5):
        ex[k] = e2[k + 1] + m * (ex[k + 1] - e2[k])
    for k in range(Nz - 1, Nz - 6, -1):
        ex[k] = e2[k - 1] + m * (ex[k - 1] - e2[k])
    return ex


def ade_jx_update(jx, pc, p1, p2, front, rear, eps0, wp, w0e, w0j, gamma, dt):
    """ADE_JxUpdate (BaseFDTD11.py:543-563), cells front-1 .. rear-1."""
    coef = 1 / (eps0 * wp * w0e * w0j)
    s = slice(front - 1, rear)
    jx[s] = coef * (w0e * w0e * p1[s] + (gamma / dt) * (pc[s] - p1[s]) +
                    (pc[s] - 2 * p1[s] + p2[s]) / (dt * dt))
    return jx


def varin_pbar(pbar, ex, q, front, rear, eps0, chi1, chi3, alpha3):
    """ADE_NonLin_Pol_Ex_Pbar (BaseFDTD11.py:567-576), cells front .. rear-1."""
    s = slice(front, rear)
    E = ex[s]
    pbar[s] = eps0 * (chi1 * E + chi3 * (alpha3 * E * E * E + (1 - alpha3) * q[s] * E))
    return pbar


def varin_jp(jx, pc, pbar, front, rear, w0e, gamma, dt):
    """ADE_Lin_Curr_And_Pol_Varin (BaseFDTD11.py:579-593), cells front .. rear-1."""
    G = (gamma * dt) / 2
    A, D, B = 1 - G, 1 + G, w0e * w0e * dt
    s = slice(front, rear)
    jx[s] = (A / D) * jx[s] + (B / D) * (pbar[s] - pc[s])
    pc[s] = pc[s] + dt * jx[s]
    return jx, pc


def varin_qg(g, q, ex, front, rear, nl_gamma, nl_w0, dt):
    """ADE_Nonlin_Q_and_G (BaseFDTD11.py:596-607), cells front .. rear-1."""
    Gm = (nl_gamma * dt) / 2
    e, f, h = 1 - Gm, 1 + Gm, nl_w0 * nl_w0 * dt
    s = slice(front, rear)
    g[s] = (e / f) * g[s] + (h / f) * (ex[s] * ex[s] - q[s])
    q[s] = q[s] + dt * g[s]
    return g, q
