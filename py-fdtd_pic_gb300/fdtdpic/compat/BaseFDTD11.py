"""BaseFDTD11.py's functions: the set-up functions the integrators call once per run, the
per-step functions the integrators call every step, and the per-step functions no integrator
calls.

The integrators of this package (:mod:`Solver_Engine`) fuse many steps into one launch.  The
per-step functions here keep the reference's finer unit of work for loops built out of them:
each is one GPU launch over the state's arrays in FP64, with the reference's index ranges and
operation order (:mod:`fdtdpic.stepops`), writing its results back into the same numpy arrays
as the reference updates them in place.  A loop of these calls in the order of
``IntegratorNL1D`` (Solver_Engine.py:236-267) reproduces the reference's run.  The uncalled ones
(MUR1DEx, ADE_JxUpdate and Varin's three ADE updates) are one launch each too
(:mod:`fdtdpic.variants`).  The CPML set-up chain (CPML_ScalingCalc .. denominators) runs once
per grid on the host, in numpy.
"""
from __future__ import annotations

import sys

import numpy as np

from .. import physics_setup as ps


def FieldInit(V, P):
    """Argument checks and zeroed fields (:36-82); a failed check prints and exits as the
    reference does (TypeError for non-integer sizes propagates)."""
    if type(P.Nz) != int:
        raise TypeError("Grid spaces must be a positive integer value")
    if type(P.timeSteps) != int:
        raise TypeError("Number of timeSteps must be positive integer valued")
    msg = None
    if P.timeSteps > 2 ** 17:
        msg = "timeSteps max too large"
    elif P.Nz > 25000:
        msg = "Grid size too big"
    elif P.Nz == 0:
        msg = "Cannot have grid size 0!"
    elif P.timeSteps == 0:
        msg = "Cannot have zero timeSteps!"
    elif P.Nz < 0:
        msg = "Grid size cannot be negative"
    elif P.timeSteps < 0:
        msg = "Cannot have negative timeSteps"
    if msg is not None:
        print(msg)
        sys.exit()
    n = P.Nz + 1
    V.Ex = np.zeros(n)
    V.Hy = np.zeros(n)
    V.polarisationCurr = np.zeros(n)
    V.Dx = np.zeros(n)
    V.tempVarPol = np.zeros(n)
    V.tempTempVarPol = np.zeros(n)
    V.tempVarE = np.zeros(n)
    V.tempTempVarE = np.zeros(n)
    return (V.tempVarPol, V.tempTempVarE, V.tempVarE, V.tempTempVarPol, V.polarisationCurr,
            V.Ex, V.Dx, V.Hy)


def Gaussian(V, P):
    """Gaussian source of the free-space runs (:86-96)."""
    return ps.gaussian(P)


def SmoothTurnOn(V, P, tempfreq=0):
    """Switched sine source pair (Exs, Hys) as lists (:104-120)."""
    return ps.smooth_turn_on(P, tempfreq)


def EmptySpaceCalc(V, P):
    """Uniform update coefficients (:124-132)."""
    ue, _, uh, _ = ps.update_coefficients(P, False)
    V.UpHyMat = np.full(P.Nz + 1, uh)
    V.UpExMat = np.full(P.Nz + 1, ue)
    return V.UpHyMat, V.UpExMat


def Material(V, P):
    """Slab constants over cells [0, Nz) (:136-161): inside [front, rear) epsRe/muRe and the
    loss coefficients, 1 elsewhere.  Index Nz of the Nz+1 arrays is left as it was."""
    nz = P.Nz
    k = np.arange(nz)
    slab = (k >= int(P.materialFrontEdge)) & (k < int(P.materialRearEdge))
    V.epsilon = np.where(slab, P.epsRe, 1.0)
    V.mu = np.where(slab, P.muRe, 1.0)
    for name, inside in (("UpExHcompsCo", P.eHcompsCo), ("UpExSelf", P.eSelfCo),
                         ("UpHyEcompsCo", P.hEcompsCo), ("UpHySelf", P.hSelfCo)):
        arr = getattr(V, name)
        arr[:nz] = np.where(slab, inside, 1.0)
    return V.epsilon, V.mu, V.UpExHcompsCo, V.UpExSelf, V.UpHyEcompsCo, V.UpHySelf


def UpdateCoef(V, P):
    """Update coefficients divided by epsilon/mu across the slab (:167-182)."""
    ue, _, uh, _ = ps.update_coefficients(P, False)
    UpHyMat = np.full(P.Nz + 1, uh)
    UpExMat = np.full(P.Nz + 1, ue)
    sl = slice(int(P.materialFrontEdge), int(P.materialRearEdge))
    UpExMat[sl] = UpExMat[sl] / V.epsilon[sl]
    UpHyMat[sl] = UpHyMat[sl] / V.mu[sl]
    return UpHyMat, UpExMat


def CPML_FieldInit(V, P, C_V, C_P):
    """Fresh CPML profiles and auxiliary fields (:196-220)."""
    n = P.Nz + 1
    C_V.kappa_Ex = np.ones(n)
    C_V.kappa_Hy = np.ones(n)
    C_V.psi_Ex = np.zeros(n)
    C_V.psi_Hy = np.zeros(n)
    for name in ("alpha_Ex", "alpha_Hy", "sigma_Ex", "sigma_Hy", "beX", "bmY", "ceX", "cmY",
                 "eLoss_CPML", "mLoss_CPML", "Ca", "Cb", "Cc", "C1", "C2", "C3"):
        setattr(C_V, name, np.zeros(n))
    C_V.den_Exdz = np.ones(n)
    C_V.den_Hydz = np.ones(n)
    return C_V


def AnalyticalReflectionE(V, P):
    """Fresnel normal-incidence reflection |(n2 - 1)/(n2 + 1)| of the Lorentz slab at freq_in,
    n2 = Re(sqrt(eps(freq_in))) (:882-923)."""
    eps = ps.complex_eps(V.plasmaFreqE, V.omega_0E, V.gammaE, P.freq_in)
    n2 = np.real(np.sqrt(eps))
    reflection = abs((n2 - 1) / (1 + n2))
    print(reflection, "NEW ANALYTICAL REFLECTION USING FRESNEL NORMAL INCIDENCE.")
    return reflection


# ---- per-step functions the reference defines but does not call ------------------------------
# Each copies the arrays it reads to the GPU, runs the update there in FP64 (the reference's
# values) and writes the result back into the same numpy arrays, as the reference updates them
# in place; returns what the reference returns.


def _variant(op, V, P, names, **constants):
    import torch

    from .. import variants
    arrs = [getattr(V, k) for k in names]
    n = len(arrs[0])
    rec = variants.make_rows(n, int(P.Nz), int(P.materialFrontEdge), int(P.materialRearEdge),
                             c0=P.c0, dt=P.delT, dz=P.dz, eps0=P.permit_0, **constants)
    rows = variants.Rows(rec)
    dev = rows.device.device
    ts = [torch.from_numpy(np.ascontiguousarray(a, np.float64)).reshape(1, n).to(dev) for a in arrs]
    variants.run(op, rows, ts)
    for a, t in zip(arrs, ts):
        a[...] = t.reshape(n).cpu().numpy()


def MUR1DEx(V, P, C_V, C_P):
    """First-order Mur update of Ex's cells 1-4 and Nz-5..Nz-1 from ``tempTempVarE``
    (:769-788)."""
    from .._lib import VAR_MUR_EX
    _variant(VAR_MUR_EX, V, P, ("Ex", "tempTempVarE"))
    return V.Ex


def ADE_JxUpdate(V, P, C_V, C_P):
    """Polarisation current over cells materialFrontEdge-1 .. materialRearEdge-1 (:543-563).
    Reads ``V.omega_0`` as the reference does (its Variables has no such member, so unless the
    caller set one this raises AttributeError, as the reference's call would)."""
    from .._lib import VAR_ADE_JX
    w0j = V.omega_0
    _variant(VAR_ADE_JX, V, P, ("Jx", "polarisationCurr", "tempVarPol", "tempTempVarPol"),
             plasma_freq=V.plasmaFreqE, omega0=V.omega_0E, gamma=V.gammaE, omega0_j=w0j)
    return V.Jx


def ADE_NonLin_Pol_Ex_Pbar(V, P):
    """Varin's instantaneous nonlinear polarisation Pbar3 (:567-576).  The reference stops in
    the debugger when Pbar3 is already non-zero on entry; that check is not carried over."""
    from .._lib import VAR_VARIN_PBAR
    _variant(VAR_VARIN_PBAR, V, P, ("Pbar3", "Ex", "Qx3"), chi1=V.chi1Stat, chi3=V.chi3Stat,
             alpha3=V.alpha3)
    return V.Pbar3


def ADE_Lin_Curr_And_Pol_Varin(V, P):
    """Varin's Lorentz current and polarisation driven by Pbar3 (:579-593)."""
    from .._lib import VAR_VARIN_JP
    _variant(VAR_VARIN_JP, V, P, ("Jx", "polarisationCurr", "Pbar3"), omega0=V.omega_0E,
             gamma=V.gammaE)
    return V.Jx, V.polarisationCurr


def ADE_Nonlin_Q_and_G(V, P):
    """Varin's Raman oscillator G, Q driven by E^2 (:596-607)."""
    from .._lib import VAR_VARIN_QG
    _variant(VAR_VARIN_QG, V, P, ("Gx3", "Qx3", "Ex"), nl_gamma=V.nonLin3gammaE,
             nl_omega0=V.nonLin3Omega_0E)
    return V.Gx3, V.Qx3, V.Ex


# ---- CPML set-up, once per grid (BaseFDTD11.py:223-357; called by boundCondManager,
# Solver_Engine.py:70-87, in this order) ------------------------------------------------------
def _ends(V, P):
    n = len(V.Ex)
    return slice(0, P.pmlWidth), slice(n - P.pmlWidth, n)


def CPML_ScalingCalc(V, P, C_V, C_P):
    """Graded kappa, sigma, alpha over the PML columns (:223-272).  The Hy profiles become the
    Ex arrays themselves (the reference assigns the objects, so they alias from here on)."""
    pml = P.pmlWidth
    nz = np.arange(0, pml, 1)
    ramp = ((pml - nz) / (pml)) ** C_P.r_scale
    kap = 1 + (C_P.kappaMax - 1) * ramp
    sig = C_P.sigmaOpt * ramp
    alp = C_P.alphaMax * ((nz + 1) / (pml)) ** C_P.r_a_scale
    left, right = _ends(V, P)
    for name, prof in (("kappa_Ex", kap), ("sigma_Ex", sig), ("alpha_Ex", alp)):
        arr = getattr(C_V, name)
        arr[left] = prof
        arr[right] = prof[::-1]
    C_V.kappa_Hy = C_V.kappa_Ex
    C_V.sigma_Hy = C_V.sigma_Ex
    C_V.alpha_Hy = C_V.alpha_Ex
    return C_V.sigma_Ex, C_V.sigma_Hy, C_V.alpha_Ex, C_V.alpha_Hy, C_V.kappa_Ex, C_V.kappa_Hy


def _rc(C_V, P, which, sl, per_dz):
    s_, k_, a_ = (getattr(C_V, f"{q}_{which}")[sl] for q in ("sigma", "kappa", "alpha"))
    b = np.exp(-((s_ * P.delT / (k_ * P.permit_0)) + ((a_ * P.delT) / P.permit_0)))
    den = (s_ * k_ + a_ * k_ * k_)
    if per_dz:
        den = den * P.dz
    return b, (b - 1) * s_ / den


def CPML_Ex_RC_Define(V, P, C_V, C_P):
    """beX, ceX over the PML columns (:275-286)."""
    for sl in _ends(V, P):
        C_V.beX[sl], C_V.ceX[sl] = _rc(C_V, P, "Ex", sl, False)
    return C_V.beX, C_V.ceX


def CPML_HY_RC_Define(V, P, C_V, C_P):
    """bmY, cmY over the PML columns (:289-296); cmY carries the extra 1/dz."""
    for sl in _ends(V, P):
        C_V.bmY[sl], C_V.cmY[sl] = _rc(C_V, P, "Hy", sl, True)
    return C_V.bmY, C_V.cmY


def _coef_cells(V, P):
    """Cells 0..pml-1, then len-1 down to len-pml+1 (the reference's right-hand loops stop one
    cell short, so index len-pml keeps its old value)."""
    n = len(V.Hy)
    return np.r_[0:P.pmlWidth, n - 1:n - P.pmlWidth:-1]


def CPML_Ex_Update_Coef(V, P, C_V, C_P):
    """eLoss, Ca, Cb, Cc over the PML columns (:299-318)."""
    betaE = (0.5 * V.plasmaFreqE * V.plasmaFreqE * P.permit_0 * P.delT) / (1 + 0.5 * V.gammaE * P.delT)
    a = ((2 * P.permit_0 - betaE * P.delT) / (2 * P.permit_0 + betaE * P.delT))
    k = _coef_cells(V, P)
    C_V.eLoss_CPML[k] = (C_V.sigma_Ex[k] * P.delT) / (2 * P.permit_0)
    C_V.Ca[k] = a
    C_V.Cb[k] = V.UpExHcompsCo[k] * V.UpExMat[k]
    C_V.Cc[k] = P.delT / ((1 + C_V.eLoss_CPML[k]) * P.permit_0)
    return C_V.eLoss_CPML, C_V.Ca, C_V.Cb, C_V.Cc


def CPML_Hy_Update_Coef(V, P, C_V, C_P):
    """C1, C2, C3 over the PML columns (:321-330)."""
    k = _coef_cells(V, P)
    C_V.C1[k] = 1
    C_V.C2[k] = P.delT / P.permea_0
    C_V.C3[k] = P.delT / ((1 + C_V.mLoss_CPML[k]) * P.permea_0)
    return C_V.mLoss_CPML, C_V.C1, C_V.C2, C_V.C3


def denominators(V, P, C_V, C_P):
    """1/kappa over the PML columns (:333-357), each right-hand walk with its own counter:
    den_Hydz reads kappa_Hy[pml], [pml-1], ...; den_Exdz kappa_Ex[pml-1], [pml-2], ..."""
    for arr_name, kap_name, start in (("den_Hydz", "kappa_Hy", P.pmlWidth),
                                      ("den_Exdz", "kappa_Ex", P.pmlWidth - 1)):
        arr, kap = getattr(C_V, arr_name), getattr(C_V, kap_name)
        n = len(arr)
        jj = start
        for j in range(0, n):
            if j <= P.pmlWidth and P.CPMLXm:
                arr[j] = 1 / (kap[j])
            elif j >= n - P.pmlWidth and P.CPMLXp:
                arr[j] = 1 / (kap[jj])
                jj -= 1
            else:
                arr[j] = 1 / (1)
    return C_V.den_Exdz, C_V.den_Hydz


# ---- per-step functions the integrators call, one GPU launch each -----------------------------
def _curl(y, x, lo, hi, xa, xb, factors=(), self_=None, j=None):
    from .. import stepops as so
    slots = [y, x, self_, j, None, None, None, None]
    fmode, fval = [0, 0, 0], [0.0, 0.0, 0.0]
    for i, (mode, f) in enumerate(factors):
        fmode[i] = mode
        if isinstance(f, np.ndarray):
            slots[4 + i] = f
        else:
            fval[i] = float(f)
    so.run(so.make_op(so.OP_CURL, lo, hi, xa, xb, fmode, fval), slots, (0,))


def _psi(psi, y, x, b, c, C, lo, hi, xa, xb, sign):
    from .. import stepops as so
    so.run(so.make_op(so.OP_PSI, lo, hi, xa, xb, s=(sign, 0.0, 0.0, 0.0)),
           [psi, y, x, b, c, C, None, None], (0, 1))


def ADE_ExUpdate(V, P, C_V, C_P, counts):
    """Ex += (Hy[k] - Hy[k-1] - Jx[k]) UpExMat[k] den_Exdz[k] for k in [1, len(Ex)) (:664-669)."""
    from ..stepops import MUL
    _curl(V.Ex, V.Hy, 1, len(V.Ex), 0, -1, ((MUL, V.UpExMat), (MUL, C_V.den_Exdz)), j=V.Jx)
    return V.Ex


def ADE_HyUpdate(V, P, C_V, C_P):
    """Hy = Hy UpHySelf + (Ex[k+1] - Ex[k]) UpHyMat den_Hydz for k in [1, Nz) (:641-656)."""
    from ..stepops import MUL
    _curl(V.Hy, V.Ex, 1, P.Nz, 1, 0, ((MUL, V.UpHyMat), (MUL, C_V.den_Hydz)), self_=V.UpHySelf)
    return V.Hy


def CPML_Psi_e_Update(V, P, C_V, C_P):
    """psi_Ex = beX psi_Ex + ceX (Hy[k] - Hy[k-1]); Ex -= Cb psi_Ex over [1, pml) (CPMLXm) then
    [len-pml, len) (CPMLXp) (:365-376)."""
    n = len(V.Ex)
    for on, lo, hi in ((P.CPMLXm, 1, P.pmlWidth), (P.CPMLXp, n - P.pmlWidth, n)):
        if on:
            _psi(C_V.psi_Ex, V.Ex, V.Hy, C_V.beX, C_V.ceX, C_V.Cb, lo, hi, 0, -1, -1.0)
    return C_V.psi_Ex, V.Ex


def CPML_Psi_m_Update(V, P, C_V, C_P):
    """psi_Hy = bmY psi_Hy + cmY (Ex[k+1] - Ex[k]); Hy += C2 psi_Hy over [1, pml) (CPMLXm) then
    [len-pml, len-1) (CPMLXp) (:382-393)."""
    n = len(V.Ex)
    for on, lo, hi in ((P.CPMLXm, 1, P.pmlWidth), (P.CPMLXp, n - P.pmlWidth, n - 1)):
        if on:
            _psi(C_V.psi_Hy, V.Hy, V.Ex, C_V.bmY, C_V.cmY, C_V.C2, lo, hi, 1, 0, 1.0)
    return C_V.psi_Hy, V.Hy


def ADE_DxUpdate(V, P, C_V, C_P):
    """Dx += (Hy[k] - Hy[k-1]) (delT/dz) den_Exdz over the slab (:751-760)."""
    from ..stepops import MUL
    _curl(V.Dx, V.Hy, P.materialFrontEdge, P.materialRearEdge, 0, -1,
          ((MUL, P.delT / (P.dz)), (MUL, C_V.den_Exdz)))
    return V.Dx


def ADE_PolarisationCurrent_Ex(V, P, C_V, C_P, counts):
    """P = A P + B P_(n-1) + C Ex over the slab, A, B, C from the Lorentz ADE (:610-633)."""
    from .. import stepops as so
    D = (1 / P.delT ** 2) + (V.gammaE / (2 * P.delT))
    A = ((2 / P.delT ** 2) - V.omega_0E ** 2) / D
    B = ((V.gammaE / (2 * P.delT)) - 1 / P.delT ** 2) / D
    C = (P.permit_0 * V.plasmaFreqE ** 2) / D
    so.run(so.make_op(so.OP_POL, int(P.materialFrontEdge), int(P.materialRearEdge),
                      s=(A, B, C, 0.0)),
           [V.polarisationCurr, V.polarisationCurr, V.tempTempVarPol, V.Ex, None, None, None,
            None], (0,))
    return V.polarisationCurr


def ADE_ExCreate(V, P, C_V, C_P):
    """Ex = (Dx - P) / permit_0 over the slab (:713-725)."""
    from .. import stepops as so
    so.run(so.make_op(so.OP_EXCREATE, P.materialFrontEdge, P.materialRearEdge,
                      s=(P.permit_0, 0.0, 0.0, 0.0)),
           [V.Ex, V.Dx, V.polarisationCurr, None, None, None, None, None], (0,))
    return V.Ex


def AcubicFinder(V, P):
    """The Kerr amplitude A of every slab cell (:803-820 with Nonlin_Eqn_Setup :795-800 and
    Nonlin_Cubic_Solver :824-853): cubPoly[k] = (cub, qua, one, -|Dx/permit_0|^2), A = Re of
    CubicEquationSolver.solve's first root where |d| > 1e-8, else 0 -- on the GPU.  (The
    reference also leaves the last solved roots in V.roots, a scratch member; not kept.)"""
    from .. import stepops as so
    cub, qua, one, _, _ = ps.kerr_coefficients(P, V, V.plasmaFreqE)
    lo, hi = int(P.materialFrontEdge), int(P.materialRearEdge)
    d = np.zeros(len(V.Dx))
    so.run(so.make_op(so.OP_ACUBIC, lo, hi, s=(P.permit_0, cub, qua, one)),
           [V.Acubic, V.Dx, d, None, None, None, None, None], (0, 2))
    V.cubPoly[lo:hi, 0], V.cubPoly[lo:hi, 1], V.cubPoly[lo:hi, 2] = cub, qua, one
    V.cubPoly[lo:hi, 3] = d[lo:hi]
    return V.Acubic


def NonLinExUpdate(V, P):
    """Ex = Dx / (permit_0 Re(sqrt 1.2) + permit_0 chi3Stat A) over the slab (:859-877)."""
    from .. import stepops as so
    eps0 = P.permit_0
    so.run(so.make_op(so.OP_NONLIN_EX, P.materialFrontEdge, P.materialRearEdge,
                      s=(eps0 * np.real(np.sqrt(1.2)), eps0 * V.chi3Stat, 0.0, 0.0)),
           [V.Ex, V.Dx, V.Acubic, None, None, None, None, None], (0,))
    return V.Ex


def ADE_TempPolCurr(V, P, C_V, C_P):
    """The history shuffle of the Lorentz pass (:487-538), host-only: P_(n-1) and E_(n-1) become
    copies of the previous P and E, Ex and polarisationCurr become fresh copies of themselves,
    and the Dx/Hy/Jx/psi histories take the current arrays themselves (the reference assigns
    those objects without copying).  The reference's debugger stop when P is non-zero and equal
    to P_(n-1) is not carried over."""
    tTVP = np.array(V.tempVarPol, dtype=np.float64)
    tVP = np.array(V.polarisationCurr, dtype=np.float64)
    V.tempTempVarDx = V.tempVarDx
    V.tempVarDx = V.Dx
    tTVE = np.array(V.tempVarE, dtype=np.float64)
    tVE = np.array(V.Ex, dtype=np.float64)
    V.tempTempVarHy = V.tempVarHy
    V.tempVarHy = V.Hy
    V.tempTempVarJx = V.tempVarJx
    V.tempVarJx = V.Jx
    C_V.tempTempVarPsiEx = getattr(C_V, "tempVarPsiEx", None)
    C_V.tempVarPsiEx = C_V.psi_Ex
    C_V.tempTempVarPsiHy = getattr(C_V, "tempVarPsiHy", None)
    C_V.tempVarPsiHy = C_V.psi_Hy
    V.tempTempVarPol = tTVP
    V.tempVarPol = tVP
    V.polarisationCurr = np.array(tVP)
    V.tempTempVarE = tTVE
    V.tempVarE = tVE
    V.Ex = np.array(tVE)
    return (V.tempTempVarPol, V.tempVarPol, V.tempVarE, V.tempTempVarE, V.tempTempVarHy,
            V.tempVarHy, V.tempTempVarJx, V.tempVarJx, C_V.tempTempVarPsiEx, C_V.tempVarPsiEx,
            C_V.tempTempVarPsiHy, C_V.tempVarPsiHy)
