"""The legacy module BaseFDTD.py (BaseFDTD.py:27-436): the older twin of BaseFDTD11 with its own
index ranges and formulas, kept under its names and signatures.

Its per-step functions are one GPU launch each in FP64 with the legacy ranges and operation
order (:mod:`fdtdpic.stepops`), writing back into the same numpy arrays as the reference updates
them in place; its set-up functions run on the host in numpy, once per grid.  Quirks kept: the
sign of the psi terms (Ex gains +Cb psi_Ex; psi_Hy takes Ex[k] - Ex[k+1]), the split ranges of
ADE_ExUpdate, the operator precedence of alpha_Hy in CPML_ScalingCalc (nz1 - 0.5/(pml-1)),
EmptySpaceCalc leaving index Nz at 0, C2 = -delT/permea_0.
"""
from __future__ import annotations

import sys

import numpy as np

from .BaseFDTD11 import _curl, _psi


def sourceGen(T):
    """exp(-(T-30)^2/100) (:27-29)."""
    return np.exp(-(T - 30) * (T - 30) / 100)


def sourceGen2(P, T):
    """sin(2 pi freq_in delT T) (:31-33)."""
    return np.sin(2 * np.pi * P.freq_in * P.delT * T)


def FieldInit(V, P):
    """Argument checks (print and exit, as the reference does) and zeroed fields (:35-80)."""
    if type(P.Nz) != int:
        raise TypeError("Grid spaces must be a positive integer value")
    if type(P.timeSteps) != int:
        raise TypeError("Number of timeSteps must be positive integer valued")
    msg = None
    if P.timeSteps > 2 ** 14:
        msg = "timeSteps max too large"
    elif P.Nz > 3000:
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
    V.Ex_History = [[]] * P.timeSteps
    V.Hy_History = [[]] * P.timeSteps
    V.Psi_Ex_History = [[]] * P.timeSteps
    V.Psi_Hy_History = [[]] * P.timeSteps
    V.Exs = []
    V.Hys = []
    V.polarisationCurr = np.zeros(n)
    V.Dx = np.zeros(n)
    V.tempVarPol = np.zeros(n)
    V.tempTempVarPol = np.zeros(n)
    return (V.tempTempVarPol, V.polarisationCurr, V.Ex, V.Dx, V.Ex_History, V.Hy, V.Hy_History,
            V.Psi_Ex_History, V.Psi_Hy_History, V.Exs, V.Hys)


def SmoothTurnOn(V, P):
    """One switched sine period (:82-106): Exs/Hys follow sin(2 pi Sc n / ppw) until the wave
    has gone negative and come back positive, zero afterwards (the index where it turns
    positive again is zeroed in Hys too)."""
    V.Exs = np.zeros(P.timeSteps)
    V.Hys = np.zeros(P.timeSteps)
    ppw = P.c0 / (P.freq_in * P.dz)
    phase1 = phase2 = False
    p1Ind = p2Ind = 0
    for timer in range(P.timeSteps):
        V.Exs[timer] = (np.sin(2.0 * np.pi / ppw * (P.courantNo * timer)))
        V.Hys[timer] = (np.sin(2.0 * np.pi / ppw * (P.courantNo * (timer + 1))))
        if V.Exs[timer] < 0 and not phase1:
            p1Ind = timer
            phase1 = True
            print(p1Ind, "p1Ind")
        if V.Exs[timer] > 0 and phase1 and not phase2:
            p2Ind = timer
            phase2 = True
            print(p2Ind, "p2Ind")
        if phase2 and phase1:
            V.Exs[timer] = 0.0
            V.Hys[timer] = 0.0
        if V.Hys[p2Ind] != 0 and phase2:
            V.Hys[p2Ind] = 0.0
    return V.Exs, V.Hys


def EmptySpaceCalc(V, P):
    """Uniform update coefficients over cells [0, Nz); index Nz stays 0 (:109-119)."""
    V.UpHyMat = np.zeros(P.Nz + 1)
    V.UpExMat = np.zeros(P.Nz + 1)
    V.UpExMat[0:P.Nz] = P.CharImp * P.courantNo
    V.UpHyMat[0:P.Nz] = (1 / P.CharImp) * P.courantNo
    return V.UpHyMat, V.UpExMat


def Material(V, P):
    """Slab constants over cells [0, Nz) (:122-151)."""
    nz = P.Nz
    k = np.arange(nz)
    slab = (k >= int(P.materialFrontEdge)) & (k < int(P.materialRearEdge))
    V.epsilon = np.where(slab, P.epsRe, 1.0)
    V.mu = np.where(slab, P.muRe, 1.0)
    for name, inside in (("UpExHcompsCo", P.eHcompsCo), ("UpExSelf", P.eSelfCo),
                         ("UpHyEcompsCo", P.hEcompsCo), ("UpHySelf", P.hSelfCo)):
        getattr(V, name)[:nz] = np.where(slab, inside, 1.0)
    return V.epsilon, V.mu, V.UpExHcompsCo, V.UpExSelf, V.UpHyEcompsCo, V.UpHySelf


def UpdateCoef(V, P):
    """Background coefficients divided by epsilon/mu over cells [0, Nz) (:154-165)."""
    UpHyMat = np.zeros(P.Nz + 1)
    UpExMat = np.zeros(P.Nz + 1)
    UpExMat[:P.Nz] = (P.CharImp * P.courantNo) / V.epsilon[:P.Nz]
    UpHyMat[:P.Nz] = ((1 / P.CharImp) * P.courantNo) / V.mu[:P.Nz]
    return UpHyMat, UpExMat


def HyTfSfCorr(V, P, counts):
    """Hy[nzsrc-1] -= Exs[counts]/CharImp (:168-170)."""
    V.Hy[P.nzsrc - 1] -= V.Exs[counts] / P.CharImp
    return V.Hy[P.nzsrc - 1]


def ExTfSfCorr(V, P, counts):
    """Ex[nzsrc] += Hys[counts] (:172-174)."""
    V.Ex[P.nzsrc] += V.Hys[counts]
    return V.Ex[P.nzsrc]


def CPML_FieldInit(V, P, C_V, C_P):
    """Zeroed CPML arrays (:176-197)."""
    n = P.Nz + 1
    for name in ("kappa_Ex", "kappa_Hy", "psi_Ex", "psi_Hy", "alpha_Ex", "alpha_Hy", "sigma_Ex",
                 "sigma_Hy", "beX", "bmY", "ceX", "cmY", "eLoss_CPML", "mLoss_CPML", "Ca", "Cb",
                 "Cc", "C1", "C2", "C3"):
        setattr(C_V, name, np.zeros(n))
    return C_V


def CPML_ScalingCalc(V, P, C_V, C_P):
    """Graded profiles over cells [0, Nz) with the legacy mirror walk (:199-236)."""
    pml = P.pmlWidth
    jj, jjj = pml, pml - 1
    for nz in range(P.Nz):
        nz1 = nz + 1
        if nz1 <= pml:
            C_V.kappa_Ex[nz] = 1 + (C_P.kappaMax - 1) * ((pml - nz1) / (pml - 1)) ** C_P.r_scale
            C_V.sigma_Ex[nz] = C_P.sigmaOpt * ((pml - nz1) / (pml - 1)) ** C_P.r_scale
            C_V.alpha_Ex[nz] = C_P.alphaMax * (nz1 / (pml - 1)) ** C_P.r_a_scale
        elif nz >= P.Nz + 2 - pml:
            C_V.kappa_Ex[nz] = C_V.kappa_Ex[jj]
            C_V.sigma_Ex[nz] = C_V.sigma_Ex[jj]
            C_V.alpha_Ex[nz] = C_V.alpha_Ex[jj]
            jj -= 1
        else:
            C_V.kappa_Ex[nz] = 1
            C_V.sigma_Ex[nz] = 0
            C_V.alpha_Ex[nz] = 0
        if nz1 <= pml - 1:
            C_V.kappa_Hy[nz] = 1 + (C_P.kappaMax - 1) * ((pml - nz1 - 0.5) / (pml - 1)) ** C_P.r_scale
            C_V.sigma_Hy[nz] = C_P.sigmaOpt * ((pml - nz1 - 0.5) / (pml - 1)) ** C_P.r_scale
            C_V.alpha_Hy[nz] = C_P.alphaMax * (nz1 - 0.5 / (pml - 1)) ** C_P.r_a_scale
        elif nz >= P.Nz + 2 - pml:
            C_V.kappa_Hy[nz] = C_V.kappa_Hy[jjj]
            C_V.sigma_Hy[nz] = C_V.sigma_Hy[jjj]
            C_V.alpha_Hy[nz] = C_V.alpha_Hy[jjj]
            jjj -= 1
        else:
            C_V.kappa_Hy[nz] = 1
            C_V.sigma_Hy[nz] = 0
            C_V.alpha_Hy[nz] = 0
    return C_V.sigma_Ex, C_V.sigma_Hy, C_V.alpha_Ex, C_V.alpha_Hy, C_V.kappa_Ex, C_V.kappa_Hy


def CPML_Ex_RC_Define(V, P, C_V, C_P):
    """beX, ceX with the legacy walk (:239-263)."""
    pml = P.pmlWidth
    jjj = pml - 1
    s, k, a = C_V.sigma_Ex, C_V.kappa_Ex, C_V.alpha_Ex
    for nz in range(0, P.Nz):
        if nz <= pml - 1 or nz >= P.Nz + 2 - pml:
            C_V.beX[nz] = np.exp(-((s[nz] * P.delT / k[nz]) + ((a[nz] * P.delT) / P.permit_0)))
        else:
            C_V.beX[nz] = 0
        if s[nz] == 0 and nz == pml - 1 and a[nz] == 0:
            C_V.ceX[nz] = 0
        elif nz <= pml - 1:
            C_V.ceX[nz] = (C_V.beX[nz] - 1) * s[nz] / (s[nz] + a[nz] * k[nz]) / k[nz]
        elif nz >= P.Nz + 2 - pml:
            C_V.ceX[nz] = (C_V.beX[jjj] - 1) * s[jjj] / (s[jjj] + a[jjj] * k[jjj]) / k[jjj]
            jjj -= 1
        else:
            C_V.ceX[nz] = 0
    return C_V.beX, C_V.ceX


def CPML_HY_RC_Define(V, P, C_V, C_P):
    """bmY, cmY with the legacy walk (:266-289)."""
    pml = P.pmlWidth
    jj = jjj = pml - 2
    s, k, a = C_V.sigma_Hy, C_V.kappa_Hy, C_V.alpha_Hy
    for nz in range(0, P.Nz):
        if nz <= pml - 2:
            C_V.bmY[nz] = np.exp(-(s[nz] / (k[nz] + a[nz])) * P.delT / P.permea_0)
        elif nz >= P.Nz + 2 - pml:
            C_V.bmY[nz] = np.exp(-(s[jj] / (k[jj] + a[jj])) * P.delT / P.permea_0)
            jj -= 1
        else:
            C_V.bmY[nz] = 0
        if s[nz] == 0 and nz == pml - 1 and a[nz] == 0:
            C_V.cmY[nz] = 0
        elif nz <= pml - 1:
            C_V.cmY[nz] = (C_V.bmY[nz] - 1) * s[nz] / (s[nz] + a[nz] * k[nz]) / k[nz]
        elif nz >= P.Nz + 2 - pml:
            C_V.cmY[nz] = (C_V.bmY[jjj] - 1) * s[jjj] / (s[jjj] + a[jjj] * k[jjj]) / k[jjj]
            jjj -= 1
        else:
            C_V.cmY[nz] = 0
    return C_V.bmY, C_V.cmY


def CPML_Ex_Update_Coef(V, P, C_V, C_P):
    """eLoss, Ca, Cb, Cc over cells [0, Nz-1) (:292-299)."""
    k = slice(0, P.Nz - 1)
    C_V.eLoss_CPML[k] = (C_V.sigma_Ex[k] * P.delT) / (2 * P.permit_0)
    C_V.Ca[k] = V.UpExSelf[k]
    C_V.Cb[k] = V.UpExHcompsCo[k] * V.UpExMat[k]
    C_V.Cc[k] = P.delT / ((1 + C_V.eLoss_CPML[k]) * P.permit_0)
    return C_V.eLoss_CPML, C_V.Ca, C_V.Cb, C_V.Cc


def CPML_Hy_Update_Coef(V, P, C_V, C_P):
    """C1, C2 = -delT/permea_0, C3 over cells [0, Nz-2) (:302-307)."""
    k = slice(0, P.Nz - 2)
    C_V.C1[k] = 1
    C_V.C2[k] = -P.delT / P.permea_0
    C_V.C3[k] = P.delT / ((1 + C_V.mLoss_CPML[k]) * P.permea_0)
    return C_V.mLoss_CPML, C_V.C1, C_V.C2, C_V.C3


def denominators(V, P, C_V, C_P):
    """1/kappa with the legacy walk over cells [0, Nz) (:309-330)."""
    for arr_name, kap_name, start, edge in (("den_Hydz", "kappa_Hy", P.pmlWidth - 2, P.pmlWidth - 2),
                                            ("den_Exdz", "kappa_Ex", P.pmlWidth - 1, P.pmlWidth - 1)):
        arr, kap = getattr(C_V, arr_name), getattr(C_V, kap_name)
        jj = start
        for j in range(0, P.Nz):
            if j <= edge:
                arr[j] = 1 / (kap[j])
            elif j >= P.Nz + 2 - P.pmlWidth:
                arr[j] = 1 / (kap[jj])
                jj -= 1
            else:
                arr[j] = 1 / (1)
    return C_V.den_Exdz, C_V.den_Hydz


# ---- per-step functions, one GPU launch each ---------------------------------------------------
def CPML_Psi_e_Update(V, P, C_V, C_P):
    """psi_Ex = beX psi_Ex + ceX (Hy[k] - Hy[k-1]); Ex += Cb psi_Ex over [1, Nz-1) (:334-339)."""
    _psi(C_V.psi_Ex, V.Ex, V.Hy, C_V.beX, C_V.ceX, C_V.Cb, 1, P.Nz - 1, 0, -1, 1.0)
    return C_V.psi_Ex, V.Ex


def CPML_Psi_m_Update(V, P, C_V, C_P):
    """psi_Hy = bmY psi_Hy + cmY (Ex[k] - Ex[k+1]); Hy += C2 psi_Hy over [0, Nz-2) (:342-347)."""
    _psi(C_V.psi_Hy, V.Hy, V.Ex, C_V.bmY, C_V.cmY, C_V.C2, 0, P.Nz - 2, 0, 1, 1.0)
    return C_V.psi_Hy, V.Hy


def CPML_HyUpdate(V, P, C_V, C_P):
    """Hy = Hy UpHySelf + (Ex[k+1] - Ex[k]) UpHyMat UpHyEcompsCo over [0, Nz-2) (:351-354)."""
    from ..stepops import MUL
    _curl(V.Hy, V.Ex, 0, P.Nz - 2, 1, 0, ((MUL, V.UpHyMat), (MUL, V.UpHyEcompsCo)),
          self_=V.UpHySelf)
    return V.Hy


def CPML_ExUpdate(V, P, C_V, C_P):
    """Ex = Ex UpExSelf + (Hy[k] - Hy[k-1]) UpExHcompsCo UpExMat over [1, Nz-1) (:357-360)."""
    from ..stepops import MUL
    _curl(V.Ex, V.Hy, 1, P.Nz - 1, 0, -1, ((MUL, V.UpExHcompsCo), (MUL, V.UpExMat)),
          self_=V.UpExSelf)
    return V.Ex


def CPML_PEC(V, P, C_V, C_P):
    """Ex[0] = 0 (:363-365)."""
    V.Ex[0] = 0
    return V.Ex[0], V.Ex[P.Nz - 1]


def CPML_PMC(V, P, C_V, C_P):
    """Hy[Nz-1] = 0 (:367-369)."""
    V.Hy[P.Nz - 1] = 0
    return V.Hy[P.Nz - 1]


def ADE_TempPolCurr(V, P):
    """P_(n-2) <- P_(n-1), P_(n-1) <- P over cells [1, Nz-1), cell by cell (:371-375); host
    copies."""
    k = slice(1, P.Nz - 1)
    V.tempTempVarPol[k] = V.tempVarPol[k]
    V.tempVarPol[k] = V.polarisationCurr[k]
    return V.tempTempVarPol, V.tempVarPol


def ADE_PolarisationCurrent_Ex(V, P, C_V, C_P):
    """P = A P_(n-1) + B P_(n-2) + C Ex over [front-1, rear) (:378-389)."""
    from .. import stepops as so
    D = (1 / P.delT ** 2) + (V.gammaE / (2 * P.delT))
    A = ((2 / P.delT ** 2) - V.omega_0E ** 2) / D
    B = ((V.gammaE / (2 * P.delT)) - 1 / P.delT ** 2) / D
    C = (P.permit_0 * (V.plasmaFreqE ** 2)) / D
    so.run(so.make_op(so.OP_POL, int(P.materialFrontEdge - 1), int(P.materialRearEdge),
                      s=(A, B, C, 0.0)),
           [V.polarisationCurr, V.tempVarPol, V.tempTempVarPol, V.Ex, None, None, None, None],
           (0,))
    return V.polarisationCurr


def ADE_HyUpdate(V, P, C_V, C_P):
    """Hy = Hy UpHySelf + (Ex[k+1] - Ex[k]) UpHyMat over [1, Nz-1) (:392-395)."""
    from ..stepops import MUL
    _curl(V.Hy, V.Ex, 1, P.Nz - 1, 1, 0, ((MUL, V.UpHyMat),), self_=V.UpHySelf)
    return V.Hy


def ADE_MyUpdate():
    pass


def ADE_ExUpdate(V, P, C_V, C_P):
    """Ex = UpExSelf Ex + (Hy[k] - Hy[k-1]) UpExMat over [1, front-1), then, when the slab ends
    before Nz-1, over [rear-1, Nz) (:401-410)."""
    from ..stepops import MUL
    _curl(V.Ex, V.Hy, 1, int(P.materialFrontEdge - 1), 0, -1, ((MUL, V.UpExMat),),
          self_=V.UpExSelf)
    if P.materialRearEdge < P.Nz - 1:
        _curl(V.Ex, V.Hy, int(P.materialRearEdge - 1), P.Nz, 0, -1, ((MUL, V.UpExMat),),
              self_=V.UpExSelf)
    return V.Ex


def ADE_ExCreate(V, P, C_V, C_P):
    """Ex = (Dx - P) / permit_0 over [front-1, rear) (:413-416)."""
    from .. import stepops as so
    so.run(so.make_op(so.OP_EXCREATE, int(P.materialFrontEdge - 1), int(P.materialRearEdge),
                      s=(P.permit_0, 0.0, 0.0, 0.0)),
           [V.Ex, V.Dx, V.polarisationCurr, None, None, None, None, None], (0,))
    return V.Ex


def ADE_DxUpdate(V, P, C_V, C_P):
    """Dx += (Hy[k] - Hy[k-1]) delT / dz, then Ex = (Dx - P) / permit_0, over [front-1, rear)
    (:418-423)."""
    from ..stepops import DIV, MUL
    lo, hi = int(P.materialFrontEdge - 1), int(P.materialRearEdge)
    _curl(V.Dx, V.Hy, lo, hi, 0, -1, ((MUL, P.delT), (DIV, P.dz)))
    ADE_ExCreate(V, P, C_V, C_P)
    return V.Dx, V.Ex


def ADE_NonLinMyUpdate():
    pass


def ADE_NonLinPxUpdate():
    pass


def SpatialFiltering():
    pass


def SymbolicRegression():
    pass
