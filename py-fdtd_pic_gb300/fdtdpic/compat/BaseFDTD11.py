"""Set-up functions of BaseFDTD11.py that the integrators call once per run.

The per-step update functions (ADE_ExUpdate, CPML_Psi_e_Update, AcubicFinder, ...) have no
separate entry points here: the GPU kernels fuse a whole step (and many steps) into one launch,
so the unit of work is an integrator call (:mod:`Solver_Engine`).
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
