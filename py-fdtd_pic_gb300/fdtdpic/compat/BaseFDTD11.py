"""Set-up functions of BaseFDTD11.py that the integrators call once per run, and the per-step
functions that no integrator calls.

The per-step update functions the integrators use (ADE_ExUpdate, CPML_Psi_e_Update,
AcubicFinder, ...) have no separate entry points here: the GPU kernels fuse a whole step (and
many steps) into one launch, so the unit of work is an integrator call (:mod:`Solver_Engine`).
The uncalled ones (MUR1DEx, ADE_JxUpdate and Varin's three ADE updates) are entry points of
their own, each one GPU launch over the state's arrays (:mod:`fdtdpic.variants`), for loops
that call them as the commented-out lines of Solver_Engine.py would.
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
