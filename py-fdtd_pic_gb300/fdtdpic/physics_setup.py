"""One-off set-up of a grid, restated from the reference (runs once per run, on the host).

The time stepping itself runs on the GPU (``fdtdpic.engine``); this module turns the
reference's parameter objects into the per-grid scalars and PML coefficient table the kernels
read.  Each function names the reference code it follows (fraserac/Py-FDTD_PIC):

* :func:`update_coefficients`  EmptySpaceCalc / Material / UpdateCoef   BaseFDTD11.py:124-182
* :func:`cpml_arrays`          CPML_FieldInit .. denominators           BaseFDTD11.py:196-357
* :func:`spatial_stab`         genericStability.spatialStab             genericStability.py:12-62
* :func:`smooth_turn_on`, :func:`gaussian`, :func:`source_manager`, :func:`sig_mod`
                               BaseFDTD11.py:86-120, Solver_Engine.py:89-140
* :func:`kerr_coefficients`    AcubicFinder / NonLinExUpdate            BaseFDTD11.py:803-877
* :func:`lorentz_coefficients` ADE_PolarisationCurrent_Ex               BaseFDTD11.py:610-633
* :func:`env_setup`, :func:`mat_setup`  Environment_Setup.py:19-166, Material_Def.py:21-120

Where the reference calls ``sys.exit`` after printing a message, these raise ``SystemExit``
with that message (the same outcome for a script, catchable for a library caller).
"""
from __future__ import annotations

import math
import sys

import numpy as np

C0 = 299792458.0
CHAR_IMP = 376.730313668
TAB_ROWS = 8  # beX ceX Cb bmY cmY C2 den_Exdz den_Hydz


def _exit(msg):
    print(msg)
    sys.exit(msg)


def update_coefficients(P, free_space: bool):
    """(ue, ue_slab, uh, uh_slab): UpExMat/UpHyMat outside and inside the slab.

    The Kerr and Lorentz integrators use EmptySpaceCalc (uniform); the free-space integrator
    divides the slab by epsRe/muRe (Material + UpdateCoef)."""
    ue = P.CharImp * P.courantNo
    uh = (1 / P.CharImp) * P.courantNo
    if free_space:
        return ue, ue / P.epsRe, uh, uh / P.muRe
    return ue, ue, uh, uh


def cpml_arrays(P, ue: float, ue_h_comps: float = 1.0):
    """Full-length (Nz+1) CPML arrays exactly as boundCondManager leaves them.

    Quirks kept: the Hy profile arrays are the Ex ones (aliasing at BaseFDTD11.py:266-268);
    Cb and C2 stay 0 at index Nz+1-pml (the right-hand loops stop one short, :312, :326);
    den_Exdz/den_Hydz walk the kappa array with their own counters (:333-357)."""
    n = P.Nz + 1
    pml = P.pmlWidth
    out = {k: np.zeros(n) for k in ("beX", "ceX", "Cb", "bmY", "cmY", "C2")}
    out["den_Exdz"] = np.ones(n)
    out["den_Hydz"] = np.ones(n)
    if not (P.CPMLXp or P.CPMLXm) or pml <= 0:
        return out
    i = np.arange(pml)
    ramp = ((pml - i) / pml) ** P.r_scale
    kap_l = 1 + (P.kappaMax - 1) * ramp
    sig_l = P.sigmaOpt * ramp
    alp_l = P.alphaMax * ((i + 1) / pml) ** P.r_a_scale
    kappa = np.ones(n)
    sigma = np.zeros(n)
    alpha = np.zeros(n)
    for arr, left in ((kappa, kap_l), (sigma, sig_l), (alpha, alp_l)):
        arr[:pml] = left
        arr[n - pml:] = left[::-1]
    dt, e0 = P.delT, P.permit_0
    ends = np.r_[0:pml, n - pml:n]
    s, k, a = sigma[ends], kappa[ends], alpha[ends]
    b = np.exp(-((s * dt / (k * e0)) + ((a * dt) / e0)))
    out["beX"][ends] = b
    out["bmY"][ends] = b
    out["ceX"][ends] = (b - 1) * s / ((s * k + a * k * k))
    out["cmY"][ends] = (b - 1) * s / ((s * k + a * k * k) * P.dz)
    coef_cells = np.r_[0:pml, n - pml + 1:n]
    out["Cb"][coef_cells] = ue_h_comps * ue
    out["C2"][coef_cells] = dt / P.permea_0
    j = np.arange(n)
    right = j >= n - pml
    if P.CPMLXm:
        out["den_Hydz"][: pml + 1] = 1 / kappa[: pml + 1]
        out["den_Exdz"][: pml + 1] = 1 / kappa[: pml + 1]
    if P.CPMLXp:
        rj = j[right & ~((j <= pml) & bool(P.CPMLXm))]
        walk = np.arange(len(rj))  # the counter steps once per cell that takes this branch
        out["den_Hydz"][rj] = 1 / kappa[pml - walk]
        out["den_Exdz"][rj] = 1 / kappa[pml - 1 - walk]
    return out


def pml_table(P, arrays) -> np.ndarray:
    """(TAB_ROWS, 2*pml+1) table: columns 0..pml are cells 0..pml, the rest cells Nz+1-pml..Nz."""
    n = P.Nz + 1
    pml = P.pmlWidth
    cols = np.r_[0:pml + 1, n - pml:n]
    rows = ("beX", "ceX", "Cb", "bmY", "cmY", "C2", "den_Exdz", "den_Hydz")
    return np.stack([arrays[r][cols] for r in rows]).astype(np.float64)


def spatial_stab(fullTime, fullSpace, spaceStep, frequency, timeStep, plasmaFreq, resonantFreq,
                 gamma):
    """Numerical-dispersion correction of the plasma frequency; returns
    (lamCont, lamDisc, diff, plasmaFreq', fix)."""
    sp = spaceStep
    frq = frequency
    rad = 2 * np.pi * frq
    tim = timeStep
    if rad * tim > np.pi / 2 and frq <= 5e9:
        _exit(f"unstable timestep {rad * tim} {tim}")
    sw = np.sinc(np.pi * frq * tim)
    pf, rf, gam = plasmaFreq, resonantFreq, gamma
    es = (pf ** 2) / (rf ** 2) - 1
    damp = 1.0j * gam * rad * sw
    base = rad ** 2 * sw ** 2
    ratio = (base - es * rf ** 2 * np.cos(rad * tim) + damp) / (base - rf ** 2 * np.cos(rad * tim) + damp)
    k_num = abs((2 / sp) * np.arcsin((rad / C0) * (sp / 2) * sw * np.sqrt(ratio)))
    eps = 1 + ((((pf)) ** 2) / (rf ** 2 - (rad ** 2) - 1j * gam * rad))
    refr = np.sqrt(abs(np.real(eps)))
    fix = (C0 * tim * np.sin((k_num * refr * sp) / 2)) / (refr * sp * np.sin((k_num * C0 * tim) / 2))
    pf_new = np.sqrt(abs(fix)) * pf
    lam_cont = C0 / frq
    lam_disc = (rad / frq) / k_num
    if k_num * sp > (np.pi) / 2:
        _exit(f"unstable, wave is not resolved: {k_num * sp}")
    if k_num * sp * fullSpace < (5 * lam_disc):
        _exit(f"unstable because domain too small, {(lam_disc * 5) / sp}")
    return lam_cont, lam_disc, abs(lam_cont - lam_disc), pf_new, fix


def smooth_turn_on(P, tempfreq=0.0):
    """SineCont waveform pair (Exs, Hys) as lists: sin(2 pi/ppw * Sc * t), one step apart,
    switched off after Periods periods."""
    frq = tempfreq if tempfreq != 0 else P.freq_in
    ppw = P.c0 / (frq * P.dz)
    w = 2.0 * np.pi / ppw
    on_until = P.period * P.Periods
    ex, hy = [], []
    for t in range(P.timeSteps):
        if t * P.delT < on_until:
            ex.append(float(np.sin(w * (P.courantNo * t))))
            hy.append(float(np.sin(w * (P.courantNo * (t + 1)))))
        else:
            ex.append(0)
            hy.append(0)
    return ex, hy


def gaussian(P):
    t = np.arange(P.timeSteps)
    fc = 200
    tau = fc * 2.2
    arg = ((t - tau) * (t - tau)) / (fc * fc) * np.cos(2 * np.pi * P.freq_in * (t - tau))
    return P.Amplitude * (np.exp(-arg) * 2) / P.courantNo


def source_manager(P):
    """(Exs, Hys) of the SineCont / Gaussian sources; empty arrays when neither is set."""
    if P.SineCont:
        ex, hy = smooth_turn_on(P)
        pe, ph = np.zeros(P.timeSteps), np.zeros(P.timeSteps)
        if P.nonLinMed:
            pe, ph = smooth_turn_on(P, tempfreq=P.freq_in * 0.8)
            pe = np.asarray(pe) * P.courantNo
            ph = np.asarray(ph) * P.courantNo
            pe *= 0.1
            ph *= 0.01
        ex = np.asarray(ex) * P.courantNo + pe
        hy = np.asarray(hy) * P.courantNo + ph
        if P.TFSF:
            hy = hy * (1 / P.CharImp)
        return ex, hy
    if P.Gaussian:
        ex = gaussian(P)
        hy = gaussian(P) if P.TFSF else np.zeros(len(ex))
        return ex, hy
    return np.zeros(0), np.zeros(0)


def sig_mod(P, sig, AmpCarr=1, AmpMod=1, tau=14.6e-10):
    """Sech envelope (AmpMod + sig) * sech(2 pi t / tau), argument clipped at 50."""
    tr = np.arange(len(sig)) * (P.delT)
    a = 2 * np.pi * (1 / tau) * tr
    return (AmpMod + sig) * (1 / np.cosh(np.where(a > 50, 50, a)))


def gauss_sine(n_steps, f, dt, t0=200.0, sigma=60.0, amp=1.0):
    """Gaussian-modulated sine soft source used by the synthetic workloads:
    amp * exp(-((n-t0)/sigma)^2 / 2) * sin(2 pi f (n-t0) dt)."""
    n = np.arange(n_steps, dtype=np.float64)
    return amp * np.exp(-0.5 * ((n - t0) / sigma) ** 2) * np.sin(2.0 * np.pi * f * (n - t0) * dt)


def complex_eps(plasma_freq, omega0, gamma, freq):
    """Lorentz permittivity at freq as AcubicFinder builds it."""
    return 1 + (plasma_freq * plasma_freq) / (
        omega0 * omega0 - (2 * np.pi * freq * 2 * np.pi * freq) + 1j * gamma * 2 * np.pi * freq)


def kerr_coefficients(P, V, plasma_freq):
    """(cub, qua, one, eps0*Re(sqrt 1.2), eps0*chi3)."""
    eps = complex_eps(plasma_freq, V.omega_0E, V.gammaE, P.freq_in)
    cub = (V.alpha3 * V.chi3Stat) ** 2
    qua = 2 * np.real(V.alpha3 * eps * V.chi3Stat)
    one = np.abs(eps) ** 2
    return (float(cub), float(qua), float(one), float(P.permit_0 * np.real(np.sqrt(1.2))),
            float(P.permit_0 * V.chi3Stat))


def lorentz_coefficients(P, V, plasma_freq):
    """(A, B, C) of P_{n+1} = A P_n + B P_{n-1} + C E_n."""
    dt = P.delT
    D = (1 / dt ** 2) + (V.gammaE / (2 * dt))
    return (((2 / dt ** 2) - V.omega_0E ** 2) / D, ((V.gammaE / (2 * dt)) - 1 / dt ** 2) / D,
            (P.permit_0 * plasma_freq ** 2) / D)


def _bin_aligned_steps(freq_in, delT, minim, maxim):
    """The step-count search shared by envSetup and matSetup: the first N in [minim, maxim)
    with freq_in*N*delT an integer, else maxim-1 (the fall-through of the second loop)."""
    for N in range(minim, maxim):
        check = (freq_in * N) / (1 / delT)
        if int(check) - check == 0:
            return N, True
    return maxim - 1, False


def env_setup(newFreq_in, domainSize, minim=400, maxim=600, VExists=False, V=None, P=None,
              nonLinMed=False, LorMed=False):
    """Geometry of a run (Environment_Setup.envSetup); returns its 20-tuple."""
    freq_in = newFreq_in
    lamMin = C0 / freq_in
    if VExists:
        eps = complex_eps(V.plasmaFreqE, V.omega_0E, V.gammaE, P.freq_in)
        Nlam = int((200 if nonLinMed else 60) * (np.real(eps)) ** 1.05)
    else:
        Nlam = 350 if nonLinMed else 400
    dz = lamMin / Nlam
    delT = (dz / C0) * 0.95
    period = 1 / freq_in
    courantNo = (C0 * delT) / dz
    if courantNo > 3 or courantNo < 0:
        _exit(f"{courantNo} courantNo is unstable")
    pmlWidth = 6 * int(lamMin / dz)
    if pmlWidth >= 12000:
        _exit(f"pmlWidth too big {pmlWidth}")
    Nz = int((domainSize) / dz) + 2 * pmlWidth
    if minim == maxim:
        minim -= 1
    N, found = _bin_aligned_steps(freq_in, delT, minim, maxim)
    timeSteps = N if N >= minim else minim
    timeSteps += int(timeSteps * (Nlam / 200))
    if timeSteps >= 2 ** 15:
        _exit("timeSteps too large")
    nzsrcFromPml = int(0.05 / dz)
    if nzsrcFromPml >= Nz * 0.65:
        _exit(f"{nzsrcFromPml} src is too far into domain")
    nzsrc = nzsrcFromPml + pmlWidth
    if nzsrc - 10 <= pmlWidth:
        _exit("The probe for fft is in the PML region")
    dist = int(0.1 / dz)
    front = dist + pmlWidth
    rear = Nz - 1
    if rear - front < 10:
        _exit(f"{rear - front} width is too small or negative")
    if dist >= domainSize / dz:
        _exit("Material starts in CPML region")
    if front <= nzsrc:
        _exit("Source is inside material")
    return (Nz, timeSteps, 0, 0, 1.0, 1.0, 1.0, 1.0, front - 20, nzsrc - 100, front, rear,
            pmlWidth, nzsrc, lamMin, dz, delT, courantNo, period, Nlam)


def mat_setup(V, P, C_P, C_V, newFreq_in, domainSize, minim=400, maxim=800):
    """Older fixed-geometry set-up (Material_Def.matSetup); returns its 19-tuple."""
    freq_in = newFreq_in
    lamMin = (C0 / freq_in) * 0.1
    dz = lamMin / 20
    delT = 0.99 / (C0 * (1 / dz))
    courantNo = (C0 * delT) / dz
    if courantNo > 1 or courantNo < 0:
        _exit(f"{courantNo} courantNo is unstable")
    pmlWidth = 150
    Nz = 600 + 2 * pmlWidth
    timeSteps, _ = _bin_aligned_steps(freq_in, delT, minim, maxim)
    if timeSteps >= 10000:
        _exit("timeSteps too large")
    nzsrc = 100 + pmlWidth
    front = 300 + pmlWidth
    rear = Nz - pmlWidth - 1
    return (Nz, timeSteps, 0, 0, 1.0, 1.0, 1.0, 1.0, nzsrc + int((front - nzsrc) / 2),
            nzsrc - (100 + 10) + 50, front, rear, pmlWidth, nzsrc, lamMin, dz, delT, courantNo,
            1 / freq_in)


def f32(x):
    """float32 rounding of a jitclass float32 field (MasterController.py spec lists)."""
    return float(np.float32(x))


def sigma_opt(dz, permit_0, permea_0):
    return 0.5 * (0.8 * (1) / (dz * (permea_0 / permit_0) ** 0.5))


def safe_int(x):
    return int(math.floor(x)) if isinstance(x, float) else int(x)
