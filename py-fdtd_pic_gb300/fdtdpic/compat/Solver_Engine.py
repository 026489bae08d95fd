"""The reference's integrator entry points (Solver_Engine.py:142-371), stepped on the GPU.

``IntegratorFreeSpace1D``, ``IntegratorNL1D`` and ``IntegratorLinLor1D`` take
``(V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf)``, write their results into ``V`` and
``C_V`` as the reference does, and return its 8-tuple
``(Ex, Hy, Exs, Hys, psi_Ex, psi_Hy, x1ColBe, x1ColAf)``.  Members written: Ex, Hy, Dx,
polarisationCurr, Acubic, Port1/Port2 (Kerr), x1ColBe/x1ColAf (free space, Lorentz),
Ex_History, plasmaFreqE (the spatialStab rescale), UpExMat/UpHyMat (and for free space
epsilon, mu and the UpEx*/UpHy* material arrays), and C_V's psi_Ex, psi_Hy and CPML
coefficient arrays.

Each call runs in one of two GPU forms: grids that fit in shared memory in the resident batch
kernel, larger ones on the global-memory path.  Sources come from this module's
``SourceManager`` (looked up at call time, so it can be replaced as in the reference).

``prepare`` / ``run_prepared`` / ``finish_prepared`` split a call into host set-up, GPU
stepping and write-back, so that many calls can share one batched launch
(``MasterController.Controller_batch``, ``LoopedSim``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from types import SimpleNamespace

import numpy as np

from .. import engine
from .. import physics_setup as ps
from ..grid import CP_with, grids_from_reference
from . import BaseFDTD11

PRECISION = "f64"  # "f64": within 1e-12 of the reference; "f32": FP32 state


def SourceManager(V, P, C_V, C_P):
    """(Exs, Hys) for SineCont / Gaussian sources; ([], []) when neither is set (:89-124)."""
    ex, hy = ps.source_manager(P)
    if len(ex) == 0 and not (P.SineCont or P.Gaussian):
        return [], []
    return ex, hy


def SechArr(a):
    a = np.where(a > 50, 50, a)
    return 1 / np.cosh(a)


def Sig_Mod(V, P, sig, AmpCarr=1, AmpMod=1, tau=14.6e-10):
    """Sech-enveloped source (:133-140)."""
    return ps.sig_mod(P, np.asarray(sig, dtype=np.float64), AmpCarr, AmpMod, tau)


def _cpml_view(P, C_P):
    CP = SimpleNamespace(**{k: getattr(P, k) for k in (
        "Nz", "pmlWidth", "CPMLXp", "CPMLXm", "delT", "permit_0", "permea_0", "dz")})
    for k in ("kappaMax", "r_scale", "r_a_scale", "sigmaOpt", "alphaMax"):
        setattr(CP, k, getattr(C_P, k))
    return CP_with(CP, P)


def boundCondManager(V, P, C_V, C_P):
    """CPML coefficient arrays into C_V (:70-87; BaseFDTD11.py:223-357)."""
    arrays = ps.cpml_arrays(_cpml_view(P, C_P), P.CharImp * P.courantNo)
    for k, v in arrays.items():
        setattr(C_V, k, v)
    return C_V


@dataclass
class Prepared:
    name: str
    V: object
    P: object
    C_V: object
    C_P: object
    Exs: object
    Hys: object
    grids: list
    results: list = field(default_factory=list)


def _checked_sources(P, Exs, Hys, free_space):
    T = int(P.timeSteps)
    if free_space:
        tau = 1 / (P.freq_in / 5)
        Exs = Sig_Mod(None, P, Exs, tau=tau)
        Hys = Sig_Mod(None, P, Hys, AmpMod=1 / P.CharImp, tau=tau)
    ex = np.asarray(Exs, dtype=np.float64)
    hy = np.asarray(Hys, dtype=np.float64)
    # the reference indexes Exs[counts] every step and Hys[counts] with TF/SF on
    if ex.size < T:
        raise IndexError(f"source Exs has {ex.size} samples; the run indexes {T}")
    if P.TFSF and hy.size < T:
        raise IndexError(f"source Hys has {hy.size} samples; the TF/SF run indexes {T}")
    if hy.size < T:
        hy = np.zeros(T)
    return Exs, Hys, ex, hy


def prepare(name, V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf) -> Prepared:
    """Host part of one integrator call: checks, sources, coefficient arrays, grids."""
    if name not in ("IntegratorFreeSpace1D", "IntegratorNL1D", "IntegratorLinLor1D"):
        raise ValueError(f"unknown integrator {name!r}")
    if getattr(P, "atten", False):
        raise NotImplementedError("attenuation probes (P.atten) are not supported")
    BaseFDTD11.FieldInit(V, P)
    free_space = name == "IntegratorFreeSpace1D"
    if free_space:
        BaseFDTD11.EmptySpaceCalc(V, P)
        (V.epsilon, V.mu, V.UpExHcompsCo, V.UpExSelf, V.UpHyEcompsCo,
         V.UpHySelf) = BaseFDTD11.Material(V, P)
        V.UpHyMat, V.UpExMat = BaseFDTD11.UpdateCoef(V, P)
    else:
        V.UpHyMat, V.UpExMat = BaseFDTD11.EmptySpaceCalc(V, P)
    BaseFDTD11.CPML_FieldInit(V, P, C_V, C_P)
    boundCondManager(V, P, C_V, C_P)
    Exs, Hys = SourceManager(V, P, C_V, C_P)
    Exs, Hys, ex, hy = _checked_sources(P, Exs, Hys, free_space)
    grids = grids_from_reference(P, V, C_P, name, Exs=ex, Hys=hy, hist=True,
                                 probe_finish_be=probeReadFinishBe,
                                 probe_start_af=probeReadStartAf)
    rows = int(np.shape(V.Ex_History)[0]) if np.ndim(V.Ex_History) == 2 else 0
    for g in grids:
        if g.hist_rows:
            g.hist_rows = rows
            if rows == 0:
                g.hist_interval = 0
    return Prepared(name, V, P, C_V, C_P, Exs, Hys, grids)


def run_prepared(jobs):
    """Step every grid of every prepared call in one batched GPU run."""
    all_grids = [g for j in jobs for g in j.grids]
    if not all_grids:
        return
    res = engine.run(all_grids, PRECISION)
    i = 0
    for j in jobs:
        j.results = res[i:i + len(j.grids)]
        i += len(j.grids)
    for j in jobs:
        for r in j.results:
            if r.status & 1:
                print("warning: non-finite field values at the end of the run")


def finish_prepared(job: Prepared):
    """Write a prepared call's results into V / C_V; returns the reference's 8-tuple."""
    V, C_V = job.V, job.C_V
    last = job.results[-1]
    V.Ex, V.Hy, V.Dx = last.Ex, last.Hy, last.Dx
    C_V.psi_Ex, C_V.psi_Hy = last.psi_Ex, last.psi_Hy
    if job.name == "IntegratorLinLor1D":
        V.polarisationCurr = last.P
        V.x1ColBe = job.results[0].probes[:, 0].copy()
        V.x1ColAf = last.probes[:, 1].copy()
    elif job.name == "IntegratorFreeSpace1D":
        V.x1ColBe = last.probes[:, 0].copy()
        V.x1ColAf = last.probes[:, 1].copy()
    else:
        V.Acubic = last.Acubic
        V.Port1 = last.probes[:, 0].copy()
        V.Port2 = last.probes[:, 1].copy()
    if last.hist is not None:
        V.Ex_History = last.hist
    return V.Ex, V.Hy, job.Exs, job.Hys, C_V.psi_Ex, C_V.psi_Hy, V.x1ColBe, V.x1ColAf


def _integrate(name, V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf):
    job = prepare(name, V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf)
    run_prepared([job])
    return finish_prepared(job)


def IntegratorFreeSpace1D(V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf):
    """Free space, two identical passes (:142-215): x1ColBe from the first (steps up to
    probeReadFinishBe), x1ColAf and Ex_History from the second (steps from probeReadStartAf)."""
    return _integrate("IntegratorFreeSpace1D", V, P, C_V, C_P, probeReadFinishBe,
                      probeReadStartAf)


def IntegratorNL1D(V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf):
    """Kerr slab, one pass (:220-271): Port1/Port2 at the slab edges every step."""
    return _integrate("IntegratorNL1D", V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf)


def IntegratorLinLor1D(V, P, C_V, C_P, probeReadFinishBe, probeReadStartAf):
    """Lorentz slab, two passes (:275-371): pass 0 without polarisation (x1ColBe), pass 1
    with the ADE polarisation (x1ColAf, Ex_History)."""
    return _integrate("IntegratorLinLor1D", V, P, C_V, C_P, probeReadFinishBe,
                      probeReadStartAf)
