"""Host description of one 1D grid ("instance") and its packing into the kernels' layout.

A :class:`Grid` is what one ``FdtdInstance`` (include/fdtdpic.h) describes: geometry, the
mode of the reference integrator it runs, its scalar coefficients, its PML table and its source
arrays.  :func:`grids_from_reference` builds the grids a reference integrator call needs from the
reference's own parameter objects (``Params``/``Variables``/``CPML_Params`` attribute names):

* ``IntegratorNL1D``        -> one Kerr grid, probes at materialFrontEdge / materialRearEdge
* ``IntegratorLinLor1D``    -> two grids, pass 0 (no polarisation) and pass 1 (Lorentz ADE)
* ``IntegratorFreeSpace1D`` -> one grid: its two passes are identical, so both probe windows
  (x1Loc for steps <= 0.7T, x2Loc for steps >= 0.05T) are sampled from the same run
"""
from __future__ import annotations

from dataclasses import dataclass, field
from types import SimpleNamespace

import numpy as np

from . import physics_setup as ps
from ._lib import (INSTANCE_DTYPE, MODE_FREESPACE, MODE_KERR, MODE_LINLOR, STATE_ARRAYS,
                   TAB_ROWS)

NO_PROBE = (0, 1, 0)  # (cell, lo, hi) with lo > hi: never sampled


@dataclass
class Grid:
    nz: int
    n_steps: int
    pml: int
    mode: int
    front: int
    rear: int
    nzsrc: int
    exs: np.ndarray
    hys: np.ndarray
    table: np.ndarray
    ue: float
    ue_slab: float
    uh: float
    uh_slab: float
    dtdz: float
    eps0: float
    sc: float
    cpml_lo: bool = True
    cpml_hi: bool = True
    tfsf: bool = False
    pol_active: bool = False
    pol: tuple = (0.0, 0.0, 0.0)
    kerr: tuple = (0.0, 0.0, 0.0, 0.0, 0.0)
    probes: tuple = (NO_PROBE, NO_PROBE)
    hist_interval: int = 0
    hist_rows: int = 0
    step_begin: int = 0
    step_end: int = -1
    resume: bool = False
    plasma_freq: float = 0.0
    tag: dict = field(default_factory=dict)

    def __post_init__(self):
        if self.step_end < 0:
            self.step_end = self.n_steps

    @property
    def n(self):
        return self.nz + 1

    def cost(self) -> float:
        """Relative work of one run (cell-steps, with Kerr slab cells weighted for the solve)."""
        slab = max(0, self.rear - self.front)
        w = 12.0 if self.mode == MODE_KERR else (2.0 if self.mode == MODE_LINLOR else 0.0)
        return (self.step_end - self.step_begin) * (self.nz + w * slab)

    def descriptor(self) -> np.ndarray:
        d = np.zeros((), INSTANCE_DTYPE)
        d["srcs_offset"] = -1  # set by pack() with the precomputed quotients
        d["nz"], d["n_steps"] = self.nz, self.n_steps
        d["step_begin"], d["step_end"] = self.step_begin, self.step_end
        d["pml"], d["cpml_lo"], d["cpml_hi"] = self.pml, int(self.cpml_lo), int(self.cpml_hi)
        d["front"], d["rear"], d["nzsrc"] = self.front, self.rear, self.nzsrc
        d["tfsf"], d["mode"], d["pol_active"] = int(self.tfsf), self.mode, int(self.pol_active)
        d["resume"] = int(self.resume)
        d["hist_interval"], d["hist_rows"] = self.hist_interval, self.hist_rows
        for p, (cell, lo, hi) in enumerate(self.probes):
            d["probe_cell"][p], d["probe_lo"][p], d["probe_hi"][p] = cell, lo, hi
        d["ue"], d["ue_slab"], d["uh"], d["uh_slab"] = self.ue, self.ue_slab, self.uh, self.uh_slab
        d["dtdz"], d["eps0"], d["sc"] = self.dtdz, self.eps0, self.sc
        d["pol_a"], d["pol_b"], d["pol_c"] = self.pol
        (d["kerr_a"], d["kerr_b"], d["kerr_c"], d["nl_e0"], d["nl_e0chi"]) = self.kerr
        return d


def _table_and_coef(P, free_space):
    ue, ue_slab, uh, uh_slab = ps.update_coefficients(P, free_space)
    arrays = ps.cpml_arrays(P, ue)
    return ps.pml_table(P, arrays), ue, ue_slab, uh, uh_slab


def grids_from_reference(P, V, C_P, integrator: str, Exs=None, Hys=None, hist=True,
                         probe_finish_be=None, probe_start_af=None):
    """The grid(s) one reference integrator call runs; ``Exs``/``Hys`` override SourceManager.
    ``probe_finish_be``/``probe_start_af`` are the integrators' probeReadFinishBe /
    probeReadStartAf arguments (default: Controller's int(0.7 T) and int(0.05 T)).

    V.plasmaFreqE is updated as the reference's integrators update it (spatialStab rescale:
    once for the Kerr integrator, once per pass -- compounding -- for the Lorentz one)."""
    T = int(P.timeSteps)
    user_src = Exs is not None
    common = dict(nz=int(P.Nz), n_steps=T, pml=int(P.pmlWidth), front=int(P.materialFrontEdge),
                  rear=int(P.materialRearEdge), nzsrc=int(P.nzsrc),
                  dtdz=P.delT / (P.dz), eps0=P.permit_0, sc=P.courantNo,
                  cpml_lo=bool(P.CPMLXm), cpml_hi=bool(P.CPMLXp), tfsf=bool(P.TFSF))
    CP = SimpleNamespace(**{k: getattr(P, k) for k in (
        "Nz", "pmlWidth", "CPMLXp", "CPMLXm", "delT", "permit_0", "permea_0", "dz")})
    for k in ("kappaMax", "r_scale", "r_a_scale", "sigmaOpt", "alphaMax"):
        setattr(CP, k, getattr(C_P, k))
    n_hist = int(T / P.vidInterval) if hist and P.vidInterval > 0 else 0
    fin_be = int(T * 0.7) if probe_finish_be is None else int(probe_finish_be)
    st_af = int(T * 0.05) if probe_start_af is None else int(probe_start_af)

    if integrator == "IntegratorNL1D":
        table, ue, ue_s, uh, uh_s = _table_and_coef(CP_with(CP, P), False)
        pf = ps.spatial_stab(T, P.Nz, P.dz, P.freq_in, P.delT, V.plasmaFreqE, V.omega_0E,
                             V.gammaE)[3]
        V.plasmaFreqE = pf
        if not user_src:
            Exs, Hys = ps.source_manager(P)
        g = Grid(mode=MODE_KERR, exs=_arr(Exs, T), hys=_arr(Hys, T), table=table, ue=ue,
                 ue_slab=ue_s, uh=uh, uh_slab=uh_s,
                 kerr=ps.kerr_coefficients(P, V, pf),
                 probes=((int(P.materialFrontEdge), 0, T - 1), (int(P.materialRearEdge), 0, T - 1)),
                 hist_interval=int(P.vidInterval) if n_hist else 0, hist_rows=n_hist,
                 plasma_freq=float(pf), **common)
        return [g]

    if integrator == "IntegratorLinLor1D":
        grids = []
        for i in (0, 1):
            table, ue, ue_s, uh, uh_s = _table_and_coef(CP_with(CP, P), False)
            pf = ps.spatial_stab(T, P.Nz, P.dz, P.freq_in, P.delT, V.plasmaFreqE, V.omega_0E,
                                 V.gammaE)[3]
            V.plasmaFreqE = pf
            if not user_src:
                Exs, Hys = ps.source_manager(P)
            probes = (((int(P.x1Loc), 0, min(fin_be, T - 1)), NO_PROBE) if i == 0 else
                      (NO_PROBE, (int(P.x2Loc), st_af, T - 1)))
            grids.append(Grid(mode=MODE_LINLOR, exs=_arr(Exs, T), hys=_arr(Hys, T), table=table,
                              ue=ue, ue_slab=ue_s, uh=uh, uh_slab=uh_s, pol_active=(i == 1),
                              pol=ps.lorentz_coefficients(P, V, pf), probes=probes,
                              hist_interval=int(P.vidInterval) if (n_hist and i == 1) else 0,
                              hist_rows=n_hist if i == 1 else 0, plasma_freq=float(pf),
                              tag=dict(pass_index=i), **common))
        return grids

    if integrator == "IntegratorFreeSpace1D":
        table, ue, ue_s, uh, uh_s = _table_and_coef(CP_with(CP, P), True)
        if not user_src:
            Exs, Hys = ps.source_manager(P)
            tau = 1 / (P.freq_in / 5)
            Exs = ps.sig_mod(P, Exs, tau=tau)
            Hys = ps.sig_mod(P, Hys, AmpMod=1 / P.CharImp, tau=tau)
        g = Grid(mode=MODE_FREESPACE, exs=_arr(Exs, T), hys=_arr(Hys, T), table=table, ue=ue,
                 ue_slab=ue_s, uh=uh, uh_slab=uh_s,
                 probes=((int(P.x1Loc), 0, min(fin_be, T - 1)), (int(P.x2Loc), st_af, T - 1)),
                 hist_interval=int(P.vidInterval) if n_hist else 0, hist_rows=n_hist,
                 plasma_freq=float(V.plasmaFreqE), **common)
        return [g]
    raise ValueError(f"unknown integrator {integrator!r}")


def CP_with(CP, P):
    """The attribute view cpml_arrays needs (Params fields + CPML_Params fields)."""
    CP.courantNo, CP.CharImp = P.courantNo, P.CharImp
    CP.epsRe, CP.muRe = getattr(P, "epsRe", 1.0), getattr(P, "muRe", 1.0)
    return CP


def _arr(a, T):
    a = np.asarray(a, dtype=np.float64)
    if a.size == 0:
        return np.zeros(T)
    if a.size < T:
        raise ValueError(f"source array has {a.size} samples, the run needs {T}")
    return a


# ------------------------------------------------------------------------------------------
# synthetic workloads (the configurations the benchmarks and tests use)
# ------------------------------------------------------------------------------------------
def lorentz_kerr_grid(nz, n_steps, *, dz=0.015, sc=0.5, front, rear, pml=20, nzsrc=100,
                      probes=(50, 950), d_eps=2.0, f0=1.5e9, gamma=2 * np.pi * 0.1e9,
                      chi3=1e-2, freq_in=1e9, mode=MODE_KERR, source=None, eps0=None, mu0=None,
                      apply_stab=True, pol_active=True):
    """A grid of the synthetic workloads: Lorentz slab [front, rear) (Kerr or Lorentz ADE),
    Gaussian-modulated soft source at nzsrc, PML pml cells, probes sampled every step."""
    import scipy.constants as sc_const
    eps0 = sc_const.epsilon_0 if eps0 is None else eps0
    mu0 = sc_const.mu_0 if mu0 is None else mu0
    dt = sc * dz / ps.C0
    P = SimpleNamespace(Nz=nz, timeSteps=n_steps, dz=dz, delT=dt, courantNo=ps.f32(sc),
                        materialFrontEdge=front, materialRearEdge=rear, pmlWidth=pml,
                        nzsrc=nzsrc, freq_in=freq_in, permit_0=eps0, permea_0=mu0,
                        CharImp=ps.CHAR_IMP, c0=ps.C0, CPMLXm=True, CPMLXp=True, TFSF=False,
                        epsRe=1.0, muRe=1.0)
    C_P = SimpleNamespace(kappaMax=1.0, r_scale=4.0, r_a_scale=1.0,
                          sigmaOpt=ps.sigma_opt(dz, eps0, mu0), alphaMax=ps.f32(0.05))
    w0 = 2 * np.pi * f0
    V = SimpleNamespace(plasmaFreqE=np.sqrt(d_eps) * w0, omega_0E=w0, gammaE=gamma,
                        chi3Stat=chi3, alpha3=ps.f32(0.7))
    pf = V.plasmaFreqE
    if apply_stab:
        pf = ps.spatial_stab(n_steps, nz, dz, freq_in, dt, pf, w0, gamma)[3]
    CP = SimpleNamespace(**vars(C_P))
    for k in ("Nz", "pmlWidth", "CPMLXp", "CPMLXm", "delT", "permit_0", "permea_0", "dz"):
        setattr(CP, k, getattr(P, k))
    table, ue, ue_s, uh, uh_s = _table_and_coef(CP_with(CP, P), mode == MODE_FREESPACE)
    src = ps.gauss_sine(n_steps, freq_in, dt) if source is None else np.asarray(source, float)
    return Grid(nz=nz, n_steps=n_steps, pml=pml, mode=mode, front=front, rear=rear, nzsrc=nzsrc,
                exs=src, hys=np.zeros(n_steps), table=table, ue=ue, ue_slab=ue_s, uh=uh,
                uh_slab=uh_s, dtdz=dt / dz, eps0=eps0, sc=P.courantNo,
                pol_active=pol_active and mode == MODE_LINLOR,
                pol=ps.lorentz_coefficients(P, V, pf), kerr=ps.kerr_coefficients(P, V, pf),
                probes=((probes[0], 0, n_steps - 1), (probes[1], 0, n_steps - 1)),
                plasma_freq=float(pf))


def pack(grids, itemsize):
    """Descriptor array + coefficient table + source pool + buffer sizes for a batch."""
    desc = np.zeros(len(grids), INSTANCE_DTYPE)
    tabs, srcs = [], []
    src_index = {}
    off_tab = off_src = off_probe = off_state = off_hist = 0
    for i, g in enumerate(grids):
        d = g.descriptor()
        if g.table.shape != (TAB_ROWS, 2 * g.pml + 1):
            raise ValueError("PML table shape does not match pmlWidth")
        d["pml_offset"] = off_tab
        tabs.append(g.table.ravel())
        off_tab += g.table.size
        key = (id(g.exs), id(g.hys), g.n_steps, float(g.sc))
        if key not in src_index:
            src_index[key] = off_src
            exs = np.asarray(g.exs[:g.n_steps], np.float64)
            hys = np.asarray(g.hys[:g.n_steps], np.float64)
            # the per-step source values Exs[t]/Sc, Hys[t]/Sc (IEEE division: the same quotients
            # a kernel would form), so no kernel divides in FP64 on its critical path
            srcs += [exs, hys, exs / float(g.sc), hys / float(g.sc)]
            off_src += 4 * g.n_steps
        d["src_offset"] = src_index[key]
        d["srcs_offset"] = src_index[key] + 2 * g.n_steps
        d["probe_offset"] = off_probe
        off_probe += 2 * g.n_steps
        d["state_offset"] = off_state
        off_state += STATE_ARRAYS * g.n
        d["hist_offset"] = off_hist
        off_hist += g.hist_rows * g.n
        desc[i] = d
    return dict(desc=desc, table=np.concatenate(tabs) if tabs else np.zeros(1),
                src=np.concatenate(srcs) if srcs else np.zeros(1),
                n_probe=off_probe, n_state=off_state, n_hist=off_hist)
