"""Set-up on the device for ragged batches (``fdtdpic_setup_batch`` in the C ABI).

The host restatement of the reference's per-grid set-up (:mod:`fdtdpic.physics_setup`) costs
about a quarter of a millisecond of Python per grid -- about a second for a 4096-grid sweep,
as long as the sweep's whole GPU run.  Here the geometry of a whole batch is laid out with numpy
array operations (no per-grid objects), the plasma-frequency correction of
``genericStability.spatialStab`` (genericStability.py:12-62) is evaluated for all grids at once,
and one kernel writes every grid's CPML table and update, Kerr and Lorentz coefficients
(boundCondManager, Solver_Engine.py:70-87; BaseFDTD11.py:124-182, 223-357, 487-538, 795-820).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import physics_setup as ps
from ._lib import (INSTANCE_DTYPE, MODE_FREESPACE, MODE_KERR, MODE_LINLOR, SETUP_DTYPE,
                   STATE_ARRAYS, TAB_ROWS, check, lib)
from .engine import Packed, _dtype, _ptr, _require_cuda


@dataclass
class GridShape:
    """What the batch engine needs of a grid that exists only as a descriptor row."""
    nz: int
    n_steps: int
    front: int
    rear: int
    mode: int
    step_begin: int = 0
    step_end: int = -1

    def __post_init__(self):
        if self.step_end < 0:
            self.step_end = self.n_steps

    @property
    def n(self):
        return self.nz + 1

    def cost(self) -> float:
        """Relative work of one run (as fdtdpic.grid.Grid.cost)."""
        slab = max(0, self.rear - self.front)
        w = 12.0 if self.mode == MODE_KERR else (2.0 if self.mode == MODE_LINLOR else 0.0)
        return (self.step_end - self.step_begin) * (self.nz + w * slab)


def spatial_stab_batch(full_time, full_space, space_step, frequency, time_step, plasma_freq,
                       resonant_freq, gamma):
    """:func:`fdtdpic.physics_setup.spatial_stab` for arrays of grids (full_space, plasma_freq,
    resonant_freq, gamma per grid): the corrected plasma frequencies, element for element the
    scalar function's values; exits as the reference does when any grid fails a check."""
    full_space = np.asarray(full_space, np.float64)
    pf = np.asarray(plasma_freq, np.float64)
    rf = np.asarray(resonant_freq, np.float64)
    gam = np.asarray(gamma, np.float64) * np.ones_like(pf)
    sp, frq, tim = space_step, frequency, time_step
    rad = 2 * np.pi * frq
    if rad * tim > np.pi / 2 and frq <= 5e9:
        ps._exit(f"unstable timestep {rad * tim} {tim}")
    sw = np.sinc(np.pi * frq * tim)
    # squares as the scalar function forms them: ** 2 of a Python float (the sweep's resonant
    # frequencies) or of a numpy scalar (its plasma frequencies) is libm's pow, not always x * x
    # to the last place as the array square is
    rf2 = np.array([float(v) ** 2 for v in rf])
    pf2 = np.array([np.float64(v) ** 2 for v in pf])
    es = pf2 / rf2 - 1
    damp = 1.0j * gam * rad * sw
    base = rad ** 2 * sw ** 2
    ratio = (base - es * rf2 * np.cos(rad * tim) + damp) / (base - rf2 * np.cos(rad * tim) + damp)
    # abs() of each complex value as a numpy scalar: numpy's array absolute takes another
    # hypot than its scalar one, and the scalar function's values are the reference here
    k_num = np.array([abs(v) for v in
                      (2 / sp) * np.arcsin((rad / ps.C0) * (sp / 2) * sw * np.sqrt(ratio))])
    eps = 1 + (pf2 / (rf2 - (rad ** 2) - 1j * gam * rad))
    refr = np.sqrt(abs(np.real(eps)))
    fix = (ps.C0 * tim * np.sin((k_num * refr * sp) / 2)) / (refr * sp * np.sin((k_num * ps.C0 * tim) / 2))
    pf_new = np.sqrt(abs(fix)) * pf
    lam_disc = (rad / frq) / k_num
    bad = k_num * sp > (np.pi) / 2
    if np.any(bad):
        ps._exit(f"unstable, wave is not resolved: {(k_num * sp)[bad][0]}")
    small = k_num * sp * full_space < (5 * lam_disc)
    if np.any(small):
        ps._exit(f"unstable because domain too small, {((lam_disc * 5) / sp)[small][0]}")
    return pf_new


def setup_records(n, *, dz, dt, courant, eps0, mu0, plasma_freq, omega0, gamma, chi3,
                  alpha3=ps.f32(0.7), freq_in=1e9, kappa_max=1.0, alpha_max=ps.f32(0.05),
                  r_scale=4.0, r_a_scale=1.0, sigma_opt=None, char_imp=ps.CHAR_IMP, eps_re=1.0,
                  mu_re=1.0, free_space=False) -> np.ndarray:
    """The FdtdSetup rows of n grids (scalars broadcast, arrays per grid)."""
    rec = np.zeros(n, SETUP_DTYPE)
    vals = dict(dz=dz, dt=dt, courant=courant, eps0=eps0, mu0=mu0, char_imp=char_imp,
                eps_re=eps_re, mu_re=mu_re, kappa_max=kappa_max,
                sigma_opt=ps.sigma_opt(dz, eps0, mu0) if sigma_opt is None else sigma_opt,
                alpha_max=alpha_max, r_scale=r_scale, r_a_scale=r_a_scale,
                plasma_freq=plasma_freq, omega0=omega0, gamma=gamma, chi3=chi3, alpha3=alpha3,
                freq_in=freq_in)
    for k, v in vals.items():
        rec[k] = v
    rec["free_space"] = 1 if free_space else 0
    return rec


def run_setup(desc: np.ndarray, records: np.ndarray, device=None, stream=None):
    """Device copies of the descriptors with their coefficient fields filled, and the PML table
    pool (pml_offset of each descriptor indexes it), from fdtdpic_setup_batch enqueued on
    ``stream`` (default: torch's current stream): they are ready on that stream."""
    _require_cuda()
    L = lib()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    n = len(desc)
    n_tab = int((TAB_ROWS * (2 * desc["pml"].astype(np.int64) + 1)).sum()) if n else 0
    d_desc = torch.from_numpy(np.ascontiguousarray(desc).view(np.uint8).copy()).to(dev)
    d_rec = torch.from_numpy(np.ascontiguousarray(records).view(np.uint8).copy()).to(dev)
    d_tab = torch.empty(max(1, n_tab), dtype=torch.float64, device=dev)
    st = ctypes.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    check(L.fdtdpic_setup_batch(n, _ptr(d_rec), _ptr(d_desc), _ptr(d_tab), st),
          "fdtdpic_setup_batch")
    return d_desc, d_tab


def sweep_layout(spec, eps0=None, mu0=None, mode=MODE_KERR):
    """Host part of :func:`sweep_batch`, numpy only: the batch's descriptors (geometry and
    offsets; coefficient fields left zero), FdtdSetup rows, source pool, shapes and dt, laid
    out as :func:`fdtdpic.grid.pack` lays out :func:`fdtdpic.sweep.make_sweep_grids`."""
    import scipy.constants as sc_const

    from .sweep import DZ, SC, sweep_parameters
    eps0 = sc_const.epsilon_0 if eps0 is None else eps0
    mu0 = sc_const.mu_0 if mu0 is None else mu0
    params = sweep_parameters(spec)
    n = len(params)
    nz = np.array([p["nz"] for p in params], np.int64)
    front = np.array([p["front"] for p in params], np.int64)
    rear = np.array([p["rear"] for p in params], np.int64)
    d_eps = np.array([p["d_eps"] for p in params])
    f0 = np.array([p["f0"] for p in params])
    chi3 = np.array([p["chi3"] for p in params])
    T = spec.n_steps
    dt = SC * DZ / ps.C0
    gamma = 2 * np.pi * 0.1e9
    w0 = 2 * np.pi * f0
    pf = spatial_stab_batch(T, nz, DZ, spec.freq_in, dt, np.sqrt(d_eps) * w0, w0, gamma)

    desc = np.zeros(n, INSTANCE_DTYPE)
    desc["nz"], desc["n_steps"], desc["step_begin"], desc["step_end"] = nz, T, 0, T
    desc["pml"], desc["cpml_lo"], desc["cpml_hi"] = spec.pml, 1, 1
    desc["front"], desc["rear"], desc["nzsrc"] = front, rear, spec.nzsrc
    desc["mode"] = mode
    desc["pol_active"] = 1 if mode == MODE_LINLOR else 0
    desc["probe_cell"][:, 0], desc["probe_cell"][:, 1] = 50, nz - 50
    desc["probe_lo"] = 0
    desc["probe_hi"] = T - 1
    per_tab = TAB_ROWS * (2 * spec.pml + 1)
    desc["pml_offset"] = np.arange(n, dtype=np.int64) * per_tab
    desc["src_offset"], desc["srcs_offset"] = 0, 2 * T
    desc["probe_offset"] = np.arange(n, dtype=np.int64) * 2 * T
    sizes = STATE_ARRAYS * (nz + 1)
    desc["state_offset"] = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    courant = ps.f32(SC)
    rec = setup_records(n, dz=DZ, dt=dt, courant=courant, eps0=eps0, mu0=mu0, plasma_freq=pf,
                        omega0=w0, gamma=gamma, chi3=chi3, freq_in=spec.freq_in,
                        free_space=mode == MODE_FREESPACE)
    exs = ps.gauss_sine(T, spec.freq_in, dt)
    hys = np.zeros(T)
    src = np.concatenate([exs, hys, exs / float(courant), hys / float(courant)])
    shapes = [GridShape(int(nz[i]), T, int(front[i]), int(rear[i]), mode) for i in range(n)]
    return dict(desc=desc, records=rec, src=src, shapes=shapes, dt=dt,
                n_state=int(sizes.sum()), n_probe=2 * T * n)


def sweep_batch(spec, precision="f32", eps0=None, mu0=None, mode=MODE_KERR, device=None):
    """The seeded sweep batch of :func:`fdtdpic.sweep.make_sweep_grids`, set up on the device:
    returns (Packed, dt) ready for :class:`fdtdpic.sweep.Sweep` (``packed=``)."""
    _require_cuda()
    L = lib()
    prec, tdt = _dtype(precision)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    lay = sweep_layout(spec, eps0, mu0, mode)
    d_desc, d_tab = run_setup(lay["desc"], lay["records"], dev)
    # host copy of the completed descriptors (the engine reads geometry and coefficients there)
    desc_full = d_desc.cpu().numpy().view(INSTANCE_DTYPE).copy()
    shapes = lay["shapes"]
    n = len(shapes)
    smem = np.array([L.fdtd1d_resident_smem_bytes(desc_full[i:i + 1].ctypes.data, prec)
                     for i in range(n)], np.int64)
    resident = [i for i in range(n) if smem[i] > 0]
    global_idx = [i for i in range(n) if smem[i] == 0]
    order = sorted(resident, key=lambda i: -shapes[i].cost())
    packed = Packed(
        grids=shapes, prec=prec, tdtype=tdt, desc_host=desc_full, d_desc=d_desc, d_table=d_tab,
        d_src=torch.from_numpy(lay["src"]).to(dev),
        d_state=torch.zeros(max(1, lay["n_state"]), dtype=tdt, device=dev),
        d_probe=torch.zeros(max(1, lay["n_probe"]), dtype=tdt, device=dev), d_hist=None,
        d_queue=torch.zeros(1, dtype=torch.int32, device=dev),
        d_status=torch.zeros(n, dtype=torch.int32, device=dev),
        d_fallbacks=torch.zeros(n, dtype=torch.int32, device=dev), resident=resident,
        d_order=torch.tensor(order, dtype=torch.int32, device=dev) if order else None,
        smem_bytes=int(smem[resident].max()) if resident else 0, global_idx=global_idx)
    return packed, lay["dt"]
