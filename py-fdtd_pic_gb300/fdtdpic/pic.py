"""Electron-beam PIC coupled to one grid, on the GPU (``fdtdpic_run`` in the C ABI).

The reference leaves its ``Jx`` hook (MasterController.py:93,159; BaseFDTD11.py:667) empty; this
module fills it with a beam of macroparticles.  Positions are an int32 cell plus a fraction in
[0, 1) (units of dz), momenta are u/c = gamma v / c.  See include/fdtdpic.h for the step.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import F64, ST, check, lib
from .engine import _dtype, _ptr, _require_cuda
from .grid import Grid, pack

C0 = 299792458.0
PATH_CELLS_INSIDE = 16  # FDTDPIC_PATH_CELLS_INSIDE
Q_E = -1.602176634e-19
M_E = 9.1093837139e-31


class FdtdPicTiming(ctypes.Structure):
    _fields_ = [("push_ms", ctypes.c_float), ("field_ms", ctypes.c_float),
                ("sort_ms", ctypes.c_float), ("steps", ctypes.c_int32),
                ("path", ctypes.c_int32)]


class PicBeam(ctypes.Structure):
    _fields_ = [("n_part", ctypes.c_int32), ("clo", ctypes.c_int32), ("chi", ctypes.c_int32),
                ("sort_every", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("path", ctypes.c_int32), ("kE", ctypes.c_double), ("kH", ctypes.c_double),
                ("sc", ctypes.c_double), ("kJ", ctypes.c_double), ("kJz", ctypes.c_double),
                ("jscale", ctypes.c_double)]


@dataclass
class Beam:
    """Host copy of a beam: (cell, frac, ux, uz, id) plus its domain and macro-weight."""
    cell: np.ndarray
    frac: np.ndarray
    ux: np.ndarray
    uz: np.ndarray
    id: np.ndarray
    clo: int
    chi: int
    weight: float  # electrons per unit area per macroparticle [m^-2]

    @property
    def n(self):
        return len(self.cell)


def make_beam(n_part, clo, chi, dz, density=1e14, v_mean=0.3, v_spread=0.003, seed=20261203,
              sort=True):
    """Seeded beam: positions uniform over cells [clo, chi), vz ~ N(v_mean c, v_spread c),
    vx = 0, equal weights giving ``density`` [m^-3]; sorted by position unless sort=False."""
    rng = np.random.Generator(np.random.PCG64(seed))
    zeta = clo + (chi - clo) * rng.random(n_part)
    vz = rng.normal(v_mean, v_spread, n_part)
    uz = vz / np.sqrt(1.0 - vz * vz)
    if sort:
        order = np.argsort(zeta, kind="stable")
        zeta, uz = zeta[order], uz[order]
    cell = np.floor(zeta).astype(np.int32)
    weight = density * (chi - clo) * dz / max(1, n_part)
    return Beam(cell=cell, frac=zeta - cell, ux=np.zeros(n_part), uz=uz.copy(),
                id=np.arange(n_part, dtype=np.int32), clo=int(clo), chi=int(chi), weight=weight)


def beam_constants(dz, dt, weight, mu0, q=Q_E, m=M_E):
    """(kE, kH, sc, kJ, kJz) of the Boris step and deposit, momentum in units of c."""
    return dict(kE=q * dt / (2.0 * m * C0), kH=-q * mu0 * dt / (2.0 * m), sc=C0 * dt / dz,
                kJ=q * weight * C0, kJz=q * weight * dz / dt)


PASS_PLAN_KEYS = ("steps", "halo", "tiles", "wmin", "wmax", "loaded", "particles_per_range",
                  "smem_one_tile", "smem_wrap_pair", "scratch_bytes")


def pass_plan(grid: Grid, beam: Beam, precision="f32", pass_steps=0, tile_cells=0,
              smem_optin=232448):
    """The tiling a ``PicRun(path="pass")`` takes, computed on the host for a device with
    ``smem_optin`` bytes of opt-in shared memory per CTA (GB300: 232,448): a dict of
    PASS_PLAN_KEYS, or None when the pass path does not apply (fdtdpic_pass_plan)."""
    L = lib()
    prec, _ = _dtype(precision)
    desc = pack([grid], 8 if prec == F64 else 4)["desc"]
    pb = PicBeam()
    pb.n_part, pb.clo, pb.chi = beam.n, beam.clo, beam.chi
    pb.sort_every, pb.chunk, pb.path = pass_steps, tile_cells, 3 | PATH_CELLS_INSIDE
    out = (ctypes.c_int64 * len(PASS_PLAN_KEYS))()
    n = L.fdtdpic_pass_plan(prec, desc.ctypes.data, ctypes.byref(pb), int(smem_optin), out,
                            len(PASS_PLAN_KEYS))
    if n < 0:
        return None
    return dict(zip(PASS_PLAN_KEYS, (int(v) for v in out[:n])))


@dataclass
class PicSnapshot:
    """Everything a :class:`PicRun` carries between calls, on the host (see PicRun.snapshot)."""
    step_done: int
    path: int
    state: torch.Tensor
    hyp: torch.Tensor
    jx: torch.Tensor
    jz: torch.Tensor
    probe: torch.Tensor
    status: torch.Tensor
    cell: torch.Tensor
    frac: torch.Tensor
    ux: torch.Tensor
    uz: torch.Tensor
    id: torch.Tensor

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in (
            self.state, self.hyp, self.jx, self.jz, self.probe, self.status, self.cell,
            self.frac, self.ux, self.uz, self.id))


class PicRun:
    """One grid plus a beam, resident on the GPU; ``step(n)`` advances n steps.

    path: "auto" (the streaming kernels: push, field and re-binning launches captured in CUDA
    graphs; measured faster than the persistent tiled kernel on GB300), "streaming", "tiled"
    (one cooperative launch for all steps; grids that tile over the SMs only) or "pass" (long
    grids: pass_steps whole steps per launch over tiles of about tile_cells cells held in shared
    memory; 0 for the library's defaults, 8 steps and 512 cells; beams inside their domain)."""

    def __init__(self, grid: Grid, beam: Beam, dz: float, dt: float, mu0: float,
                 precision="f32", sort_every=32, chunk=0, path="auto", device=None,
                 pass_steps=0, tile_cells=0):
        _require_cuda()
        self.L = lib()
        self.prec, self.tdt = _dtype(precision)
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.dev = dev
        self.grid = grid
        g = grid
        pk = pack([g], 8 if self.prec == F64 else 4)
        self.desc = pk["desc"]
        self.d_desc = torch.from_numpy(self.desc.view(np.uint8).copy()).to(dev)
        self.d_table = torch.from_numpy(pk["table"]).to(dev)
        self.d_src = torch.from_numpy(pk["src"]).to(dev)
        self.d_state = torch.zeros(pk["n_state"], dtype=self.tdt, device=dev)
        self.d_probe = torch.zeros(pk["n_probe"], dtype=self.tdt, device=dev)
        n = g.nz + 1
        self.d_hyp = torch.zeros(n, dtype=self.tdt, device=dev)
        self.d_jx = torch.zeros(n, dtype=self.tdt, device=dev)
        self.d_jz = torch.zeros(n, dtype=self.tdt, device=dev)
        self.d_status = torch.zeros(2, dtype=torch.int32, device=dev)
        self.beam = beam
        self.d_cell = torch.from_numpy(np.ascontiguousarray(beam.cell, np.int32)).to(dev)
        self.d_frac = torch.from_numpy(np.ascontiguousarray(beam.frac)).to(dev, self.tdt)
        self.d_ux = torch.from_numpy(np.ascontiguousarray(beam.ux)).to(dev, self.tdt)
        self.d_uz = torch.from_numpy(np.ascontiguousarray(beam.uz)).to(dev, self.tdt)
        self.d_id = torch.from_numpy(np.ascontiguousarray(beam.id, np.int32)).to(dev)
        self.pb = PicBeam()
        self.pb.n_part, self.pb.clo, self.pb.chi = beam.n, beam.clo, beam.chi
        self.pb.sort_every, self.pb.chunk = sort_every, chunk
        if path == "pass":  # the pass path reads these two fields as its pass length and tiles
            self.pb.sort_every, self.pb.chunk = pass_steps, tile_cells
        self.constants = beam_constants(dz, dt, beam.weight, mu0)
        for name, v in self.constants.items():
            setattr(self.pb, name, v)
        self.pb.jscale = self.L.fdtdpic_pic_jscale(ctypes.byref(self.pb))
        self.path_mode = {"auto": 0, "streaming": 1, "tiled": 2, "pass": 3}[path]
        self._set_inside(beam)
        self.scratch_bytes = int(self.L.fdtdpic_pic_scratch_bytes(
            self.prec, self.desc.ctypes.data, ctypes.byref(self.pb)))
        self.d_scratch = torch.zeros(max(1, self.scratch_bytes), dtype=torch.uint8, device=dev)
        self.step_done = 0

    def _set_inside(self, beam):
        # FDTDPIC_PATH_CELLS_INSIDE when every initial cell lies in the beam domain (the wrap
        # keeps it there), which lets the streaming path overlap each step's H phase with the
        # next push
        c = np.asarray(beam.cell)
        inside = c.size == 0 or (int(c.min()) >= beam.clo and int(c.max()) < beam.chi)
        self.pb.path = self.path_mode | (PATH_CELLS_INSIDE if inside else 0)

    def step(self, n_steps, stream=None, timing=None):
        """Enqueue the next n_steps steps on ``stream`` (default: torch's current stream; the
        run's buffers are set up on the stream current at construction, which another stream
        first waits for).  Asynchronous unless ``timing`` is given: then the call runs launch
        by launch and fills the FdtdPicTiming with per-kernel GPU time."""
        g = self.grid
        t0 = self.step_done
        t1 = min(g.n_steps, t0 + n_steps)
        d = self.desc.copy()
        d["step_begin"], d["step_end"] = t0, t1
        d["resume"] = 1 if t0 > 0 else 0
        s = stream or torch.cuda.current_stream(self.dev)
        # the descriptor goes in on the launch stream: after the work already queued there (which
        # reads the previous call's descriptor), before this call's kernels
        with torch.cuda.stream(s):
            self.d_desc.copy_(torch.from_numpy(d.view(np.uint8).copy()), non_blocking=False)
        st = ctypes.c_void_p(s.cuda_stream)
        check(self.L.fdtdpic_run(
            self.prec, d.ctypes.data, _ptr(self.d_desc), _ptr(self.d_table), _ptr(self.d_src),
            _ptr(self.d_state), _ptr(self.d_probe), ctypes.byref(self.pb), _ptr(self.d_cell),
            _ptr(self.d_frac), _ptr(self.d_ux), _ptr(self.d_uz), _ptr(self.d_id),
            _ptr(self.d_jx), _ptr(self.d_jz), _ptr(self.d_hyp), _ptr(self.d_scratch),
            self.scratch_bytes, _ptr(self.d_status),
            ctypes.byref(timing) if timing is not None else None, st), "fdtdpic_run")
        self.step_done = t1

    def reset(self, beam: Beam | None = None):
        """Back to step 0 with the initial beam (device-to-device; for repeated runs)."""
        b = self.beam if beam is None else beam
        self._set_inside(b)
        self.d_cell.copy_(torch.from_numpy(np.ascontiguousarray(b.cell, np.int32)))
        self.d_frac.copy_(torch.from_numpy(np.ascontiguousarray(b.frac)))
        self.d_ux.copy_(torch.from_numpy(np.ascontiguousarray(b.ux)))
        self.d_uz.copy_(torch.from_numpy(np.ascontiguousarray(b.uz)))
        self.d_id.copy_(torch.from_numpy(np.ascontiguousarray(b.id, np.int32)))
        self.d_hyp.zero_()
        self.d_probe.zero_()
        self.d_status.zero_()
        self.step_done = 0

    def snapshot(self) -> "PicSnapshot":
        """Host copy of everything the run carries between calls: the grid state (Ex, Hy, Dx,
        P, P one step back, both psi arrays, Acubic), Hy one half step back, the last grid
        currents, the probe traces so far, the status words, the particles (in their current
        order, with their ids) and the step reached.  The scratch holds nothing between calls
        (the deposit accumulators are cleared by every step that reads them; the step counter
        and the re-binning buffers are set by each call), so :meth:`restore` of this snapshot
        into a run of the same grid and beam sizes continues exactly: bit for bit the run that
        was never stopped.  Synchronises the device."""
        torch.cuda.synchronize(self.dev)
        cp = lambda t: t.to("cpu", copy=True)  # noqa: E731
        return PicSnapshot(step_done=self.step_done, path=int(self.pb.path),
                           state=cp(self.d_state), hyp=cp(self.d_hyp), jx=cp(self.d_jx),
                           jz=cp(self.d_jz), probe=cp(self.d_probe), status=cp(self.d_status),
                           cell=cp(self.d_cell), frac=cp(self.d_frac), ux=cp(self.d_ux),
                           uz=cp(self.d_uz), id=cp(self.d_id))

    def restore(self, snap: "PicSnapshot"):
        """Load a snapshot taken from a run of the same grid and beam sizes and precision; the
        next :meth:`step` continues from its step."""
        pairs = ((self.d_state, snap.state), (self.d_hyp, snap.hyp), (self.d_jx, snap.jx),
                 (self.d_jz, snap.jz), (self.d_probe, snap.probe), (self.d_status, snap.status),
                 (self.d_cell, snap.cell), (self.d_frac, snap.frac), (self.d_ux, snap.ux),
                 (self.d_uz, snap.uz), (self.d_id, snap.id))
        for dst, src in pairs:
            if dst.shape != src.shape or dst.dtype != src.dtype:
                raise ValueError("snapshot of another grid, beam or precision: "
                                 f"{tuple(src.shape)} {src.dtype} vs {tuple(dst.shape)} {dst.dtype}")
        for dst, src in pairs:
            dst.copy_(src)
        self.pb.path = (self.pb.path & ~PATH_CELLS_INSIDE) | (snap.path & PATH_CELLS_INSIDE)
        self.step_done = int(snap.step_done)

    def run_host(self, cell, frac, ux, uz, n_steps=None, stream=None):
        """One run from a beam in host memory: copy it in (pinned host tensors copy
        asynchronously), start from zero fields, run ``n_steps`` (default: every step of the
        grid) and return the probe traces and the final Ex as host tensors.  Particle ids are
        the beam's indices."""
        st = stream or torch.cuda.current_stream(self.dev)
        c = torch.as_tensor(cell)
        inside = c.numel() == 0 or (int(c.min()) >= self.beam.clo and int(c.max()) < self.beam.chi)
        self.pb.path = self.path_mode | (PATH_CELLS_INSIDE if inside else 0)
        with torch.cuda.stream(st):
            for dst, src in ((self.d_cell, c), (self.d_frac, frac), (self.d_ux, ux),
                             (self.d_uz, uz)):
                dst.copy_(torch.as_tensor(src), non_blocking=True)
            self.d_id.copy_(torch.arange(self.d_id.numel(), dtype=torch.int32,
                                         device=self.dev), non_blocking=True)
            self.d_hyp.zero_()
            self.d_status.zero_()
        self.step_done = 0
        self.step(self.grid.n_steps if n_steps is None else n_steps, stream=st)
        with torch.cuda.stream(st):
            probes = self.d_probe.to("cpu", non_blocking=False)
            ex = self.d_state[:self.grid.nz + 1].to("cpu", non_blocking=False)
        return probes, ex

    def fields(self):
        n = self.grid.nz + 1
        s = self.d_state.double().cpu().numpy()
        return {k: s[v * n:(v + 1) * n].copy() for k, v in ST.items()}

    def particles(self):
        """Host copy ordered by particle id: (cell, frac, ux, uz)."""
        idx = self.d_id.cpu().numpy()
        order = np.argsort(idx)
        return (self.d_cell.cpu().numpy()[order], self.d_frac.double().cpu().numpy()[order],
                self.d_ux.double().cpu().numpy()[order], self.d_uz.double().cpu().numpy()[order])

    def probes(self):
        return self.d_probe.double().cpu().numpy().reshape(self.grid.n_steps, 2)

    def currents(self):
        return self.d_jx.double().cpu().numpy(), self.d_jz.double().cpu().numpy()

    def status(self):
        return self.d_status.cpu().numpy()


def large_case(nz=1 << 24, n_part=64 << 20, total=20000, dz=0.015, nzsrc=100, precision="f32",
               sort_every=32, path="auto", chunk=0, pass_steps=0, tile_cells=0):
    """The large single-instance workload: ``nz`` cells, ``n_part`` macroparticles spread over
    the whole grid, a Kerr slab over the middle half, ``total`` steps (at the default sizes:
    2^24 cells, 64M particles, 20,000 steps, FP32)."""
    import scipy.constants as sc

    from .grid import lorentz_kerr_grid
    g = lorentz_kerr_grid(nz, total, front=nz // 4, rear=3 * nz // 4, nzsrc=nzsrc,
                          probes=(50, nz - 50), chi3=1e-2)
    beam = make_beam(n_part, 50, nz - 51, dz, seed=7, sort=False)
    return PicRun(g, beam, dz, 0.5 * dz / C0, sc.mu_0, precision=precision,
                  sort_every=sort_every, chunk=chunk, path=path, pass_steps=pass_steps,
                  tile_cells=tile_cells)


def _main(argv=None):
    """``python -m fdtdpic.pic --nz N --particles P --steps S``: the large-instance workload at
    the given sizes; prints milliseconds per step (CUDA events) and the per-kernel split."""
    import argparse
    import json

    ap = argparse.ArgumentParser(prog="python -m fdtdpic.pic")
    ap.add_argument("--nz", type=int, default=1 << 24)
    ap.add_argument("--particles", type=int, default=64 << 20)
    ap.add_argument("--steps", type=int, default=256)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32")
    ap.add_argument("--path", choices=["auto", "streaming", "tiled", "pass"], default="auto")
    ap.add_argument("--chunk", type=int, default=0, help="particles per push CTA (0: default)")
    ap.add_argument("--pass-steps", type=int, default=0, help="pass path: steps a launch")
    ap.add_argument("--tile-cells", type=int, default=0, help="pass path: cells a tile")
    a = ap.parse_args(argv)
    run = large_case(a.nz, a.particles, a.warmup + 2 * a.steps, precision=a.precision,
                     path=a.path, chunk=a.chunk, pass_steps=a.pass_steps,
                     tile_cells=a.tile_cells)
    run.step(a.warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    run.step(a.steps)
    e1.record()
    e1.synchronize()
    tm = FdtdPicTiming()
    run.step(a.steps, timing=tm)
    ms = e0.elapsed_time(e1) / a.steps
    print(json.dumps({"nz": a.nz, "n_part": a.particles, "steps": a.steps,
                      "ms_per_step": round(ms, 4),
                      "kernel_ms_per_step": {"push": round(tm.push_ms / a.steps, 4),
                                             "field": round(tm.field_ms / a.steps, 4),
                                             "sort": round(tm.sort_ms / a.steps, 4)},
                      "status": [int(x) for x in run.status()]}))


if __name__ == "__main__":
    _main()
