"""Batched sweep: thousands of independent grids in ONE persistent launch, then reflection vs
frequency from a batched DFT of their probe traces.

The reference sweeps sequentially: ``LoopedSim(loop=True)`` (MasterController.py:533-569)
rebuilds the parameter objects and runs one integrator per frequency point, then
``results(RefCo=True)`` takes an FFT peak-bin ratio of two probe traces
(MasterController.py:485-500, TransformHandler.py:34-78).  Here every instance of a batch (its
own grid length, slab and material) is a CTA-resident grid of the persistent batch kernel, and
|R(f)| = |DFT(probe 2)| / |DFT(probe 1)| is evaluated at every requested frequency.

``make_sweep_grids`` builds the seeded synthetic batch of the 4096-instance workload:
Nz ~ U{500..8000}, slab width U[0.05, 0.30] Nz centred between the source and the far PML,
d_eps ~ U[0.5, 4], f0 ~ U[0.8, 2.5] GHz, chi3 ~ logU[1e-4, 1e-1], Kerr integrator semantics,
dz = 15 mm, dt = 0.5 dz/c, PML 20, Gaussian-modulated 1 GHz source at cell 100, probes at
cells 50 and Nz-50.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import engine
from . import physics_setup as ps
from ._lib import MODE_KERR, check, lib
from .grid import lorentz_kerr_grid

DZ = 0.015
SC = 0.5


@dataclass
class SweepSpec:
    n_inst: int = 4096
    n_steps: int = 8192
    nz_lo: int = 500
    nz_hi: int = 8000
    slab_lo: float = 0.05
    slab_hi: float = 0.30
    deps_lo: float = 0.5
    deps_hi: float = 4.0
    f0_lo: float = 0.8e9
    f0_hi: float = 2.5e9
    chi3_lo: float = 1e-4
    chi3_hi: float = 1e-1
    seed: int = 20261203
    pml: int = 20
    nzsrc: int = 100
    freq_in: float = 1e9
    n_freqs: int = 512
    f_lo: float = 0.2e9
    f_hi: float = 3.0e9

    def freqs(self):
        return np.linspace(self.f_lo, self.f_hi, self.n_freqs)


def sweep_parameters(spec: SweepSpec):
    """Seeded per-instance parameters of the batch (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    nz = rng.integers(spec.nz_lo, spec.nz_hi + 1, spec.n_inst)
    width = np.maximum(1, np.round(rng.uniform(spec.slab_lo, spec.slab_hi, spec.n_inst) * nz)).astype(int)
    deps = rng.uniform(spec.deps_lo, spec.deps_hi, spec.n_inst)
    f0 = rng.uniform(spec.f0_lo, spec.f0_hi, spec.n_inst)
    chi3 = 10.0 ** rng.uniform(np.log10(spec.chi3_lo), np.log10(spec.chi3_hi), spec.n_inst)
    out = []
    for i in range(spec.n_inst):
        n = int(nz[i])
        centre = (spec.nzsrc + (n - spec.pml)) // 2
        front = max(spec.nzsrc + 2, centre - int(width[i]) // 2)
        rear = min(n - spec.pml - 2, front + int(width[i]))
        out.append(dict(nz=n, front=int(front), rear=int(rear), d_eps=float(deps[i]),
                        f0=float(f0[i]), chi3=float(chi3[i]), probes=(50, n - 50)))
    return out


def make_sweep_grids(spec: SweepSpec, eps0=None, mu0=None, mode=MODE_KERR):
    """The grids of the batch; all share one source array (same dt)."""
    dt = SC * DZ / ps.C0
    src = ps.gauss_sine(spec.n_steps, spec.freq_in, dt)
    hys = np.zeros(spec.n_steps)
    grids = []
    for p in sweep_parameters(spec):
        g = lorentz_kerr_grid(p["nz"], spec.n_steps, dz=DZ, sc=SC, front=p["front"],
                              rear=p["rear"], pml=spec.pml, nzsrc=spec.nzsrc,
                              probes=p["probes"], d_eps=p["d_eps"], f0=p["f0"],
                              gamma=2 * np.pi * 0.1e9, chi3=p["chi3"], freq_in=spec.freq_in,
                              mode=mode, source=src, eps0=eps0, mu0=mu0)
        g.hys = hys  # one shared source pair in the packed source pool
        grids.append(g)
    return grids, dt


class Sweep:
    """A batch resident on the GPU: ``run()`` enqueues the persistent batch launch, the DFT of
    both probe traces of every instance and |R(f)|; ``capture()`` records that sequence once
    as a CUDA graph, after which ``run()`` replays it.  dft: "tc" (tensor cores, split-BF16x3;
    ``dft_error()`` reports a tensor-core wait that gave up) or "cuda" (FP32 CUDA cores)."""

    def __init__(self, grids, dt, freqs, precision="f32", threads=256, grid_ctas=0, dft="tc",
                 packed=None):
        self.L = lib()
        if packed is not None:  # a batch already on the device (fdtdpic.device_setup)
            grids = packed.grids
        self.grids = grids
        self.n = len(grids)
        steps = {g.n_steps for g in grids}
        if len(steps) != 1:
            raise ValueError("a sweep's grids must share their step count (one DFT length)")
        self.S = steps.pop()
        self.packed = engine.upload(grids, precision) if packed is None else packed
        if self.packed.global_idx:
            raise ValueError("every grid of a sweep must fit the resident kernel")
        self.threads, self.grid_ctas = threads, grid_ctas
        dev = self.packed.d_state.device
        self.freqs = np.asarray(freqs, np.float64)
        self.F = len(self.freqs)
        self.d_freqs = torch.from_numpy(self.freqs).to(dev)
        self.d_tw = torch.empty(int(self.L.fdtdpic_dft_twiddle_bytes(self.F, self.S)),
                                dtype=torch.uint8, device=dev)
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        check(self.L.fdtdpic_dft_twiddles(engine._ptr(self.d_freqs), self.F, self.S, dt,
                                          engine._ptr(self.d_tw), st), "fdtdpic_dft_twiddles")
        self.d_X = torch.empty(2 * self.n * self.F * 2, dtype=torch.float64, device=dev)
        self.d_R = torch.empty(self.n * self.F, dtype=torch.float64, device=dev)
        if dft not in ("tc", "cuda"):
            raise ValueError("dft must be 'tc' (tensor cores) or 'cuda' (CUDA cores)")
        self.dft = dft
        self.d_err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.tc_bytes = int(self.L.fdtdpic_dft_tc_scratch_bytes(2 * self.n, self.S, self.F))
        self.d_tc = (torch.empty(self.tc_bytes, dtype=torch.uint8, device=dev)
                     if dft == "tc" else None)
        self.graph = None

    @classmethod
    def from_spec(cls, spec, precision="f32", device_setup=True, **kw):
        """The seeded batch of ``spec``; with device_setup its CPML tables and coefficients are
        computed by fdtdpic_setup_batch instead of per grid on the host."""
        if device_setup:
            from .device_setup import sweep_batch
            packed, dt = sweep_batch(spec, precision)
            return cls(None, dt, spec.freqs(), precision=precision, packed=packed, **kw)
        grids, dt = make_sweep_grids(spec)
        return cls(grids, dt, spec.freqs(), precision=precision, **kw)

    def _enqueue(self, stream):
        self.launch_fields(stream)
        self.launch_spectra(stream)

    def launch_fields(self, stream):
        """The persistent batch launch: every instance's steps and probe traces."""
        engine.launch(self.packed, stream=stream, threads=self.threads, grid_ctas=self.grid_ctas)

    def launch_spectra(self, stream):
        """DFT of both probe traces of every instance, then |R(f)|."""
        p = self.packed
        st = ctypes.c_void_p(stream.cuda_stream)
        if self.dft == "tc":
            if self.d_tc is None:
                self.d_tc = torch.empty(self.tc_bytes, dtype=torch.uint8, device=p.d_probe.device)
            check(self.L.fdtdpic_dft_probes_tc(p.prec, engine._ptr(p.d_probe), 2 * self.n, self.S,
                                               2, 2 * self.S, 1, 2, engine._ptr(self.d_tw),
                                               self.F, engine._ptr(self.d_X),
                                               engine._ptr(self.d_tc), self.tc_bytes,
                                               engine._ptr(self.d_err), st),
                  "fdtdpic_dft_probes_tc")
        else:
            check(self.L.fdtdpic_dft_probes(p.prec, engine._ptr(p.d_probe), 2 * self.n, self.S,
                                            2, 2 * self.S, 1, 2, engine._ptr(self.d_tw), self.F,
                                            engine._ptr(self.d_X), st), "fdtdpic_dft_probes")
        check(self.L.fdtdpic_reflection_ratio(engine._ptr(self.d_X), self.n, self.F,
                                              engine._ptr(self.d_R), st),
              "fdtdpic_reflection_ratio")

    def capture(self):
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._enqueue(s)  # warm-up outside capture (sets the kernel attributes)
        torch.cuda.current_stream().wait_stream(s)
        with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
            self._enqueue(s)
        self.graph = g
        return g

    def run(self, stream=None):
        """Replay the captured graph, or enqueue the sequence on ``stream`` (default: torch's
        current stream; another stream first waits for the stream the batch was uploaded on)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._enqueue(stream or torch.cuda.current_stream())

    def dft_error(self) -> int:
        return int(self.d_err.item())

    def reflection(self):
        return self.d_R.cpu().numpy().reshape(self.n, self.F)

    def spectra(self):
        X = self.d_X.cpu().numpy().reshape(2 * self.n, self.F, 2)
        return X[..., 0] + 1j * X[..., 1]

    def probes(self):
        return self.d_probe_view()

    def d_probe_view(self):
        return self.packed.d_probe.double().cpu().numpy().reshape(self.n, self.S, 2)

    def cell_steps(self):
        return float(sum((g.nz + 1) * (g.step_end - g.step_begin) for g in self.grids))


def shard_indices(grids, rank, world):
    """Instances of rank ``rank`` out of ``world`` when a sweep is split across GPUs: longest
    (by predicted cost) first, each to the currently lightest rank -- the instances are
    independent, so the ranks need no collective on the data path, only a gather of results."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    order = sorted(range(len(grids)), key=lambda i: (-grids[i].cost(), i))
    load = [0.0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += grids[i].cost()
        if r == rank:
            mine.append(i)
    return sorted(mine)


def plain_per_instance_rate(grids, precision="f32", threads=256, max_instances=32):
    """Cell-steps/s of the plain form -- one instance per launch, launched one after another --
    on up to max_instances of the batch (the baseline the batched launch is compared with)."""
    sub = grids[:max_instances]
    p = engine.upload(sub, precision)
    st = torch.cuda.current_stream()
    # one launch per instance: each its own single-instance batch
    singles = [engine.upload([g], precision) for g in sub]
    for s in singles[:2]:
        engine.launch(s, stream=st, threads=threads, grid_ctas=1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for s in singles:
        engine.launch(s, stream=st, threads=threads, grid_ctas=1)
    e1.record()
    e1.synchronize()
    del p
    cells = sum((g.nz + 1) * g.n_steps for g in sub)
    return cells / (e0.elapsed_time(e1) * 1e-3), e0.elapsed_time(e1)


def plain_global_rate(grids, precision="f32", max_instances=4):
    """Cell-steps/s of the other plain form: each instance alone on the global-memory path
    (fdtd1d_run_global, fields in HBM, an E and an H launch per step over every SM), one
    instance after another, on up to max_instances of the batch."""
    sub = grids[:max_instances]
    singles = []
    for g in sub:
        s = engine.upload([g], precision)
        s.global_idx, s.resident = [0], []
        singles.append(s)
    st = torch.cuda.current_stream()
    engine.launch(singles[0], stream=st)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for s in singles:
        engine.launch(s, stream=st)
    e1.record()
    e1.synchronize()
    cells = sum((g.nz + 1) * g.n_steps for g in sub)
    return cells / (e0.elapsed_time(e1) * 1e-3), e0.elapsed_time(e1)


# ------------------------------------------------------------------------------------------
# autotuner: CTA size and grid for the resident batch kernel, cached per device and bucket
# ------------------------------------------------------------------------------------------
_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "fdtdpic", "autotune.json")


def _bucket(grids):
    nz = np.array([g.nz for g in grids])
    return f"n{len(grids)}_nzmean{int(nz.mean()) // 500 * 500}_nzmax{int(nz.max()) // 1000 * 1000}"


def autotune(grids, precision="f32", probe_steps=256, candidates=(128, 256, 512, 1024),
             sample=None, cache=True):
    """Pick threads-per-CTA for the resident batch kernel by timing a short run
    (probe_steps steps) of a sample of the batch for each candidate; cached on disk by device
    name, precision and batch shape."""
    dev_name = torch.cuda.get_device_name()
    key = f"{dev_name}|{precision}|{_bucket(grids)}"
    table = {}
    if cache and os.path.exists(_CACHE):
        try:
            table = json.load(open(_CACHE))
        except Exception:
            table = {}
    if key in table:
        return table[key]
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    pick = grids if sample is None else grids[:sample]
    if sample is None:
        pick = grids[:min(len(grids), 4 * sm)]
    short = []
    for g in pick:
        h = _copy_grid(g)
        h.step_end = min(h.n_steps, probe_steps)
        short.append(h)
    best, timings = None, {}
    for th in candidates:
        p = engine.upload(short, precision)
        engine.launch(p, threads=th)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        engine.launch(p, threads=th)
        e1.record()
        e1.synchronize()
        timings[th] = e0.elapsed_time(e1)
        if best is None or timings[th] < timings[best]:
            best = th
    res = {"threads": int(best), "timings_ms": {str(k): v for k, v in timings.items()}}
    if cache:
        table[key] = res
        os.makedirs(os.path.dirname(_CACHE), exist_ok=True)
        tmp = _CACHE + f".{os.getpid()}"
        json.dump(table, open(tmp, "w"))
        os.replace(tmp, _CACHE)
    return res


def _copy_grid(g):
    from dataclasses import replace
    return replace(g)


def _main(argv=None):
    """One sweep of the seeded ragged batch: ``python -m fdtdpic.sweep --instances N --steps T``
    (profiling driver; prints the field and spectra times)."""
    import argparse
    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=8192)
    ap.add_argument("--dft", choices=["tc", "cuda"], default="tc")
    ap.add_argument("--threads", type=int, default=256)
    a = ap.parse_args(argv)
    spec = SweepSpec(n_inst=a.instances, n_steps=a.steps)
    grids, dt = make_sweep_grids(spec)
    sw = Sweep(grids, dt, spec.freqs(), precision="f32", threads=a.threads, dft=a.dft)
    st = torch.cuda.current_stream()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    sw.launch_fields(st)
    e1.record()
    sw.launch_spectra(st)
    e2.record()
    e2.synchronize()
    print(json.dumps(dict(instances=sw.n, steps=sw.S, fields_ms=e0.elapsed_time(e1),
                          spectra_ms=e1.elapsed_time(e2), dft=a.dft,
                          dft_error=sw.dft_error())))


if __name__ == "__main__":
    _main()
