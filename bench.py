#!/usr/bin/env python
"""Benchmark of the 1D FDTD + electron-beam PIC time-stepping path on GB300.

Workload (one bench step = one whole run): a 4096-cell grid (dz = 15 mm, dt = 0.5 dz/c,
PML 20 cells, Lorentz/Kerr slab in cells 400-599 with d_eps=2, f0=1.5 GHz, gamma=2 pi 0.1 GHz,
chi3=1e-2, Gaussian-modulated 1 GHz soft source at cell 100, probes at cells 50 and 4046)
advanced 8192 steps together with a beam of 1,048,576 macroparticles (uniform over cells
50-4045, vz ~ N(0.3c, 0.003c), density 1e14 m^-3), FP32 state.  Synthetic, seeded inputs.

  value   (cell-steps + particle-steps) / s of the device-resident run, in millions
  e2e     the same through the public API with the beam copied from pinned host memory and
          the probe traces and final Ex read back inside the timed region

``--impl reference`` times the reference CPU path instead: the reference itself cannot run
(numba and its Tests package are absent), so this is the FP64 C restatement of its algorithm
(the oracle), on all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "py-fdtd_pic_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NZ, T, NP = 4096, 8192, 1 << 20
DZ = 0.015
FRONT, REAR, NZSRC, PROBES = 400, 600, 100, (50, 4046)
CLO, CHI = 50, 4045
METRIC = "Mcell-steps/s + Mparticle-steps/s vs plain GPU kernel; p50/p99 sweep latency"
UNIT = "Mcell-steps/s + Mparticle-steps/s"
WORKLOAD = "fdtd_pic_1inst_nz4096_steps8192_np1048576"
BYTES_PER_PARTICLE = 24  # z, ux, uz read + write at 4 B (6p, p = 4)
BYTES_PER_CELL = 16      # Ex, Hy read + write at 4 B (4p)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _setup(precision):
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    grid = lorentz_kerr_grid(NZ, T, front=FRONT, rear=REAR, nzsrc=NZSRC, probes=PROBES, chi3=1e-2)
    beam = make_beam(NP, CLO, CHI, DZ)
    dt = 0.5 * DZ / 299792458.0
    run = PicRun(grid, beam, DZ, dt, sc.mu_0, precision=precision, sort_every=32)
    return grid, beam, run, dt


def run_ours(args):
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    from fdtdpic.pic import FdtdPicTiming

    grid, beam, run, dt = _setup(args.precision)
    # device-resident copy of the initial beam: each bench step restarts from it
    init = [t.clone() for t in (run.d_cell, run.d_frac, run.d_ux, run.d_uz, run.d_id)]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def reset_device():
        for dst, src in zip((run.d_cell, run.d_frac, run.d_ux, run.d_uz, run.d_id), init):
            dst.copy_(src)
        run.d_hyp.zero_()
        run.d_status.zero_()
        run.step_done = 0

    for _ in range(args.warmup):
        reset_device()
        run.step(T)
    torch.cuda.synchronize()
    assert int(run.status()[0]) == 0, "particles left the grid"

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    times = []
    with Clocks(local) as clk:
        barrier()
        for _ in range(args.steps):
            flush.fill_(1)  # > L2 (129 MB): nothing of the previous step stays cached
            reset_device()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run.step(T)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
    ms = sum(times) / len(times)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    units = (NZ + NP) * T
    value = units * world / (ms * 1e-3) / 1e6

    # end to end through the public API: beam from pinned host memory, results read back
    h = [t.cpu().pin_memory() for t in init]
    e2e_times = []
    h2d = sum(t.numel() * t.element_size() for t in h)
    d2h = 0
    for _ in range(max(1, min(args.steps, 3))):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for dst, src in zip((run.d_cell, run.d_frac, run.d_ux, run.d_uz, run.d_id), h):
            dst.copy_(src, non_blocking=True)
        run.d_hyp.zero_()
        run.step_done = 0
        run.step(T)
        probes = run.d_probe.to("cpu", non_blocking=False)
        ex = run.d_state[:NZ + 1].to("cpu", non_blocking=False)
        e1.record()
        e1.synchronize()
        e2e_times.append(e0.elapsed_time(e1))
        d2h = probes.numel() * probes.element_size() + ex.numel() * ex.element_size()
    e2e_ms = statistics.median(e2e_times)

    # per-kernel GPU time (CUDA events around every launch) for the roofline
    reset_device()
    tm = FdtdPicTiming()
    run.step(T, timing=tm)
    torch.cuda.synchronize()
    tiled = tm.path == 2
    if tiled:
        # one persistent launch runs every step: its algorithmic bytes are all steps' particle
        # and cell traffic
        push_ms = tm.push_ms
        achieved = (BYTES_PER_PARTICLE * NP + BYTES_PER_CELL * NZ) * T / (push_ms * 1e-3) / 1e9
    else:
        push_ms = tm.push_ms / T
        achieved = BYTES_PER_PARTICLE * NP / (push_ms * 1e-3) / 1e9
    peak, peak_kind = _peaks()
    traffic = None
    prof = os.path.join(ROOT, "profiles", "pic_push_kernel_traffic.json")
    if os.path.exists(prof):
        try:
            traffic = float(json.load(open(prof))["dram_bytes_per_launch"])
        except Exception:
            traffic = None

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return None
    # our kernels per run: tiled = init, bin, the persistent kernel, offsets, unbin, status;
    # streaming = push + fused field per step, 3 re-binning kernels every 32 steps, 3 others
    launches_per_run = 6 if tiled else 2 * T + 3 * (T // 32) + 3
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "f32" else "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "nz": NZ, "time_steps": T, "n_part": NP,
                   "slab": [FRONT, REAR], "mode": "kerr", "sort_every": 32,
                   "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"one instance per GPU x{world}"},
        "mcell_steps_per_s": round(NZ * T * world / (ms * 1e-3) / 1e6, 1),
        "mparticle_steps_per_s": round(NP * T * world / (ms * 1e-3) / 1e6, 1),
        "e2e": {"value": round(units * world / (e2e_ms * 1e-3) / 1e6, 1), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_ms, 3)},
        "roofline": {"bound": "hbm",
                     "kernel": "pic_tiled_kernel<float>" if tiled else "pic_push_kernel<float>",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 3), "peak_source": peak_kind,
                     "traffic": traffic,
                     "per_launch_ms": round(push_ms, 5),
                     "bytes_per_launch": ((BYTES_PER_PARTICLE * NP + BYTES_PER_CELL * NZ) * T
                                          if tiled else BYTES_PER_PARTICLE * NP),
                     "kernel_share": {"push": round(tm.push_ms, 2), "field": round(tm.field_ms, 2),
                                      "sort": round(tm.sort_ms, 2)}},
        "gpu_launches": launches_per_run * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return out


def _oracle_setup(n_part):
    import numpy as np
    import scipy.constants as sc
    from oracle import oracle as O
    dt = 0.5 * DZ / O.C0
    P = O.RefParams(Nz=NZ, timeSteps=T, dz=DZ, delT=dt, courantNo=O.f32(0.5),
                    materialFrontEdge=FRONT, materialRearEdge=REAR, pmlWidth=20, nzsrc=NZSRC,
                    freq_in=1e9, permit_0=sc.epsilon_0, permea_0=sc.mu_0, nonLinMed=True,
                    FreeSpace=False, plasmaFreqE=np.sqrt(2.0) * 2 * np.pi * 1.5e9,
                    omega_0E=2 * np.pi * 1.5e9, gammaE=2 * np.pi * 0.1e9, chi3Stat=1e-2,
                    sigmaOpt=O.sigma_opt(DZ, sc.epsilon_0, sc.mu_0))
    cell, frac, ux, uz = O.beam(n_part, CLO, CHI)
    w = 1e14 * (CHI - CLO) * DZ / n_part
    k = O.pic_constants(DZ, dt, w, sc.mu_0)
    src = O.gauss_sine(T, 1e9, dt)
    return O, P, (cell, frac, ux, uz), k, src


def cpu_baseline(seconds=15.0):
    """The FP64 C oracle on all host cores, on the first steps of the same workload."""
    import numpy as np
    O, P, (cell, frac, ux, uz), k, src = _oracle_setup(NP)
    cores = os.cpu_count() or 1
    steps = 4
    t0 = time.perf_counter()
    O.integrate_pic(P, O.KERR, src, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI, n_steps=steps,
                    probe_cells=PROBES, n_threads=cores)
    dt_ = time.perf_counter() - t0
    steps = max(steps, min(2000, int(seconds / max(dt_ / steps, 1e-6))))
    O, P, (cell, frac, ux, uz), k, src = _oracle_setup(NP)
    t0 = time.perf_counter()
    O.integrate_pic(P, O.KERR, src, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI, n_steps=steps,
                    probe_cells=PROBES, n_threads=cores)
    el = time.perf_counter() - t0
    return {"value": round((NZ + NP) * steps / el / 1e6, 2), "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": f"first {steps} of {T} steps of the same workload (FP64 oracle, "
                      f"{cores} OpenMP threads)", "seconds": round(el, 2)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import numpy as np
    cores = os.cpu_count() or 1
    per_step_s = []
    steps_sample = None
    for i in range(args.warmup + args.steps):
        O, P, (cell, frac, ux, uz), k, src = _oracle_setup(NP)
        if steps_sample is None:
            t0 = time.perf_counter()
            O.integrate_pic(P, O.KERR, src, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI,
                            n_steps=2, probe_cells=PROBES, n_threads=cores)
            one = (time.perf_counter() - t0) / 2
            steps_sample = max(2, min(T, int(args.cpu_seconds / max(one, 1e-6))))
            O, P, (cell, frac, ux, uz), k, src = _oracle_setup(NP)
        t0 = time.perf_counter()
        O.integrate_pic(P, O.KERR, src, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI,
                        n_steps=steps_sample, probe_cells=PROBES, n_threads=cores)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            per_step_s.append(el)
    el = statistics.median(per_step_s)
    value = (NZ + NP) * steps_sample / el / 1e6
    sample = (f"first {steps_sample} of {T} steps of {WORKLOAD} per step (FP64 C oracle "
              f"restating the reference algorithm; the reference itself needs numba)")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(el * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "nz": NZ, "time_steps": T, "n_part": NP},
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--time-steps", type=int, default=None,
                    help="shorter runs for profiling under ncu (the line is then not a bench "
                         "number and says so in config.time_steps)")
    args = ap.parse_args()
    if args.time_steps:
        global T
        T = int(args.time_steps)
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
