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
# particles re-binned by cell every SORT_EVERY steps (64 measured best on GB300 for the headline:
# 114.8 ms a run against 117.4 at 32, 123.1 at 16; the results are the same bits at any interval)
SORT_EVERY = 64


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region, of the GPU this process runs on (named by
    its UUID: under CUDA_VISIBLE_DEVICES the local ordinal is not nvidia-smi's index)."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.gpu_id = _gpu_id(device)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_id}", f"--query-gpu={self.Q}",
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
                "samples": len(sm), "gpu": self.gpu_id}


def _gpu_id(device):
    """nvidia-smi's name for a torch device: its UUID (GPU-...), else its PCI bus id, else the
    ordinal."""
    try:
        import torch
        props = torch.cuda.get_device_properties(device)
        u = str(getattr(props, "uuid", "") or "")
        if u:
            return u if u.startswith("GPU-") else "GPU-" + u
        bus = getattr(props, "pci_bus_id", None)
        if bus is not None:
            return (f"{int(getattr(props, 'pci_domain_id', 0)):08x}:{int(bus):02x}:"
                    f"{int(getattr(props, 'pci_device_id', 0)):02x}.0")
    except Exception:
        pass
    return str(device)


def _setup(precision):
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    grid = lorentz_kerr_grid(NZ, T, front=FRONT, rear=REAR, nzsrc=NZSRC, probes=PROBES, chi3=1e-2)
    beam = make_beam(NP, CLO, CHI, DZ)
    dt = 0.5 * DZ / 299792458.0
    run = PicRun(grid, beam, DZ, dt, sc.mu_0, precision=precision, sort_every=SORT_EVERY)
    return grid, beam, run, dt


def _launch_shares(precision):
    """Per-kernel shares of the headline run's GPU time from the committed ncu launch list of
    this workload (profiles/fdtd_pic_nz4096_np1m_launch_list.json), or None."""
    path = os.path.join(ROOT, "profiles", "fdtd_pic_nz4096_np1m_launch_list.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d[precision]
    except Exception:
        return None


def l2_copy_gbs(dev, mib=32, reps=200):
    """Device-to-device copy bandwidth of a buffer that stays in the 129 MB L2 (read + write
    bytes per second), CUDA events around reps back-to-back copies after a warm-up."""
    import torch
    n = (mib << 20) // 4
    a = torch.ones(n, dtype=torch.float32, device=dev)
    b = torch.empty_like(a)
    for _ in range(20):
        b.copy_(a)
    e0, e1 = _events()
    e0.record()
    for _ in range(reps):
        b.copy_(a)
    e1.record()
    e1.synchronize()
    return 2 * a.numel() * 4 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9


def _headline(args, precision, steps, warmup, flush, world, local):
    """One precision of the headline: device-resident runs (the line's value), runs through the
    public host-buffer call (e2e), and the push launch's roofline."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    grid, beam, run, dt = _setup(precision)
    init = [t.clone() for t in (run.d_cell, run.d_frac, run.d_ux, run.d_uz, run.d_id)]

    def reset_device():
        for dst, src in zip((run.d_cell, run.d_frac, run.d_ux, run.d_uz, run.d_id), init):
            dst.copy_(src)
        run.d_hyp.zero_()
        run.d_status.zero_()
        run.step_done = 0

    for _ in range(warmup):
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
    with Clocks(dev) as clk:
        barrier()
        for _ in range(steps):
            flush.fill_(1)  # > L2 (129 MB): nothing of the previous step stays cached
            reset_device()
            e0, e1 = _events()
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

    # end to end through the public call: PicRun.run_host takes the beam from pinned host
    # memory and returns the probe traces and the final Ex on the host
    host = [t.cpu().pin_memory() for t in init[:4]]
    h2d = sum(t.numel() * t.element_size() for t in host)
    e2e_times, d2h = [], 0
    for _ in range(max(1, min(steps, 3))):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        probes, ex = run.run_host(*host)
        e1.record()
        e1.synchronize()
        e2e_times.append(e0.elapsed_time(e1))
        d2h = probes.numel() * probes.element_size() + ex.numel() * ex.element_size()
    e2e_ms = statistics.median(e2e_times)

    # the push launch's time: its share of the run's GPU time in the committed ncu launch list
    # of this workload, times this run's measured step time
    from fdtdpic.pic import FdtdPicTiming
    reset_device()
    tm = FdtdPicTiming()
    run.step(64, timing=tm)  # which kernels this workload takes (path 3: push carries H)
    torch.cuda.synchronize()
    fused = tm.path == 3
    bpp = BYTES_PER_PARTICLE * (2 if precision == "f64" else 1)
    kernel = ("pic_push_kernel<%s, FUSE_H>" % ("double" if precision == "f64" else "float")
              if fused else "pic_push_kernel")
    shares = _launch_shares(precision)
    n_push = T  # one push launch per step (fused except after each re-binning)
    if shares and "push" in shares:
        per_launch = shares["push"] * ms / n_push
        source = ("launch-list share %.3f (profiles/fdtd_pic_nz4096_np1m_launch_list.json) x "
                  "this run's ms_per_step / %d push launches" % (shares["push"], n_push))
    else:
        per_launch, source = None, "no launch list committed for this precision"
    peak, peak_kind = _peaks()
    roof = {"bound": "hbm", "kernel": kernel, "path": "streaming", "unit": "GB/s",
            "peak": peak, "peak_source": peak_kind, "bytes_per_launch": bpp * NP,
            "per_launch_ms": None if per_launch is None else round(per_launch, 5),
            "per_launch_source": source, "achieved": None, "frac": None, "traffic": None}
    if per_launch:
        achieved = bpp * NP / (per_launch * 1e-3) / 1e9
        roof.update(achieved=round(achieved, 1), frac=round(achieved / peak, 3))
        l2 = l2_copy_gbs(dev)
        beam_mib = NP * (4 + 3 * (8 if precision == "f64" else 4)) / 2 ** 20
        roof.update(l2_gbs=round(l2, 1), l2_frac=round(achieved / l2, 3),
                    l2_note="the beam (%d MiB: cell, frac, ux, uz) and fields stay in L2 "
                            "between steps: l2_frac is achieved / a live L2-resident copy's "
                            "bandwidth" % beam_mib)
    prof = os.path.join(ROOT, "profiles", "pic_push_kernel_traffic.json")
    if os.path.exists(prof) and precision == "f32":
        try:
            roof["traffic"] = float(json.load(open(prof))["dram_bytes_per_launch"])
        except Exception:
            pass
    # our kernels per run (the beam lies inside its domain, so each push launch carries the
    # previous step's H phase): push and E phase per step, a standalone H phase before each
    # re-binning and at each block's end (one per SORT_EVERY steps), five re-binning kernels
    # (histogram, three-launch scan, scatter) every SORT_EVERY steps, the step counter's advance
    # per graph block (2 SORT_EVERY steps), and init, constants, step-counter set and finish
    launches_per_run = 2 * T + 6 * (T // SORT_EVERY) + T // (2 * SORT_EVERY) + 4
    return dict(ms=ms, value=units * world / (ms * 1e-3) / 1e6, clocks=clk.summary(),
                e2e={"value": round(units * world / (e2e_ms * 1e-3) / 1e6, 1), "unit": UNIT,
                     "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                     "ms_per_step": round(e2e_ms, 3),
                     "call": "PicRun.run_host(cell, frac, ux, uz) from pinned host tensors"},
                roofline=roof, launches=launches_per_run * steps, run=run)


def run_ours(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    h = _headline(args, args.precision, args.steps, args.warmup, flush, world, local)
    h.pop("run")
    f64 = None
    if args.precision == "f32" and not args.no_f64:
        f64 = _headline(args, "f64", max(3, min(args.steps, 3)), 3, flush, world, local)
        f64.pop("run")
        torch.cuda.empty_cache()
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return None
    ms = h["ms"]
    out = {
        "metric": METRIC, "value": round(h["value"], 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "f32" else "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "nz": NZ, "time_steps": T, "n_part": NP,
                   "slab": [FRONT, REAR], "mode": "kerr", "sort_every": SORT_EVERY,
                   "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"one instance per GPU x{world}"},
        "mcell_steps_per_s": round(NZ * T * world / (ms * 1e-3) / 1e6, 1),
        "mparticle_steps_per_s": round(NP * T * world / (ms * 1e-3) / 1e6, 1),
        "e2e": h["e2e"], "roofline": h["roofline"], "gpu_launches": h["launches"],
        "clocks": h["clocks"],
    }
    if f64 is not None:
        out["f64"] = {"dtype": "f64", "value": round(f64["value"], 1), "unit": UNIT,
                      "steps": max(3, min(args.steps, 3)), "warmup": 3,
                      "ms_per_step": round(f64["ms"], 3), "e2e": f64["e2e"],
                      "roofline": f64["roofline"], "clocks": f64["clocks"],
                      "note": "the same workload in FP64 on the GPU, beside the FP64 CPU "
                              "reference arm"}
    for name, fn in (("sweep", bench_sweep), ("serve", bench_serve), ("knee", bench_serve_knee),
                     ("large", bench_large), ("variants", bench_variants)):
        if name in args.extra:
            try:
                out[name] = fn(args, flush)
            except Exception as e:  # a failing extra section must not hide the headline line
                out[name] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return out


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_sweep(args, flush):
    """The 4096-instance batched sweep (Nz ~ U{500..8000}, 8192 steps, Kerr slabs of random
    width and material, FP32): one persistent launch for all instances, then the 4096 x 2 probe
    DFTs at 512 frequencies and |R(f)|.  Compared with the plain form: the same kernel with one
    instance per launch, launched one after another (timed on the first 16 instances)."""
    import torch
    from fdtdpic import sweep
    spec = sweep.SweepSpec()
    # set-up, wall clock until the batch is ready to run: per grid on the host (the host
    # restatement of the reference's set-up, then packing and upload) and on the device
    # (fdtdpic.device_setup: batch layout in numpy, one set-up kernel)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    swd = sweep.Sweep.from_spec(spec, "f32", device_setup=True)
    torch.cuda.synchronize()
    setup_device_s = time.perf_counter() - t0
    del swd
    t0 = time.perf_counter()
    grids, dt = sweep.make_sweep_grids(spec)
    sw = sweep.Sweep(grids, dt, spec.freqs(), precision="f32", threads=256)
    torch.cuda.synchronize()
    setup_host_s = time.perf_counter() - t0
    st = torch.cuda.current_stream()
    sw.run()
    torch.cuda.synchronize()
    f_ms, s_ms = [], []
    for _ in range(max(1, min(args.steps, 3))):
        flush.fill_(1)
        a0, a1 = _events()
        b1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        sw.launch_fields(st)
        a1.record()
        sw.launch_spectra(st)
        b1.record()
        b1.synchronize()
        f_ms.append(a0.elapsed_time(a1))
        s_ms.append(a1.elapsed_time(b1))
    fields_ms, spectra_ms = statistics.median(f_ms), statistics.median(s_ms)
    # the same spectra on the CUDA cores, for comparison
    sw.dft = "cuda"
    c_ms = []
    for _ in range(2):
        b0, b1 = _events()
        b0.record()
        sw.launch_spectra(st)
        b1.record()
        b1.synchronize()
        c_ms.append(b0.elapsed_time(b1))
    sw.dft = "tc"
    cells = sw.cell_steps()
    status = sw.packed.d_status.cpu().numpy()
    fallbacks = int(sw.packed.d_fallbacks.cpu().numpy().sum())
    plain_rate, plain_ms = sweep.plain_per_instance_rate(grids, max_instances=16)
    global_rate, _ = sweep.plain_global_rate(grids, max_instances=4)
    best_plain = max(plain_rate, global_rate)
    batched = cells / ((fields_ms + spectra_ms) * 1e-3)
    dft_flops = 2.0 * (2 * sw.n) * (2 * sw.F) * sw.S  # real GEMM [2n x S] x [S x 2F]
    return {"workload": "sweep_4096inst_nz500-8000_steps8192_kerr_f32",
            "instances": sw.n, "time_steps": sw.S, "freqs": sw.F,
            "fields_ms": round(fields_ms, 2), "spectra_ms": round(spectra_ms, 2),
            "mcell_steps_per_s": round(batched / 1e6, 1),
            "plain_mcell_steps_per_s": round(plain_rate / 1e6, 1),
            "plain_global_mcell_steps_per_s": round(global_rate / 1e6, 1),
            "vs_plain": round(batched / best_plain, 1),
            "dft": "tcgen05 split-BF16x3, FP32 sums over 1024-step groups, compensated FP32 sums across groups",
            "dft_gemm_tflops": round(dft_flops / (spectra_ms * 1e-3) / 1e12, 2),
            "dft_tensor_tflops": round(3 * dft_flops / (spectra_ms * 1e-3) / 1e12, 2),
            "dft_cuda_core_ms": round(min(c_ms), 2), "dft_tc_error": sw.dft_error(),
            "fp64_cubic_resolves": fallbacks, "bad_status": int((status != 0).sum()),
            "setup_s": {"host": round(setup_host_s, 3), "device": round(setup_device_s, 3)},
            "plain": "the better of two one-instance-per-launch forms: the resident kernel with "
                     "one CTA (16 instances in sequence) and the global-memory path over every "
                     "SM (fdtd1d_run_global, 4 instances in sequence)"}


def bench_serve(args, flush):
    """Continuous-batching server on the served request stream (Poisson arrivals at 2000/s,
    Nz log-uniform 256-65536, steps 1k-50k, beams of 0-2M particles, sweep materials, FP32,
    150 GB HBM budget), run in real time for --serve-seconds.  The offered load is far above
    one GPU's capacity: the numbers are the completed requests' throughput and latency and the
    queue left at the end."""
    from fdtdpic import server
    secs = args.serve_seconds
    reqs = server.make_request_stream(rate=2000.0, duration=secs)
    srv = server.Server(precision="f32", hbm_budget=150e9)
    try:
        st = srv.run_stream(reqs, secs)
    finally:
        srv.close()
        srv.stream.synchronize()  # the rounds still in flight, before the next section
    st.update(workload="serve_poisson2000_nz256-65536_steps1k-50k_np0-2M_f32",
              offered=len(reqs), offered_rps=round(len(reqs) / secs, 1))
    return {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st.items()}


def bench_serve_knee(args, flush):
    """Saturation knee of the server: the served request stream (as in the serve section)
    offered open-loop at each of --knee-rates for --knee-seconds, then polled for --knee-grace
    seconds more without new arrivals.  Per rate: requests completed within that time, their
    throughput and p50/p99 latency, the backlog left (submitted, not completed) and the fraction
    of the time the slot rounds kept the GPU busy (the big requests' streaming runs, on streams
    of their own, are not in it).  The stream's service times are heavy-tailed (a request of 2M particles and 50k
    steps runs for minutes), so the run stops at the grace limit instead of draining.  The knee
    is the highest offered rate at which at least 90% of the requests completed."""
    from fdtdpic import server
    secs, grace = args.knee_seconds, args.knee_grace
    rows = []
    for rate in [float(r) for r in args.knee_rates.split(",") if r]:
        reqs = server.make_request_stream(rate=rate, duration=secs)
        srv = server.Server(precision="f32", hbm_budget=150e9)
        try:
            t0 = srv.clock()
            srv.run_stream(reqs, secs)
            t_end = t0 + secs + grace
            while (srv.pending or srv.active or srv.inflight) and srv.clock() < t_end:
                srv.poll()
                if not srv.active and not srv.inflight:
                    time.sleep(1e-3)  # waiting for the preparation thread
            elapsed = srv.clock() - t0
            st = srv.stats(elapsed, submitted=len(reqs))
        finally:
            srv.close()
            srv.stream.synchronize()
        done = st["completed"]
        rows.append({"offered_rps": rate, "submitted": len(reqs), "completed": done,
                     "completed_frac": round(done / len(reqs), 3) if reqs else None,
                     "throughput_rps": round(st["throughput_rps"], 2),
                     "p50_s": None if st["p50_s"] is None else round(st["p50_s"], 3),
                     "p99_s": None if st["p99_s"] is None else round(st["p99_s"], 3),
                     "backlog": len(reqs) - done,
                     "gpu_busy_rounds": (round(st["gpu_busy_s"] / elapsed, 3)
                                         if elapsed > 0 else None)})
    knee = max((r["offered_rps"] for r in rows
                if r["completed_frac"] is not None and r["completed_frac"] >= 0.9), default=None)
    return {"workload": "serve_nz256-65536_steps1k-50k_np0-2M_f32", "window_s": secs,
            "grace_s": grace, "rates": rows, "knee_rps": knee}


def bench_large(args, flush):
    """One large instance: Nz = 2^24 cells, 64M macroparticles over the whole grid, Kerr slab
    over the middle half, FP32, streaming PIC path; timed over --large-steps of its 20,000 steps
    after a 64-step warm-up (the rate per step is the same over the run)."""
    import torch
    from fdtdpic.pic import FdtdPicTiming, large_case
    nz, npart, total = 1 << 24, 64 << 20, 20000
    run = large_case(nz, npart, total, dz=DZ, nzsrc=NZSRC)
    run.step(64)
    torch.cuda.synchronize()
    n = args.large_steps
    e0, e1 = _events()
    e0.record()
    run.step(n)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    tm = FdtdPicTiming()
    run.step(64, timing=tm)
    slab = nz // 2
    alg = (nz * BYTES_PER_CELL + slab * 8 + nz * 8 + npart * BYTES_PER_PARTICLE)
    peak, kind = _peaks()
    gbs = alg * n / (ms * 1e-3) / 1e9
    out = {"workload": "large_nz16777216_np67108864_kerr_f32", "timed_steps": n,
           "ms_per_step": round(ms / n, 3),
           "mcell_steps_per_s": round(nz * n / (ms * 1e-3) / 1e6, 1),
           "mparticle_steps_per_s": round(npart * n / (ms * 1e-3) / 1e6, 1),
           "algorithmic_gbs": round(gbs, 1), "hbm_frac": round(gbs / peak, 3),
           "peak_source": kind, "bytes_per_step": alg,
           "kernel_ms_per_step": {"push": round(tm.push_ms / 64, 3),
                                  "field": round(tm.field_ms / 64, 3),
                                  "sort": round(tm.sort_ms / 64, 3)},
           "status": [int(x) for x in run.status()]}
    # beside the algorithmic count: the DRAM traffic ncu measured for a step's launches
    dram = _large_dram_bytes_per_step()
    if dram:
        dgbs = dram * n / (ms * 1e-3) / 1e9
        out.update(dram_bytes_per_step=int(dram), dram_gbs=round(dgbs, 1),
                   dram_frac=round(dgbs / peak, 3),
                   dram_source="ncu DRAM bytes of a step's push, E and H launches "
                               "(profiles/pic_kernels_large_half.json: half size x 2; the "
                               "re-binning launches not included) / this run's ms_per_step")
    return out


def _large_dram_bytes_per_step():
    """DRAM bytes of one full-size large-instance step (its push, E and H launches), from the
    committed ncu capture of the same kernels at half size, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "pic_kernels_large_half.json")) as f:
            d = json.load(f)
        return float(d["half_size_dram_bytes_per_step"]) * float(d["scale_to_full_size"])
    except Exception:
        return None


def bench_variants(args, flush):
    """Varin's one-pass ADE step (fdtdpic_variant_run, FDTD_VAR_VARIN_STEP) over 16 grids of
    2^22 cells, FP32: each cell reads Jx, P, Gx3, Qx3, Ex and writes Pbar3, Jx, P, Gx3, Qx3
    (40 B); 2.7 GB per launch, so the inputs stay well above L2 between launches."""
    import numpy as np
    import torch
    from fdtdpic import variants
    rows_n, n = 16, 1 << 22
    rec = variants.make_rows(np.full(rows_n, n), n - 1, 0, n, dt=1.6e-12, dz=1e-3,
                             eps0=8.854e-12, omega0=2 * np.pi * 1.5e9, gamma=2 * np.pi * 1e8,
                             chi1=0.2, chi3=1e-3, alpha3=0.699999988079071,
                             nl_gamma=2 * np.pi * 3e8, nl_omega0=2 * np.pi * 4e9)
    rows = variants.Rows(rec)
    g = torch.Generator(device="cuda").manual_seed(3)
    arrs = [torch.randn(rows_n, n, device="cuda", generator=g) * 1e-3 for _ in range(6)]
    for _ in range(3):
        variants.varin_step(*arrs, rows)
    torch.cuda.synchronize()
    k = 10
    e0, e1 = _events()
    e0.record()
    for _ in range(k):
        variants.varin_step(*arrs, rows)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / k
    alg = rows_n * n * 40
    peak, kind = _peaks()
    gbs = alg / (ms * 1e-3) / 1e9
    return {"workload": "varin_step_16x4194304_f32", "per_launch_ms": round(ms, 4),
            "bytes_per_launch": alg, "achieved_gbs": round(gbs, 1),
            "hbm_frac": round(gbs / peak, 3), "peak_source": kind,
            "finite": bool(torch.isfinite(arrs[1]).all().item())}


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
    ap.add_argument("--extra", default="sweep,serve,knee,large,variants",
                    help="comma-separated extra sections: sweep, serve, knee, large, variants "
                         "('' for none)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-f64", action="store_true", help="skip the FP64 run of the headline")
    ap.add_argument("--knee-rates", default="1,2,4,8,16",
                    help="offered request rates (per second) of the serving knee section")
    ap.add_argument("--knee-seconds", type=float, default=8.0)
    ap.add_argument("--knee-grace", type=float, default=4.0)
    ap.add_argument("--large-steps", type=int, default=256)
    ap.add_argument("--time-steps", type=int, default=None,
                    help="shorter runs for profiling under ncu (the line is then not a bench "
                         "number and says so in config.time_steps)")
    args = ap.parse_args()
    args.extra = [x for x in args.extra.split(",") if x]
    if args.time_steps:
        global T
        T = int(args.time_steps)
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
