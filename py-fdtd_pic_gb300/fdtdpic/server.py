"""Serving sweep requests with continuous batching.

A request is one grid run (any size, any step count) with an optional electron beam.  The
server keeps every admitted request's fields and particles resident in HBM and advances all of
them together in *rounds*: one launch of ``fdtdpic_slots_run`` whose work items are chunks of
the active requests' steps, one CTA per item (include/fdtdpic.h).  Between rounds it admits
waiting requests into free slots as HBM budget allows and retires the ones whose last chunk
ran.  Chunk lengths come from a per-step cost model so that every item takes about the same
time; a short request therefore finishes in a few rounds while long ones keep running beside
it, and a request that arrives mid-run joins at the next round.  Rounds are enqueued ahead of
the GPU (at most ``max_inflight`` at a time); the host only waits for a round to read back the
probes of the requests that finished in it.

A beam request whose predicted work would hold one CTA for longer than ``big_ms`` runs instead
on the streaming PIC kernels (``fdtdpic_run``: every SM on its push, field and re-binning
steps, CUDA-graph blocks), on a low-priority side stream beside the rounds, which keep a
high-priority stream; the two paths give the same results bit for bit.

Results do not depend on the mix: a request's arithmetic is fixed by its own inputs and chunk
boundaries, and beam deposits are exact integer sums.

No counterpart in the reference, which runs one simulation per ``Controller`` call
(MasterController.py:451-469) and sweeps by looping over them (``LoopedSim``, :530-600).
"""
from __future__ import annotations

import collections
import ctypes
import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import physics_setup as ps
from ._lib import F64, INSTANCE_DTYPE, STATE_ARRAYS, check, lib
from .engine import _dtype, _require_cuda
from .grid import Grid, lorentz_kerr_grid, pack
from .pic import C0, Beam, PicBeam, PicRun, beam_constants

_PTR = "<u8"
SLOT_DTYPE = np.dtype([
    ("inst", INSTANCE_DTYPE), ("pml_tab", _PTR), ("src", _PTR), ("state", _PTR),
    ("probe", _PTR), ("hist", _PTR), ("n_part", "<i4"), ("clo", "<i4"), ("chi", "<i4"),
    ("reserved", "<i4"), ("cell", _PTR), ("frac", _PTR), ("ux", _PTR), ("uz", _PTR),
    ("hyp", _PTR), ("jx", _PTR), ("jz", _PTR), ("acc", _PTR), ("kE", "<f8"), ("kH", "<f8"),
    ("sc", "<f8"), ("kJ", "<f8"), ("kJz", "<f8"), ("jscale", "<f8"), ("status", "<i4", (4,)),
], align=True)
ITEM_DTYPE = np.dtype([("slot", "<i4"), ("t0", "<i4"), ("t1", "<i4"), ("first", "<i4")])


def check_slot_layout(L=None):
    L = L or lib()
    n = L.fdtdpic_slot_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_slot_layout(out.ctypes.data, n)
    names = ["inst", "pml_tab", "src", "state", "probe", "hist", "n_part", "clo", "chi",
             "reserved", "cell", "frac", "ux", "uz", "hyp", "jx", "jz", "acc", "kE", "kH", "sc",
             "kJ", "kJz", "jscale", "status"]
    want = [SLOT_DTYPE.itemsize] + [SLOT_DTYPE.fields[f][1] for f in names] + [ITEM_DTYPE.itemsize]
    if list(out) != want:
        raise RuntimeError(f"FdtdSlot layout mismatch: C {list(out)} vs numpy {want}")


@dataclass
class Request:
    """One run to serve: a grid, an optional beam (with its physical constants), an arrival
    time on the server's clock.  ``grid_fn``/``beam_fn`` build the grid/beam when the request
    is admitted (a stream of many requests then costs nothing until they run); ``nz``,
    ``n_steps``, ``n_part`` describe them before that."""
    grid: Grid | None = None
    beam: Beam | None = None
    dz: float = 0.015
    dt: float = 0.0
    mu0: float = 4e-7 * math.pi
    arrival: float = 0.0
    rid: int = -1
    grid_fn: object = None
    beam_fn: object = None
    nz: int = 0
    n_steps: int = 0
    n_part: int = 0
    pml: int = 20

    def __post_init__(self):
        if self.grid is not None:
            self.nz, self.n_steps, self.pml = self.grid.nz, self.grid.n_steps, self.grid.pml
        if self.beam is not None:
            self.n_part = self.beam.n


@dataclass
class Done:
    rid: int
    arrival: float
    admitted: float
    finished: float
    probes: np.ndarray
    status: np.ndarray
    fields: dict | None = None
    particles: dict | None = None
    error: str | None = None  # None: ran to completion with a clean status word

    @property
    def latency(self):
        return self.finished - self.arrival


class _Rejected(ValueError):
    """A request the library's slot check refused."""


@dataclass
class _Big:
    """A beam request running on the streaming kernels (side stream), a segment of steps at a
    time; `snap` holds it on the host while it is parked."""
    req: Request
    run: object
    done_ev: object
    nbytes: int
    admitted: float
    stream: object = None
    snap: object = None
    preempt: bool = False


@dataclass
class _Active:
    req: Request
    slot: int
    bufs: dict
    nbytes: int
    next_step: int
    cost_ns: float  # predicted ns per step for one CTA
    admitted: float
    outs: dict = field(default_factory=dict)
    cancelled: bool = False


class Server:
    """Continuous-batching server on one GPU.

    precision: "f32" (default) or "f64"; hbm_budget: bytes of request buffers held at once;
    max_active: requests resident at once (default 2 x the CTAs one round runs); chunk_ms: the
    target duration of one work item; keep_state: also return final fields and particles;
    big_ms: beam requests predicted to hold one CTA longer than this run on the streaming
    kernels (None: never), at most max_big at a time while no request waits for a slot and at
    most max_big_busy while some do.  Each streaming run is latency-bound and holds few SMs, so
    several share an otherwise idle GPU (on GB300 the served stream's knee moved from 4 to 8 req/s
    going from 2 to 8 concurrent runs, 16 gained nothing), but under overload eight starved the
    slot rounds (12.8 instead of ~200 req/s completed), hence the lower limit then.

    Failures retire the request with ``Done.error`` set and leave the others untouched: a
    request whose preparation raised ("prepare: ..."), one cancelled with :meth:`cancel`
    ("cancelled"), one whose buffers could not be allocated while nothing else held memory
    ("out of device memory"; with other requests resident it waits for them to retire and is
    tried again), one whose kernel flagged a status bit ("status: ...")."""

    def __init__(self, precision="f32", hbm_budget=150e9, max_active=None, chunk_ms=3.0,
                 threads=512, smem_bytes=64 * 1024, max_inflight=2, keep_state=False,
                 max_admit_per_poll=64, prefetch=128, device=None, clock=time.perf_counter,
                 big_ms=100.0, max_big=8, max_big_busy=2, fault_hook=None, big_segment=4096):
        _require_cuda()
        self.L = lib()
        check_slot_layout(self.L)
        self.prec, self.tdt = _dtype(precision)
        self.W = 2 if self.prec == F64 else 1
        self.dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.budget = float(hbm_budget)
        self.threads = threads
        self.smem = int(smem_bytes)
        self.ctas = int(self.L.fdtdpic_slots_grid(self.prec, self.smem, threads))
        if self.ctas <= 0:
            raise ValueError(f"no slot kernel launch fits threads={threads}, smem={smem_bytes}")
        self.max_active = int(max_active or 2 * self.ctas)
        self.chunk_ns = chunk_ms * 1e6
        self.max_inflight = max_inflight
        self.max_admit = max_admit_per_poll
        self.big_ns = None if big_ms is None else float(big_ms) * 1e6
        self.max_big = max(1, int(max_big))
        self.max_big_busy = max(1, min(self.max_big, int(max_big_busy)))
        self.a_cell, self.a_cell_global, self.a_part = 2.5, 6.0, 4.0
        self.keep_state = keep_state
        self.clock = clock
        # fault_hook(stage, req), if given, runs before a request's device buffers are
        # allocated (stage "alloc"); an exception it raises is handled exactly as a failed
        # allocation (tests inject out-of-memory this way, on the host)
        self.fault_hook = fault_hook
        self.cancelled: set = set()
        self.oom_retries = 0
        # streaming runs advance big_segment steps per enqueue; at each segment's end a run is
        # parked on the host (PicRun.snapshot, its device memory released) when more runs hold
        # the GPU than the current streaming limit allows, or when preempt() asked for it, and
        # resumed (PicRun.restore) ahead of new streaming admissions -- bit for bit the run it
        # would have been
        self.big_segment = max(1, int(big_segment))
        self.parked: collections.deque = collections.deque()
        self.preemptions = 0
        # rounds on a high-priority stream; each streaming-kernel request on a low-priority
        # stream of its own (its set-up's copies then wait for nothing else)
        self.stream = torch.cuda.Stream(device=self.dev, priority=-1)
        self.big: list[_Big] = []
        n = self.max_active
        self.h_slots = torch.zeros(n * SLOT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        self.slots_np = self.h_slots.numpy().view(SLOT_DTYPE)
        self.d_slots = torch.zeros(n * SLOT_DTYPE.itemsize, dtype=torch.uint8, device=self.dev)
        self.d_queue = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.free = list(range(n - 1, -1, -1))
        self.active: dict[int, _Active] = {}
        # admission pipeline: submitted -> prepared on the host by a worker thread (grid, beam,
        # pinned staging copies) -> admitted into a slot by the scheduling thread
        self._inbox: queue.Queue = queue.Queue()
        self._ready: collections.deque = collections.deque()
        self._ready_cv = threading.Condition()
        self._prefetch = max(1, int(prefetch))
        # submitted and not yet admitted: submit() may run on another thread than the
        # scheduling one, so the count changes under a lock
        self._unadmitted = 0
        self._count_lock = threading.Lock()
        self._closing = False
        # requests for the streaming kernels are recognised on submission and prepared by a
        # second thread, at most max_big ahead, so they never hold up the rounds' requests
        self._big_inbox: queue.Queue = queue.Queue()
        self._big_ready: collections.deque = collections.deque()
        self._worker = threading.Thread(target=self._prepare_loop, daemon=True)
        self._worker.start()
        self._big_worker = threading.Thread(target=self._prepare_big_loop, daemon=True)
        self._big_worker.start()
        self.bytes_in_use = 0
        self.inflight: collections.deque = collections.deque()
        self.done: list[Done] = []
        # cost model: ns per step per CTA = a_cell * (nz+1) * (1 or global factor) + a_part * np
        # (constants set above, before the preparation threads start)
        self.scale = 1.0
        self.rounds = 0
        self.cell_steps = 0.0
        self.particle_steps = 0.0
        self.gpu_ms = 0.0
        self._items_pin = [torch.zeros(n * ITEM_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
                           for _ in range(max_inflight + 1)]
        self._items_dev = [torch.zeros(n * ITEM_DTYPE.itemsize, dtype=torch.uint8,
                                       device=self.dev) for _ in range(max_inflight + 1)]
        self._ring = 0

    # ---- sizes and costs --------------------------------------------------------------------
    def request_bytes(self, req: Request) -> int:
        return slot_request_bytes(self.prec, req.nz, req.n_steps, req.n_part, req.pml)

    def big_request_bytes(self, req: Request) -> int:
        return streaming_request_bytes(self.prec, req.nz, req.n_steps, req.n_part, req.pml,
                                       self.L)

    def _step_cost_ns(self, g: Grid, n_part: int) -> float:
        resident = n_part == 0 and self._resident_bytes(g) <= self.smem
        a = self.a_cell if resident else self.a_cell_global
        slab = max(0, g.rear - g.front)
        return self.scale * (a * (g.nz + 1 + 4 * slab) + self.a_part * n_part) + 200.0

    def _resident_bytes(self, g: Grid) -> int:
        d = g.descriptor()
        return int(self.L.fdtd1d_resident_smem_bytes(np.ascontiguousarray(d).ctypes.data,
                                                      self.prec) or (1 << 40))

    # ---- admission ----------------------------------------------------------------------------
    @property
    def pending(self) -> int:
        """Requests submitted and not yet admitted."""
        return self._unadmitted

    def _count(self, d: int):
        with self._count_lock:
            self._unadmitted += d

    def submit(self, req: Request):
        """Queue a request (any thread)."""
        self._count(1)
        self._inbox.put(req)

    def cancel(self, rid: int):
        """Cancel request ``rid``.  A request not yet admitted is dropped when it reaches
        admission; one in a slot is retired after the rounds already enqueued for it (its
        probes then hold the steps run so far); a streaming run already enqueued runs out and
        its result is discarded.  Each is reported with ``error="cancelled"``."""
        self.cancelled.add(rid)

    def _fail(self, req: Request, now: float, error: str):
        """Retire a request that never ran."""
        self.done.append(Done(rid=req.rid, arrival=req.arrival, admitted=now, finished=now,
                              probes=np.zeros((0, 2)), status=np.zeros(4, np.int32),
                              error=error))

    def close(self):
        """Stop the preparation threads (pending requests are dropped) and wait for the work
        already enqueued on the GPU."""
        self._closing = True
        self._inbox.put(None)
        self._big_inbox.put(None)
        with self._ready_cv:
            self._ready_cv.notify_all()
        for t in (self._worker, self._big_worker):
            t.join(timeout=30.0)
        for b in self.big:
            b.done_ev.synchronize()
        self.stream.synchronize()

    def _is_big(self, req: Request) -> bool:
        """A beam request whose predicted work would hold one CTA longer than big_ms (from its
        sizes alone, so it is known on submission)."""
        if self.big_ns is None or not req.n_part:
            return False
        per_step = self.a_part * req.n_part + self.a_cell_global * (req.nz + 1)
        return per_step * req.n_steps > self.big_ns

    def _prepare_big_loop(self):
        while True:
            req = self._big_inbox.get()
            if req is None:
                return
            with self._ready_cv:
                while len(self._big_ready) >= self.max_big and not self._closing:
                    self._ready_cv.wait(0.05)
            try:
                if req.grid is None:
                    req.grid = req.grid_fn()
                if req.beam is None and req.beam_fn is not None:
                    req.beam = req.beam_fn()
                req._host, req._error = None, None
            except Exception as e:  # reported when the request reaches admission
                req._host, req._error = None, e
            with self._ready_cv:
                self._big_ready.append(req)
                self._ready_cv.notify_all()

    def _prepare_loop(self):
        ts = 8 if self.prec == F64 else 4
        tdt_np = np.float64 if self.prec == F64 else np.float32
        while True:
            req = self._inbox.get()
            if req is None:
                return
            if self._is_big(req):
                self._big_inbox.put(req)
                continue
            with self._ready_cv:
                while len(self._ready) >= self._prefetch and not self._closing:
                    self._ready_cv.wait(0.05)
            try:
                if req.grid is None:
                    req.grid = req.grid_fn()
                if req.beam is None and req.beam_fn is not None:
                    req.beam = req.beam_fn()
                pk = pack([req.grid], ts)
                host = dict(desc=pk["desc"][0].copy(), n_state=pk["n_state"],
                            n_probe=pk["n_probe"],
                            table=torch.from_numpy(pk["table"]).pin_memory(),
                            src=torch.from_numpy(pk["src"]).pin_memory())
                b = req.beam
                if b is not None and b.n > 0:
                    for k, a, dt_ in (("cell", b.cell, np.int32), ("frac", b.frac, tdt_np),
                                      ("ux", b.ux, tdt_np), ("uz", b.uz, tdt_np)):
                        host[k] = torch.from_numpy(np.ascontiguousarray(a, dtype=dt_)).pin_memory()
                req._host = host
                req._error = None
            except Exception as e:  # reported when the request reaches admission
                req._host, req._error = None, e
            with self._ready_cv:
                self._ready.append(req)
                self._ready_cv.notify_all()

    def _admit(self, now):
        """Admit prepared requests in arrival order while budget allows: streaming-kernel
        requests while fewer than max_big run, the others while slots are free."""
        admitted = 0
        self._resume_parked(now)
        big_limit = streaming_limit(bool(self._ready), bool(self.free), self.max_big,
                                    self.max_big_busy)
        while len(self.big) < big_limit:
            with self._ready_cv:
                if not self._big_ready:
                    break
                req = self._big_ready[0]
                need = self.big_request_bytes(req)
                if not (req._error is not None or req.rid in self.cancelled or
                        fits_budget(self.bytes_in_use, need, self.budget,
                                    bool(self.active or self.big))):
                    break
                self._big_ready.popleft()
                self._ready_cv.notify_all()
            if not self._admit_one(req, need, now, big=True):
                break
            admitted += 1
        while self.free and admitted < self.max_admit:
            with self._ready_cv:
                if not self._ready:
                    break
                req = self._ready[0]
                need = self.request_bytes(req)
                if not (req._error is not None or req.rid in self.cancelled or
                        fits_budget(self.bytes_in_use, need, self.budget,
                                    bool(self.active or self.big))):
                    break
                self._ready.popleft()
                self._ready_cv.notify_all()
            if not self._admit_one(req, need, now, big=False):
                break
            admitted += 1
        return admitted

    def _admit_one(self, req: Request, need: int, now: float, big: bool) -> bool:
        """Place one request taken off a ready queue.  False when its allocation failed while
        other requests hold memory: it goes back to the head of its queue to wait for them."""
        self._count(-1)
        if req._error is not None:
            self._fail(req, now, f"prepare: {type(req._error).__name__}: {req._error}")
            return True
        if req.rid in self.cancelled:
            self.cancelled.discard(req.rid)
            self._fail(req, now, "cancelled")
            return True
        try:
            if self.fault_hook is not None:
                self.fault_hook("alloc", req)
            (self._place_big if big else self._place)(req, need, now)
            return True
        except _Rejected as e:
            self._fail(req, now, str(e))
            return True
        except (torch.cuda.OutOfMemoryError, MemoryError) as e:
            if self.active or self.big or self.inflight:
                self.oom_retries += 1
                self._count(1)
                with self._ready_cv:
                    (self._big_ready if big else self._ready).appendleft(req)
                return False
            self._fail(req, now, f"out of device memory: {e}")
            return True

    def _place_big(self, req: Request, need: int, now: float, parked: _Big = None):
        """Run a beam request on the streaming kernels, on a low-priority stream of its own, a
        segment of steps per enqueue (graph blocks of 64 steps); a parked run is restored from
        its snapshot first."""
        g = req.grid
        req._host = None
        st = torch.cuda.Stream(device=self.dev, priority=0)
        with torch.cuda.stream(st):
            run = PicRun(g, req.beam, req.dz, req.dt, req.mu0,
                         precision="f64" if self.prec == F64 else "f32", path="streaming",
                         device=self.dev)
            if parked is not None:
                run.restore(parked.snap)
            run.step(self.big_segment, stream=st)
            ev = torch.cuda.Event()
            ev.record(st)
        self.bytes_in_use += need
        if parked is None:
            self.big.append(_Big(req=req, run=run, done_ev=ev, nbytes=need, admitted=now,
                                 stream=st))
        else:
            parked.run, parked.done_ev, parked.stream, parked.snap = run, ev, st, None
            parked.nbytes, parked.preempt = need, False
            self.big.append(parked)

    def preempt(self, rid: int) -> bool:
        """Park streaming run ``rid`` at the end of its current segment (snapshot to the host,
        device memory released); it resumes when the streaming limit allows.  False when no
        such run is active."""
        for b in self.big:
            if b.req.rid == rid:
                b.preempt = True
                return True
        return False

    def _park(self, b: _Big):
        b.snap = b.run.snapshot()  # synchronises the device; the segment has run
        b.run = None
        b.done_ev = None
        self.bytes_in_use -= b.nbytes
        self.big.remove(b)
        self.parked.append(b)
        self.preemptions += 1

    def _resume_parked(self, now):
        """Parked runs come back, oldest first, while the streaming limit and budget allow."""
        limit = streaming_limit(bool(self._ready), bool(self.free), self.max_big,
                                self.max_big_busy)
        while self.parked and len(self.big) < limit:
            b = self.parked[0]
            need = self.big_request_bytes(b.req)
            if not fits_budget(self.bytes_in_use, need, self.budget, bool(self.active or self.big)):
                break
            self.parked.popleft()
            try:
                self._place_big(b.req, need, now, parked=b)
            except (torch.cuda.OutOfMemoryError, MemoryError):
                self.parked.appendleft(b)
                break

    def _complete_big(self, block=False):
        """Retire streaming-kernel requests whose work has run (the oldest first when
        blocking)."""
        n = 0
        limit = streaming_limit(bool(self._ready), bool(self.free), self.max_big,
                                self.max_big_busy)
        for b in list(self.big):
            if not b.done_ev.query():
                if not block or n:
                    continue
                b.done_ev.synchronize()
            run, g = b.run, b.req.grid
            if run.step_done < g.n_steps and b.req.rid not in self.cancelled:
                # a segment ended: park it (asked for, or more runs than the limit allows: the
                # youngest go first), or enqueue its next segment
                over = len(self.big) > limit and b is self.big[-1]
                if b.preempt or over:
                    self._park(b)
                    continue
                with torch.cuda.stream(b.stream):
                    run.step(self.big_segment, stream=b.stream)
                    b.done_ev = torch.cuda.Event()
                    b.done_ev.record(b.stream)
                continue
            self.big.remove(b)
            st = run.status()
            status = np.zeros(4, np.int32)
            status[:2] = st[:2]
            fields = parts = None
            if self.keep_state:
                f = run.fields()
                jx, jz = run.currents()
                fields = dict(Ex=f["Ex"], Hy=f["Hy"], Jx=jx, Jz=jz)
                cell, frac, ux, uz = run.particles()
                parts = dict(cell=cell, frac=frac, ux=ux, uz=uz)
            cancelled = b.req.rid in self.cancelled
            self.cancelled.discard(b.req.rid)
            self.done.append(Done(rid=b.req.rid, arrival=b.req.arrival, admitted=b.admitted,
                                  finished=self.clock(), probes=run.probes(), status=status,
                                  fields=None if cancelled else fields,
                                  particles=None if cancelled else parts,
                                  error="cancelled" if cancelled else status_error(status)))
            self.cell_steps += (g.nz + 1) * g.n_steps
            self.particle_steps += b.req.n_part * g.n_steps
            self.bytes_in_use -= b.nbytes
            b.run = None
            n += 1
        return n

    def _place(self, req: Request, need: int, now: float):
        g = req.grid
        host = req._host
        tdt, dev = self.tdt, self.dev
        n = g.nz + 1
        slot = self.free.pop()
        try:
            with torch.cuda.stream(self.stream):
                desc = host["desc"]
                desc["step_begin"], desc["step_end"], desc["resume"] = 0, g.n_steps, 0
                bufs = dict(table=host["table"].to(dev, non_blocking=True),
                            src=host["src"].to(dev, non_blocking=True),
                            state=torch.empty(host["n_state"], dtype=tdt, device=dev),
                            probe=torch.zeros(host["n_probe"], dtype=tdt, device=dev))
                s = self.slots_np[slot:slot + 1]  # a view: assignments land in the pinned table
                s[...] = np.zeros(1, SLOT_DTYPE)
                s["inst"] = desc
                s["pml_tab"], s["src"] = bufs["table"].data_ptr(), bufs["src"].data_ptr()
                s["state"], s["probe"] = bufs["state"].data_ptr(), bufs["probe"].data_ptr()
                n_part = 0
                if "cell" in host:
                    b = req.beam
                    n_part = b.n
                    bufs.update(cell=host["cell"].to(dev, non_blocking=True),
                                frac=host["frac"].to(dev, non_blocking=True),
                                ux=host["ux"].to(dev, non_blocking=True),
                                uz=host["uz"].to(dev, non_blocking=True),
                                hyp=torch.empty(n, dtype=tdt, device=dev),
                                jx=torch.empty(n, dtype=tdt, device=dev),
                                jz=torch.empty(n, dtype=tdt, device=dev),
                                acc=torch.empty(2 * self.W * n, dtype=torch.int64, device=dev))
                    pb = PicBeam()
                    pb.n_part, pb.clo, pb.chi = b.n, b.clo, b.chi
                    consts = beam_constants(req.dz, req.dt, b.weight, req.mu0)
                    for k, v in consts.items():
                        setattr(pb, k, v)
                    jscale = self.L.fdtdpic_pic_jscale(ctypes.byref(pb))
                    s["n_part"], s["clo"], s["chi"] = b.n, b.clo, b.chi
                    for k in ("cell", "frac", "ux", "uz", "hyp", "jx", "jz", "acc"):
                        s[k] = bufs[k].data_ptr()
                    for k, v in consts.items():
                        s[k] = v
                    s["jscale"] = jscale
                rc = self.L.fdtdpic_slot_check(self.prec, s.ctypes.data)
                if rc != 0:
                    raise _Rejected(f"rejected by fdtdpic_slot_check ({rc})")
                sz = SLOT_DTYPE.itemsize
                self.d_slots[slot * sz:(slot + 1) * sz].copy_(
                    self.h_slots[slot * sz:(slot + 1) * sz], non_blocking=True)
        except BaseException:
            self.free.append(slot)  # nothing of this request was handed to a round
            raise
        req._host = None  # the staging copies are released once the copies have run
        self.bytes_in_use += need
        self.active[slot] = _Active(req=req, slot=slot, bufs=bufs, nbytes=need, next_step=0,
                                    cost_ns=self._step_cost_ns(g, n_part), admitted=now)

    # ---- rounds ---------------------------------------------------------------------------------
    def _round(self, now):
        if not self.active:
            return False
        items = []
        finishing = []
        pred_ns = 0.0
        work = [0.0, 0.0]  # cell-steps, particle-steps of this round
        cancelled = []
        for slot, a in self.active.items():
            g = a.req.grid
            if a.req.rid in self.cancelled:
                # retired behind the rounds already enqueued for it; no new items
                a.cancelled = True
                cancelled.append(a)
                continue
            if a.next_step >= g.n_steps:
                continue
            k = max(1, int(self.chunk_ns / max(a.cost_ns, 1.0)))
            t0 = a.next_step
            t1 = min(g.n_steps, t0 + k)
            items.append((slot, t0, t1, 1 if t0 == 0 else 0))
            pred_ns += a.cost_ns * (t1 - t0)
            work[0] += (g.nz + 1) * (t1 - t0)
            work[1] += a.req.n_part * (t1 - t0)
            a.next_step = t1
            if t1 >= g.n_steps:
                finishing.append(a)
        finishing += cancelled
        if not items and not cancelled:
            return False
        # longest items first: the queue then ends with short ones
        items.sort(key=lambda it: -self.active[it[0]].cost_ns * (it[2] - it[1]))
        r = self._ring
        self._ring = (self._ring + 1) % len(self._items_pin)
        arr = self._items_pin[r].numpy().view(ITEM_DTYPE)
        for i, (slot, t0, t1, first) in enumerate(items):
            arr[i] = (slot, t0, t1, first)
        nb = len(items) * ITEM_DTYPE.itemsize
        with torch.cuda.stream(self.stream):
            self._items_dev[r][:nb].copy_(self._items_pin[r][:nb], non_blocking=True)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            if items:
                check(self.L.fdtdpic_slots_run(
                    self.prec, ctypes.c_void_p(self.d_slots.data_ptr()), self.max_active,
                    ctypes.c_void_p(self._items_dev[r].data_ptr()), len(items),
                    ctypes.c_void_p(self.d_queue.data_ptr()), self.smem, self.threads, 0,
                    ctypes.c_void_p(self.stream.cuda_stream)), "fdtdpic_slots_run")
            e1.record(self.stream)
            for a in finishing:
                a.outs["probe"] = a.bufs["probe"].to("cpu", non_blocking=True)
                sz = SLOT_DTYPE.itemsize
                a.outs["slot"] = self.d_slots[a.slot * sz:(a.slot + 1) * sz].to(
                    "cpu", non_blocking=True)
                if self.keep_state:
                    a.outs["state"] = a.bufs["state"].to("cpu", non_blocking=True)
                    for k in ("cell", "frac", "ux", "uz", "jx", "jz"):
                        if k in a.bufs:
                            a.outs[k] = a.bufs[k].to("cpu", non_blocking=True)
            done_ev = torch.cuda.Event()
            done_ev.record(self.stream)
        for a in finishing:
            del self.active[a.slot]
            self.cancelled.discard(a.req.rid)
        self.inflight.append((done_ev, e0, e1, finishing, pred_ns, len(items), work))
        self.rounds += 1 if items else 0
        return True

    def _complete(self, block=False):
        n = 0
        while self.inflight:
            ev, e0, e1, finishing, pred_ns, n_items, work = self.inflight[0]
            if not block and not ev.query():
                break
            ev.synchronize()
            self.inflight.popleft()
            now = self.clock()
            ms = e0.elapsed_time(e1)
            self.gpu_ms += ms
            self.cell_steps += work[0]
            self.particle_steps += work[1]
            # calibrate the cost model: a round lasts about its predicted work over the CTAs
            if pred_ns > 0 and n_items >= self.ctas // 2:
                ratio = (ms * 1e6) / (pred_ns / min(self.ctas, n_items))
                self.scale = min(100.0, max(0.01, 0.8 * self.scale + 0.2 * self.scale * ratio))
            for a in finishing:
                g = a.req.grid
                slot_rec = a.outs["slot"].numpy().view(SLOT_DTYPE)[0]
                fields = None
                parts = None
                if self.keep_state:
                    st = a.outs["state"].double().numpy()
                    nn = g.nz + 1
                    fields = dict(Ex=st[:nn].copy(), Hy=st[nn:2 * nn].copy())
                    if "jx" in a.outs:
                        fields.update(Jx=a.outs["jx"].double().numpy(),
                                      Jz=a.outs["jz"].double().numpy())
                    if "cell" in a.outs:
                        parts = {k: a.outs[k].numpy() for k in ("cell", "frac", "ux", "uz")}
                status = np.array(slot_rec["status"])
                self.cancelled.discard(a.req.rid)  # a cancel that came after its last round
                self.done.append(Done(
                    rid=a.req.rid, arrival=a.req.arrival, admitted=a.admitted, finished=now,
                    probes=a.outs["probe"].double().numpy().reshape(g.n_steps, 2),
                    status=status, fields=fields, particles=parts,
                    error="cancelled" if a.cancelled else status_error(status)))
                self.bytes_in_use -= a.nbytes
                self.free.append(a.slot)
                a.bufs.clear()
                n += 1
        return n

    # ---- driving --------------------------------------------------------------------------------
    def poll(self, now=None, block=False):
        """One scheduling pass: retire finished rounds, admit, enqueue a round if there is
        room in flight.  Returns the number of requests completed in this pass."""
        now = self.clock() if now is None else now
        n = self._complete(block=False) + self._complete_big(block=False)
        self._admit(now)
        while len(self.inflight) >= self.max_inflight:
            n += self._complete(block=True)
            self._admit(self.clock())
        self._round(self.clock())
        if block:
            n += self._complete(block=True)
        return n

    def drain(self):
        """Run until every submitted request has completed."""
        while self.pending or self.active or self.inflight or self.big or self.parked:
            self.poll()
            if not self.active and not self.pending:
                if self.inflight:
                    self._complete(block=True)
                else:
                    self._complete_big(block=True)
            elif not self.active and not self.inflight:
                with self._ready_cv:  # waiting for the preparation thread
                    if not self._ready:
                        self._ready_cv.wait(0.01)
        return self.done

    def run_stream(self, requests, duration):
        """Real-time run: each request is submitted when the clock reaches its arrival time
        (seconds from start); stops admitting at ``duration`` and returns the statistics of
        the requests completed by then."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t_start = self.clock()
        i = 0
        while True:
            now = self.clock() - t_start
            while i < len(reqs) and reqs[i].arrival <= now:
                r = reqs[i]
                r.arrival = t_start + r.arrival
                self.submit(r)
                i += 1
            if now >= duration:
                break
            if (not self.active and not self.pending and not self.inflight and not self.big
                    and not self.parked):
                if i >= len(reqs):
                    break
                time.sleep(min(1e-3, max(0.0, reqs[i].arrival - now)))
                continue
            self.poll()
            if not self.active and not self.inflight:
                with self._ready_cv:  # waiting for the preparation thread
                    if not self._ready:
                        self._ready_cv.wait(0.005)
        elapsed = self.clock() - t_start
        self._complete(block=False)
        return self.stats(elapsed, submitted=i)

    def stats(self, elapsed, submitted=None):
        lat = np.array([d.latency for d in self.done])
        svc = np.array([d.finished - d.admitted for d in self.done])
        pct = (lambda a, q: float(np.percentile(a, q)) if a.size else None)
        return dict(completed=len(self.done), submitted=submitted, elapsed_s=elapsed,
                    throughput_rps=len(self.done) / elapsed if elapsed > 0 else 0.0,
                    p50_s=pct(lat, 50), p99_s=pct(lat, 99), service_p50_s=pct(svc, 50),
                    service_p99_s=pct(svc, 99), queue_depth=self.pending,
                    active=len(self.active), streaming=len(self.big), rounds=self.rounds,
                    mcell_steps_per_s=self.cell_steps / elapsed / 1e6 if elapsed > 0 else 0.0,
                    mparticle_steps_per_s=self.particle_steps / elapsed / 1e6
                    if elapsed > 0 else 0.0, gpu_busy_s=self.gpu_ms / 1e3)


# ------------------------------------------------------------------------------------------
# the served request stream: Poisson arrivals, ragged grids, optional beams
# ------------------------------------------------------------------------------------------
def slot_request_bytes(prec: int, nz: int, n_steps: int, n_part: int, pml: int) -> int:
    """Device bytes a request served in a slot holds: state, probes, sources, PML table and,
    with a beam, its particles, Hy one half step back, the currents and the deposit
    accumulators."""
    ts = 8 if prec == F64 else 4
    w = 2 if prec == F64 else 1
    n = nz + 1
    b = (STATE_ARRAYS * n * ts + 2 * n_steps * ts + 2 * n_steps * 8 + 8 * (2 * pml + 1) * 8)
    if n_part:
        b += n_part * (4 + 3 * ts) + 3 * n * ts + 2 * w * n * 8
    return int(b) + 4096


def streaming_request_bytes(prec: int, nz: int, n_steps: int, n_part: int, pml: int,
                            L=None) -> int:
    """Device bytes a request run on the streaming kernels holds: the slot form's buffers
    plus particle ids, two more field-sized arrays and the streaming path's scratch
    (fdtdpic_scratch_bytes: the re-binning copy of every particle array and the deposit
    accumulators)."""
    L = L or lib()
    ts = 8 if prec == F64 else 4
    scratch = int(L.fdtdpic_scratch_bytes(prec, int(nz), int(n_part)))
    return (slot_request_bytes(prec, nz, n_steps, n_part, pml) + 4 * int(n_part) + scratch +
            2 * (nz + 1) * ts)


def fits_budget(in_use: int, need: int, budget: float, others_resident: bool) -> bool:
    """Admission rule: a request is admitted when its bytes fit what the budget leaves, or
    when nothing else is resident (a request larger than the whole budget still runs alone)."""
    return in_use + need <= budget or not others_resident


def status_error(status) -> str | None:
    """The error a request's status word reports (include/fdtdpic.h FDTD_STATUS_*), or None."""
    bits = int(status[1]) if len(status) > 1 else 0
    what = [name for bit, name in ((1, "non-finite fields"), (2, "skipped"),
                                   (4, "bounded wait gave up"), (8, "buffer overflow"))
            if bits & bit]
    if int(status[0]) > 0:
        what.append(f"{int(status[0])} particles left the grid")
    return ("status: " + ", ".join(what)) if what else None


def streaming_limit(requests_waiting: bool, slots_free: bool, max_big: int,
                    max_big_busy: int) -> int:
    """How many streaming runs big requests may hold: several use an otherwise idle GPU well,
    but while prepared requests wait for a slot, or no slot is free, the slot rounds need the
    SMs, so then at most max_big_busy."""
    return max_big_busy if (requests_waiting or not slots_free) else max_big


def make_request_stream(rate=2000.0, duration=60.0, seed=20261203, nz_lo=256, nz_hi=65536,
                        steps_lo=1000, steps_hi=50000, np_max=2_000_000, dz=0.015, sc=0.5,
                        max_requests=None):
    """Seeded stream: arrivals Poisson(rate) over [0, duration); per request
    Nz = round(exp U[ln nz_lo, ln nz_hi]), steps ~ U{steps_lo..steps_hi},
    Np = floor(exp U[0, ln(np_max + 1)]) - 1 (0 included), material as the batched sweep
    (slab width U[0.05, 0.30] Nz centred between the source and the far PML, d_eps U[0.5, 4],
    f0 U[0.8, 2.5] GHz, chi3 logU[1e-4, 1e-1]), Kerr integrator, Gaussian-modulated 1 GHz
    source at cell 100, probes at 50 and Nz-50; beam over cells [50, Nz-51), vz ~ N(0.3c,
    0.003c), density 1e14 m^-3.  Beams are generated when a request is admitted."""
    from .pic import make_beam
    rng = np.random.Generator(np.random.PCG64(seed))
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        arrivals.append(t)
        if max_requests and len(arrivals) >= max_requests:
            break
    n = len(arrivals)
    nz = np.rint(np.exp(rng.uniform(np.log(nz_lo), np.log(nz_hi), n))).astype(int)
    steps = rng.integers(steps_lo, steps_hi + 1, n)
    npart = (np.floor(np.exp(rng.uniform(0.0, np.log(np_max + 1.0), n))) - 1).astype(int)
    width = rng.uniform(0.05, 0.30, n)
    deps = rng.uniform(0.5, 4.0, n)
    f0 = rng.uniform(0.8e9, 2.5e9, n)
    chi3 = 10.0 ** rng.uniform(-4, -1, n)
    seeds = rng.integers(0, 2 ** 62, n)
    dt = sc * dz / C0
    src_cache = {}

    def grid_of(N, T, front, rear, d_eps, f, chi):
        if T not in src_cache:
            src_cache[T] = ps.gauss_sine(T, 1e9, dt)
        return lorentz_kerr_grid(N, T, dz=dz, sc=sc, front=front, rear=rear, pml=20, nzsrc=100,
                                 probes=(50, N - 50), d_eps=d_eps, f0=f, chi3=chi,
                                 source=src_cache[T])

    reqs = []
    for i in range(n):
        N, T = int(nz[i]), int(steps[i])
        pml, nzsrc = 20, 100
        w = max(1, int(round(width[i] * N)))
        centre = (nzsrc + (N - pml)) // 2
        front = max(nzsrc + 2, centre - w // 2)
        rear = max(front, min(N - pml - 2, front + w))
        r = Request(dz=dz, dt=dt, arrival=arrivals[i], rid=i, nz=N, n_steps=T, pml=pml,
                    grid_fn=(lambda N=N, T=T, fr=front, re=rear, de=float(deps[i]),
                             f=float(f0[i]), ch=float(chi3[i]): grid_of(N, T, fr, re, de, f, ch)))
        if npart[i] > 0:
            clo, chi, npi, sd = 50, N - 51, int(npart[i]), int(seeds[i])
            r.beam_fn = (lambda npi=npi, clo=clo, chi=chi, sd=sd:
                         make_beam(npi, clo, chi, dz, seed=sd, sort=False))
            r.n_part = npi
        reqs.append(r)
    return reqs
