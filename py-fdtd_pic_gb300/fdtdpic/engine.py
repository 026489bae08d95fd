"""Run grids on the GPU through the C ABI.

``run(grids, precision)`` packs any number of grids, uploads them, and runs them:
grids that fit in shared memory go into ONE launch of the resident batch kernel (persistent
CTAs pulling grids from a device work queue, longest first); larger grids run on the
global-memory path, two launches per step.  Device memory comes from PyTorch; the kernels are
the hand-written ones in libfdtdpic.so.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, INSTANCE_DTYPE, ST, check, lib
from .grid import pack


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("fdtdpic needs a CUDA device (GB300, sm_103a); none is visible")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _dtype(precision):
    if precision in (F64, "f64", "fp64", torch.float64):
        return F64, torch.float64
    if precision in (F32, "f32", "fp32", torch.float32):
        return F32, torch.float32
    raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}")


@dataclass
class Packed:
    """A batch uploaded to the device (reusable for repeated runs, e.g. benchmarks)."""
    grids: list
    prec: int
    tdtype: torch.dtype
    desc_host: np.ndarray
    d_desc: torch.Tensor
    d_table: torch.Tensor
    d_src: torch.Tensor
    d_state: torch.Tensor
    d_probe: torch.Tensor
    d_hist: torch.Tensor | None
    d_queue: torch.Tensor
    d_status: torch.Tensor
    d_fallbacks: torch.Tensor
    resident: list
    d_order: torch.Tensor | None
    smem_bytes: int
    global_idx: list


def upload(grids, precision="f64", device=None) -> Packed:
    _require_cuda()
    L = lib()
    prec, tdt = _dtype(precision)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    pk = pack(grids, 8 if prec == F64 else 4)
    desc = pk["desc"]
    smem = np.array([L.fdtd1d_resident_smem_bytes(desc[i:i + 1].ctypes.data, prec)
                     for i in range(len(grids))], np.int64)
    resident = [i for i in range(len(grids)) if smem[i] > 0]
    global_idx = [i for i in range(len(grids)) if smem[i] == 0]
    order = sorted(resident, key=lambda i: -grids[i].cost())

    def to_dev(a, dt=None):
        t = torch.from_numpy(np.ascontiguousarray(a))
        if dt is not None:
            t = t.to(dt)
        return t.pin_memory().to(dev, non_blocking=True) if t.numel() > 0 else t.to(dev)

    d_desc = to_dev(desc.view(np.uint8))
    return Packed(
        grids=list(grids), prec=prec, tdtype=tdt, desc_host=desc, d_desc=d_desc,
        d_table=to_dev(pk["table"]), d_src=to_dev(pk["src"]),
        d_state=torch.zeros(max(1, pk["n_state"]), dtype=tdt, device=dev),
        d_probe=torch.zeros(max(1, pk["n_probe"]), dtype=tdt, device=dev),
        d_hist=torch.zeros(pk["n_hist"], dtype=tdt, device=dev) if pk["n_hist"] else None,
        d_queue=torch.zeros(1, dtype=torch.int32, device=dev),
        d_status=torch.zeros(len(grids), dtype=torch.int32, device=dev),
        d_fallbacks=torch.zeros(len(grids), dtype=torch.int32, device=dev),
        resident=resident,
        d_order=torch.tensor(order, dtype=torch.int32, device=dev) if order else None,
        smem_bytes=int(smem[resident].max()) if resident else 0,
        global_idx=global_idx)


def launch(p: Packed, stream=None, threads=256, grid_ctas=0):
    """Enqueue every grid of the batch on ``stream`` (default: torch's current stream).
    :func:`upload` queues its copies and zero fills on the stream that was current then; a
    caller launching on another stream first makes it wait for that one
    (``stream.wait_stream(torch.cuda.current_stream())``)."""
    L = lib()
    st = ctypes.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    if p.resident:
        check(L.fdtd1d_run_batch(p.prec, len(p.resident), _ptr(p.d_desc), _ptr(p.d_order),
                                 _ptr(p.d_table), _ptr(p.d_src), _ptr(p.d_state),
                                 _ptr(p.d_probe), _ptr(p.d_hist), _ptr(p.d_queue),
                                 _ptr(p.d_status), _ptr(p.d_fallbacks), p.smem_bytes, threads,
                                 grid_ctas, st), "fdtd1d_run_batch")
    isz = INSTANCE_DTYPE.itemsize
    for i in p.global_idx:
        h = np.ascontiguousarray(p.desc_host[i:i + 1])
        d_inst = ctypes.c_void_p(p.d_desc.data_ptr() + i * isz)
        status = ctypes.c_void_p(p.d_status.data_ptr() + 4 * i)
        fb = ctypes.c_void_p(p.d_fallbacks.data_ptr() + 4 * i)
        check(L.fdtd1d_run_global(p.prec, h.ctypes.data, d_inst, _ptr(p.d_table), _ptr(p.d_src),
                                  _ptr(p.d_state), _ptr(p.d_probe), _ptr(p.d_hist), status, fb,
                                  st), "fdtd1d_run_global")


@dataclass
class GridResult:
    Ex: np.ndarray
    Hy: np.ndarray
    Dx: np.ndarray
    P: np.ndarray
    Pprev: np.ndarray
    psi_Ex: np.ndarray
    psi_Hy: np.ndarray
    Acubic: np.ndarray
    probes: np.ndarray  # (n_steps, 2)
    hist: np.ndarray | None
    status: int
    fallbacks: int


def download(p: Packed):
    state = p.d_state.double().cpu().numpy()
    probe = p.d_probe.double().cpu().numpy()
    hist = p.d_hist.double().cpu().numpy() if p.d_hist is not None else None
    status = p.d_status.cpu().numpy()
    fbs = p.d_fallbacks.cpu().numpy()
    out = []
    for i, g in enumerate(p.grids):
        d = p.desc_host[i]
        n = g.n
        so = int(d["state_offset"])
        arr = {k: state[so + v * n: so + (v + 1) * n].copy() for k, v in ST.items()}
        po = int(d["probe_offset"])
        ho = int(d["hist_offset"])
        out.append(GridResult(
            Ex=arr["Ex"], Hy=arr["Hy"], Dx=arr["Dx"], P=arr["P"], Pprev=arr["Pprev"],
            psi_Ex=arr["psiE"], psi_Hy=arr["psiH"], Acubic=arr["A"],
            probes=probe[po:po + 2 * g.n_steps].reshape(g.n_steps, 2).copy(),
            hist=(hist[ho:ho + g.hist_rows * n].reshape(g.hist_rows, n).copy()
                  if (hist is not None and g.hist_rows) else None),
            status=int(status[i]), fallbacks=int(fbs[i])))
    return out


def run(grids, precision="f64", threads=256, grid_ctas=0):
    """Run every grid for its [step_begin, step_end) steps; returns a GridResult per grid."""
    p = upload(grids, precision)
    launch(p, threads=threads, grid_ctas=grid_ctas)
    torch.cuda.synchronize()
    return download(p)


def cubic_root0(coef: np.ndarray) -> np.ndarray:
    """Re(roots[0]) of the reference's closed form for each row (a, b, c, d), on the GPU."""
    _require_cuda()
    c = torch.from_numpy(np.ascontiguousarray(coef, np.float64).reshape(-1, 4)).cuda()
    out = torch.empty(c.shape[0], dtype=torch.float64, device=c.device)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(lib().fdtdpic_cubic_root0(c.shape[0], _ptr(c), _ptr(out), st), "fdtdpic_cubic_root0")
    return out.cpu().numpy()
