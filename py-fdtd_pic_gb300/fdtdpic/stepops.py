"""One per-step update of the reference's module functions, one GPU launch (``fdtdpic_step_op``).

The integrators of this package fuse whole runs into a few launches.  A caller that builds its
own time loop out of the reference's module functions (``BaseFDTD11.ADE_ExUpdate``, ...) needs
their finer unit of work instead: :func:`run` takes the function's numpy arrays, runs the update
on the GPU in FP64 with the reference's operation order, and writes the arrays it changed back
in place, as the reference's functions update their ``Variables`` members in place.  The
operations and their array slots are listed in include/fdtdpic.h (FDTD_OP_*).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import check, lib
from .engine import _require_cuda

OP_CURL, OP_PSI, OP_POL, OP_EXCREATE, OP_NONLIN_EX, OP_ACUBIC = range(6)
N_SLOTS = 8
MUL, DIV = 1, 2


class FdtdStepOp(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("lo", ctypes.c_int32), ("hi", ctypes.c_int32),
                ("xa", ctypes.c_int32), ("xb", ctypes.c_int32), ("fmode", ctypes.c_int32 * 3),
                ("fval", ctypes.c_double * 3), ("s", ctypes.c_double * 4)]


_checked = False


def check_layout(L=None):
    """The ctypes struct against the library's FdtdStepOp."""
    L = L or lib()
    n = L.fdtdpic_step_op_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_step_op_layout(out.ctypes.data, n)
    want = [ctypes.sizeof(FdtdStepOp)] + [getattr(FdtdStepOp, f).offset for f in
                                          ("op", "lo", "hi", "xa", "xb", "fmode", "fval", "s")]
    if list(out) != want:
        raise RuntimeError(f"FdtdStepOp layout mismatch: C {list(out)} vs ctypes {want}")


def make_op(op, lo, hi, xa=0, xb=0, fmode=(0, 0, 0), fval=(0.0, 0.0, 0.0), s=(0.0, 0.0, 0.0, 0.0)):
    o = FdtdStepOp()
    o.op, o.lo, o.hi, o.xa, o.xb = int(op), int(lo), int(hi), int(xa), int(xb)
    for i in range(3):
        o.fmode[i] = int(fmode[i])
        o.fval[i] = float(fval[i])
    for i, v in enumerate(s):
        o.s[i] = float(v)
    return o


def run(op: FdtdStepOp, slots, writes, stream=None):
    """Run ``op`` over ``slots`` (numpy arrays of equal length, or None where the operation
    allows it).  Each distinct array goes to the device once (an array named in two slots is one
    device buffer, as it is one object in the reference); the slots in ``writes`` are copied back
    into their numpy arrays in place.  Synchronous (the results are on the host on return)."""
    global _checked
    _require_cuda()
    L = lib()
    if not _checked:
        check_layout(L)
        _checked = True
    arrs = [a for a in slots if a is not None]
    if not arrs:
        raise ValueError("an operation needs arrays")
    n = len(arrs[0])
    if any(len(a) != n for a in arrs):
        raise ValueError("the arrays of one operation have the same length")
    dev = torch.device("cuda", torch.cuda.current_device())
    bufs = {}
    ptrs = (ctypes.c_void_p * N_SLOTS)()
    dslot = [None] * N_SLOTS
    st = stream or torch.cuda.current_stream()
    # copies in, the launch and the copies back all on st, in order
    with torch.cuda.stream(st):
        for i, a in enumerate(slots):
            if a is None:
                continue
            key = id(a)
            if key not in bufs:
                bufs[key] = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
            dslot[i] = bufs[key]
            ptrs[i] = bufs[key].data_ptr()
        check(L.fdtdpic_step_op(ctypes.byref(op), ptrs, n, ctypes.c_void_p(st.cuda_stream)),
              "fdtdpic_step_op")
        done = set()
        for i in writes:
            a = slots[i]
            if a is None or id(a) in done:
                continue
            a[...] = dslot[i].cpu().numpy()
            done.add(id(a))
