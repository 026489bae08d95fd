"""The reference's uncalled per-step variants, on the GPU (``fdtdpic_variant_run``).

BaseFDTD11.py defines update functions that no integrator calls (their call sites in
Solver_Engine.py are commented out, or there are none):

* ``MUR1DEx`` (BaseFDTD11.py:769-788): first-order Mur update of the four cells after the left
  edge and the five before the right edge, from the field two steps back (``tempTempVarE``);
  commented-out calls after the H update, Solver_Engine.py:187, 318, 321.
* ``ADE_JxUpdate`` (:543-563): the polarisation current from three polarisation levels;
  commented-out calls after the E update, Solver_Engine.py:244, 302.  It reads
  ``V.omega_0``, which the reference's ``Variables`` does not have, so as shipped it raises;
  here the value is a row field (``omega0_j``).
* Varin's explicit nonlinear ADE (:567-607): ``ADE_NonLin_Pol_Ex_Pbar`` (the instantaneous
  polarisation Pbar3 from E and the Raman state Q), ``ADE_Lin_Curr_And_Pol_Varin`` (Lorentz
  current J and polarisation P driven by Pbar3) and ``ADE_Nonlin_Q_and_G`` (the Raman
  oscillator G, Q driven by E^2).  ``varin_step`` does all three for each cell in one pass.

Arrays are CUDA tensors of shape (rows, stride) -- one grid per row, float32 or float64, all of
one dtype -- updated in place.  Row parameters (``rows``) give each grid its size, slab and
constants.  FP64 gives the reference functions' values; FP32 rounds the same operations in
float.  :mod:`fdtdpic.compat.BaseFDTD11` has the reference-named wrappers taking ``(V, P, ...)``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import (F32, F64, VAR_ADE_JX, VAR_MUR_EX, VAR_VARIN_JP, VAR_VARIN_PBAR, VAR_VARIN_QG,
                   VAR_VARIN_STEP, VARIANT_DTYPE, VARIANT_FIELDS, FdtdPicError, check, lib)
from .engine import _ptr, _require_cuda

_N_ARRAYS = {VAR_MUR_EX: 2, VAR_ADE_JX: 4, VAR_VARIN_PBAR: 3, VAR_VARIN_JP: 3, VAR_VARIN_QG: 3,
             VAR_VARIN_STEP: 6}


def make_rows(n, nz, front, rear, *, dt, dz, eps0, c0=299792458.0, **constants) -> np.ndarray:
    """FdtdVariantRow records (numpy, ``VARIANT_DTYPE``): scalars broadcast over the rows,
    arrays give one value per row.  ``constants``: plasma_freq, omega0, gamma, omega0_j, chi1,
    chi3, alpha3, nl_gamma, nl_omega0 (missing ones are 0)."""
    unknown = set(constants) - set(VARIANT_FIELDS)
    if unknown:
        raise TypeError(f"unknown row fields: {sorted(unknown)}")
    cols = dict(n=n, nz=nz, front=front, rear=rear, c0=c0, dt=dt, dz=dz, eps0=eps0, **constants)
    m = max(np.size(v) for v in cols.values())
    rec = np.zeros(m, VARIANT_DTYPE)
    for k, v in cols.items():
        rec[k] = v
    return rec


class Rows:
    """Row records on the host (checked by the library at each call) and their device copy."""

    def __init__(self, records: np.ndarray, device=None):
        _require_cuda()
        self.host = np.ascontiguousarray(records, VARIANT_DTYPE)
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.device = torch.from_numpy(self.host.view(np.uint8).copy()).to(dev)

    def __len__(self):
        return len(self.host)


def run(op: int, rows: Rows, arrays, stream=None):
    """Apply variant ``op`` (fdtdpic._lib.VAR_*) to ``rows`` over ``arrays`` (the operation's
    tensors in the order of include/fdtdpic.h), in place, asynchronously on the stream."""
    L = lib()
    want = _N_ARRAYS.get(op)
    if want is None:
        raise ValueError(f"unknown variant operation {op}")
    if len(arrays) != want:
        raise ValueError(f"operation {op} takes {want} arrays, got {len(arrays)}")
    t0 = arrays[0]
    if t0.dtype not in (torch.float32, torch.float64):
        raise TypeError("arrays must be float32 or float64")
    for t in arrays:
        if not t.is_cuda or t.dtype != t0.dtype or t.dim() != 2 or not t.is_contiguous():
            raise ValueError("arrays must be contiguous 2-D CUDA tensors of one dtype")
        if t.shape != t0.shape:
            raise ValueError("arrays must have one shape (rows, stride)")
    if t0.shape[0] != len(rows):
        raise ValueError(f"{t0.shape[0]} array rows for {len(rows)} row records")
    prec = F64 if t0.dtype == torch.float64 else F32
    ptrs = (ctypes.c_void_p * want)(*[t.data_ptr() for t in arrays])
    st = ctypes.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    check(L.fdtdpic_variant_run(op, prec, len(rows), rows.host.ctypes.data, _ptr(rows.device),
                                int(t0.shape[1]), ctypes.cast(ptrs, ctypes.c_void_p), st),
          "fdtdpic_variant_run")


def check_rows(op: int, records: np.ndarray, stride: int) -> bool:
    """Whether the library accepts these rows for ``op`` (host-only; no device needed)."""
    rec = np.ascontiguousarray(records, VARIANT_DTYPE)
    try:
        check(lib().fdtdpic_variant_check(op, len(rec), rec.ctypes.data, int(stride)))
    except FdtdPicError:
        return False
    return True


def mur_ex(ex, ex_prev2, rows: Rows, stream=None):
    """MUR1DEx: Ex's edge cells from Ex and the field two steps back."""
    run(VAR_MUR_EX, rows, [ex, ex_prev2], stream)


def ade_jx(jx, pol, pol_prev, pol_prev2, rows: Rows, stream=None):
    """ADE_JxUpdate: Jx over [front-1, rear) from P^(n+1), P^n, P^(n-1)."""
    run(VAR_ADE_JX, rows, [jx, pol, pol_prev, pol_prev2], stream)


def varin_pbar(pbar3, ex, qx3, rows: Rows, stream=None):
    """ADE_NonLin_Pol_Ex_Pbar: Pbar3 over [front, rear)."""
    run(VAR_VARIN_PBAR, rows, [pbar3, ex, qx3], stream)


def varin_jp(jx, pol, pbar3, rows: Rows, stream=None):
    """ADE_Lin_Curr_And_Pol_Varin: J, then P, over [front, rear)."""
    run(VAR_VARIN_JP, rows, [jx, pol, pbar3], stream)


def varin_qg(gx3, qx3, ex, rows: Rows, stream=None):
    """ADE_Nonlin_Q_and_G: G, then Q, over [front, rear)."""
    run(VAR_VARIN_QG, rows, [gx3, qx3, ex], stream)


def varin_step(pbar3, jx, pol, gx3, qx3, ex, rows: Rows, stream=None):
    """varin_pbar, varin_jp and varin_qg in one pass over the cells (the same values)."""
    run(VAR_VARIN_STEP, rows, [pbar3, jx, pol, gx3, qx3, ex], stream)
