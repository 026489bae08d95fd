"""Spectra of probe traces on the GPU (the batched DFT kernel of libfdtdpic.so).

* :func:`dft` -- X[r, f] = sum_n x[r, n] exp(-2 pi i f n dt) for any set of frequencies.
* :func:`bin_magnitudes` -- |FFT(y)| at every bin k/(N dt) of a real trace, the quantity the
  reference's ``RefTester`` (TransformHandler.py:34-78) takes from ``fftpack.fft``.  The bins
  0..N/2 are evaluated directly and the rest mirrored (|Y_k| = |Y_{N-k}| for real input), in
  chunks of frequencies so the twiddle table stays small.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import check, lib

_CHUNK_BYTES = 256 << 20  # twiddle table budget per call


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("fdtdpic needs a CUDA device (GB300, sm_103a); none is visible")


def dft(traces, freqs, dt, stream=None) -> np.ndarray:
    """Complex spectra (R, F) of real traces (R, S) at ``freqs`` (Hz), sample spacing dt."""
    _require_cuda()
    L = lib()
    x = torch.as_tensor(np.ascontiguousarray(np.atleast_2d(traces)))
    if x.dtype not in (torch.float32, torch.float64):
        x = x.to(torch.float64)
    R, S = x.shape
    freqs = np.ascontiguousarray(np.asarray(freqs, np.float64).ravel())
    F = freqs.size
    out = np.empty((R, F), np.complex128)
    if R == 0 or F == 0:
        return out
    if S == 0:
        out[:] = 0
        return out
    st = stream or torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    # copies, launches and the read-back all on st, in order
    with torch.cuda.stream(st):
        d_x = x.cuda()
        prec = 4 if d_x.dtype == torch.float32 else 8
        per = max(1, min(F, _CHUNK_BYTES // (8 * S)))
        d_tw = torch.empty(int(L.fdtdpic_dft_twiddle_bytes(per, S)), dtype=torch.uint8,
                           device="cuda")
        d_out = torch.empty(R * per * 2, dtype=torch.float64, device="cuda")
        for f0 in range(0, F, per):
            n = min(per, F - f0)
            d_f = torch.from_numpy(freqs[f0:f0 + n].copy()).cuda()
            check(L.fdtdpic_dft_twiddles(_ptr(d_f), n, S, float(dt), _ptr(d_tw), sp),
                  "fdtdpic_dft_twiddles")
            # one trace per row: rp = 1, ldp = S, sp = 0, sn = 1
            check(L.fdtdpic_dft_probes(prec, _ptr(d_x), R, S, 1, S, 0, 1, _ptr(d_tw), n,
                                       _ptr(d_out), sp), "fdtdpic_dft_probes")
            X = d_out[:R * n * 2].cpu().numpy().reshape(R, n, 2)
            out[:, f0:f0 + n] = X[..., 0] + 1j * X[..., 1]
    return out


def bin_magnitudes(y, dt) -> np.ndarray:
    """|Y_k| for k = 0..N-1, Y = FFT of the real trace y (length N)."""
    y = np.asarray(y, np.float64).ravel()
    N = y.size
    if N == 0:
        return np.zeros(0)
    half = N // 2
    k = np.arange(half + 1)
    mag_half = np.abs(dft(y[None, :], k / (N * dt), dt)[0])
    mag = np.empty(N)
    mag[:half + 1] = mag_half
    mag[half + 1:] = mag_half[1:N - half][::-1]
    return mag
