"""``RefTester`` of TransformHandler.py:34-78: the spectral peak of a probe trace.

The reference takes ``fftpack.fft`` of the trace and keeps the largest bin of
2|Y|/timeSteps (exiting if that is the DC bin).  Here |Y| at every FFT bin comes from the
GPU DFT kernel (:func:`fdtdpic.spectrum.bin_magnitudes`).  The figures the reference draws
are not drawn.  As in the reference, ``mul`` has no effect (its early return sits inside a
string literal there).
"""
from __future__ import annotations

import sys

import numpy as np

from .. import spectrum


def RefTester(V, P, y, m, mul=False):
    """Returns (|Y| over bins N/2+10 .. N-501 scaled by 2m/N, their frequencies, peak value)."""
    y = np.asarray(y, dtype=np.float64)
    Y = spectrum.bin_magnitudes(y, P.delT)
    Ypow = (2 * Y) / P.timeSteps
    freqs = np.fft.fftfreq(len(y), d=P.delT)
    indMax = int(np.argmax(Ypow))
    if indMax != 0:
        print("Freq with largest amplitude: ", freqs[indMax])
        val = Ypow[indMax]
    else:
        print("Could not find non-DC freq")
        sys.exit()
    N = len(Y)
    lo, hi = int(N / 2) + 10, N - 500
    bob = (Y[lo:hi] * m * 2) / N
    return bob, freqs[lo:hi], val
