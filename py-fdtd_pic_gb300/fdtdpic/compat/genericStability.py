"""``spatialStab`` of genericStability.py:12-62: the numerical-dispersion rescale of the plasma
frequency; returns (lamCont, lamDisc, diff, plasmaFreq', fix)."""
from __future__ import annotations

import numpy as np

from .. import physics_setup as ps


def spatialStab(fullTime, fullSpace, spaceStep, frequency, timeStep, plasmaFreq, resonantFreq,
                gamma, lim_Of_Stability=np.pi / 2):
    return ps.spatial_stab(fullTime, fullSpace, spaceStep, frequency, timeStep, plasmaFreq,
                           resonantFreq, gamma)
