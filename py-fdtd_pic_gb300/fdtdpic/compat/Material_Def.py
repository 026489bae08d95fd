"""``matSetup`` of Material_Def.py:21-120: the older fixed-geometry set-up (returns its
19-tuple)."""
from __future__ import annotations

from .. import physics_setup as ps


def matSetup(V, P, C_P, C_V, newFreq_in, domainSize, minim=400, maxim=800):
    return ps.mat_setup(V, P, C_P, C_V, newFreq_in, domainSize, minim, maxim)
