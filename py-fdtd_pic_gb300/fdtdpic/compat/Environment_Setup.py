"""``envSetup`` of Environment_Setup.py:19-166: grid geometry from a frequency and a domain size
(returns its 20-tuple, the leading positional arguments of ``Params``)."""
from __future__ import annotations

from .. import physics_setup as ps


def envSetup(newFreq_in, domainSize, minim=400, maxim=600, VExists=False, V=None, P=None,
             nonLinMed=False, LorMed=False):
    return ps.env_setup(newFreq_in, domainSize, minim, maxim, VExists=VExists, V=V, P=P,
                        nonLinMed=nonLinMed, LorMed=LorMed)
