"""Declared scalar types for the state classes.

The reference declares its state classes as numba jitclasses (MasterController.py:82-440): a
member declared ``float32`` stores the float32-rounded value (which then enters float64
arithmetic as such), ``int32`` an integer, ``boolean`` a bool.  :func:`typed` gives a plain
Python class the same assignment behaviour for the scalar members it lists; array members are
stored by reference, as jitclass members are.
"""
from __future__ import annotations

import numpy as np


def _f32(v):
    return float(np.float32(np.real(v)))


def _f64(v):
    return float(np.real(v)) if np.iscomplexobj(v) else float(v)


_CASTS = {"f32": _f32, "f64": _f64, "i32": int, "bool": bool}


def typed(fields: dict):
    """Class decorator: ``fields`` maps member name -> "f32" | "f64" | "i32" | "bool"."""
    for kind in fields.values():
        if kind not in _CASTS:
            raise ValueError(f"unknown member type {kind!r}")

    def deco(cls):
        def __setattr__(self, name, value):
            kind = fields.get(name)
            if kind is not None:
                value = _CASTS[kind](value)
            object.__setattr__(self, name, value)

        cls.__setattr__ = __setattr__
        cls.scalar_types = dict(fields)
        return cls

    return deco
