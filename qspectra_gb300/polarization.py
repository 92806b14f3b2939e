"""Polarization vectors (host set-up; qspectra/polarization.py:14-44)."""
from numbers import Number

import numpy as np

COORD_MAP = {'x': np.array([1, 0, 0]),
             'y': np.array([0, 1, 0]),
             'z': np.array([0, 0, 1])}


def polarization_vector(p):
    """'x'/'y'/'z', an angle in the x-y plane, or a 3-vector (polarization.py:14-36)."""
    try:
        if isinstance(p, str):
            return COORD_MAP[p]
        if isinstance(p, Number):
            return np.array([np.cos(p), np.sin(p), 0])
        v = np.asanyarray(p, float).reshape(-1)
        if len(v) != 3:
            raise ValueError('polarization vectors must have length 3')
        return v
    except Exception:
        raise ValueError('invalid polarization {}'.format(p))


def check_polarizations(p, length):
    """polarization.py:39-44."""
    pols = np.array([polarization_vector(x) for x in p])
    if len(pols) != length:
        raise ValueError('%s polarizations required' % length)
    return pols
