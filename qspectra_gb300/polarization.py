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


# The three isotropic fourth-rank invariants, each a pairing of the four
# field indices into two Kronecker deltas (polarization.py:46-48).
FOURTH_ORDER_INVARIANTS = [((0, 1), (2, 3)),
                           ((0, 2), (1, 3)),
                           ((0, 3), (1, 2))]


def invariant_weights_4th_order(polarizations):
    """Weights of the invariants <xxyy>, <xyxy>, <xyyx> in the isotropic
    average of a fourth-rank response for four lab-frame polarizations
    (polarization.py:55-70; Hochstrasser, Chem. Phys. 266, 273 (2001)).

    The orientational average of four direction cosines is
    (1/30) [[4, -1, -1], [-1, 4, -1], [-1, -1, 4]] applied to the products
    of the polarization dot products taken in the three pairings.
    """
    pols = check_polarizations(polarizations, 4)
    dots = pols @ pols.T
    pair = np.array([dots[a] * dots[b] for a, b in FOURTH_ORDER_INVARIANTS])
    mix = 5.0 * np.eye(3) - np.ones((3, 3))
    return mix @ pair / 30.0


def invariant_polarizations(invariant):
    """The nine lab polarizations 'abcd' whose paired indices agree, summed to
    form one invariant (polarization.py:73-84)."""
    if invariant not in FOURTH_ORDER_INVARIANTS:
        raise ValueError('`invariant` is not one of the three 4th order tensor '
                         'invariants %r' % FOURTH_ORDER_INVARIANTS)
    out = []
    for code in range(81):
        p = ''.join('xyz'[(code // 3 ** (3 - k)) % 3] for k in range(4))
        if all(p[a] == p[b] for a, b in invariant):
            out.append(p)
    return out


def isotropic_tensor_4th_order(polarizations, threshold=1e-8):
    """(3, 3, 3, 3) lab-frame weights T such that the isotropic average equals
    sum_abcd T[a, b, c, d] R(e_a, e_b, e_c, e_d).

    Follows the reference's summation (decorators.py:67-92): an invariant
    enters with its weight only when that weight exceeds ``threshold``, so
    invariants with negative weights are left out exactly as there.
    """
    T = np.zeros((3, 3, 3, 3))
    for inv, w in zip(FOURTH_ORDER_INVARIANTS, invariant_weights_4th_order(polarizations)):
        if w > threshold:
            for p in invariant_polarizations(inv):
                T[tuple('xyz'.index(c) for c in p)] += w
    return T
