"""Scalar turbulence parameters (theory/atmosphere/__init__.py of the
reference): Rytov variance and coherence diameters."""
from __future__ import annotations

import numpy as np


def get_rytov2(Cn2, k, length):
    return 1.23 * Cn2 * k ** (7 / 6) * length ** (11 / 6)


def get_r0(Cn2, k, length):
    """Coherence diameter for plane waves."""
    return (0.423 * k ** 2 * Cn2 * length) ** (-3 / 5)


def get_r0s(Cn2, length, k):
    """Coherence diameter for spherical waves: constant Cn2, a list of slab
    values, or a callable profile (theory/atmosphere/__init__.py:14-49)."""
    try:
        acc = 0.0
        for i in range(len(Cn2)):
            try:
                length_i = length[i]
            except (IndexError, TypeError):
                length_i = length / len(Cn2)
            acc += get_r0s(Cn2[i], length_i, k) ** (-5 / 3)
        return acc ** (-3 / 5)
    except TypeError:
        pass
    if callable(Cn2):
        from scipy.integrate import quad
        return (0.423 * k ** 2 * quad(lambda z: Cn2(z) * ((length - z) / length) ** (5 / 3), 0, length)[0]) ** (-3 / 5)
    return (0.423 * k ** 2 * Cn2 * 3 / 8 * length) ** (-3 / 5)
