"""Unit conversions (same values as qspectra/constants.py:8-18)."""
from numpy import log, pi, sqrt

CM_FS_LINEAR = 2.99792458e-5
"""fs -> linear cm^-1."""
CM_FS = pi * 2 * CM_FS_LINEAR
"""fs -> angular cm^-1."""
CM_K = 0.69503476
"""Kelvin -> angular cm^-1 (Boltzmann constant folded in)."""
GAUSSIAN_SD_FWHM = 1.0 / (2 * sqrt(2 * log(2)))
"""SD / FWHM of a Gaussian."""
