"""Pulses for field-driven propagation (qspectra/pulse.py).

A pulse is a callable returning its complex electric field at times t in
the rotating frame of ``rw_freq``, with ``t_init`` and ``t_final`` bounding
where it is applied.  The GPU path tabulates the field at every RK4 stage
time on the host and passes the table to the time loop.
"""
from abc import ABCMeta, abstractmethod

import numpy as np

from .constants import GAUSSIAN_SD_FWHM


class Pulse(metaclass=ABCMeta):
    """Pulse API (pulse.py:8-47): ``pulse(t, rw_freq)`` -> complex field."""

    @abstractmethod
    def __call__(self, t, rw_freq):
        """Complex field at time(s) t in the frame rotating at rw_freq."""


class CustomPulse(Pulse):
    """Field given by a function call(t, rw_freq) (pulse.py:50-71)."""

    def __init__(self, t_init, t_final, call):
        self.t_init = t_init
        self.t_final = t_final
        self.call = call

    def __call__(self, t, rw_freq):
        return self.call(t, rw_freq)


class GaussianPulse(Pulse):
    """Gaussian envelope around a carrier (pulse.py:74-113):
    E(t) = scale exp(i fc (carrier - rw) (t - t_peak) - (t - t_peak)^2 / 2 sigma^2),
    sigma = fwhm * GAUSSIAN_SD_FWHM, applied within t_peak +- t_limits_multiple sigma.
    """

    def __init__(self, carrier_freq, fwhm, t_peak=0, scale=1, freq_convert=1,
                 t_limits_multiple=3):
        sigma = GAUSSIAN_SD_FWHM * fwhm
        self.two_sigma_squared = 2 * sigma ** 2
        self.t_init = t_peak - t_limits_multiple * sigma
        self.t_final = t_peak + t_limits_multiple * sigma
        self.t_peak = t_peak
        self.carrier_freq = carrier_freq
        self.scale = scale
        self.freq_convert = freq_convert

    def __call__(self, t, rw_freq):
        dt = np.asarray(t, float) - self.t_peak
        return self.scale * np.exp(1j * self.freq_convert * (self.carrier_freq - rw_freq) * dt
                                   - dt ** 2 / self.two_sigma_squared)
