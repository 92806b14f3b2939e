"""Bath descriptions (qspectra/bath.py).

Only the Debye (Drude-Lorentz) bath is on the accelerated path: its
correlation function is evaluated on the GPU by qsx_debye_corr, both inside
the Redfield build and through ``corr_func_complex`` / ``corr_func_real``.
"""
import numpy as np
import torch

from . import _native


class DebyeBath:
    """Drude-Lorentz bath, J(x) = 2λγx/(γ² + x²) (bath.py:69-102)."""

    def __init__(self, temperature, reorg_energy, cutoff_freq,
                 matsubara_cutoff=1000):
        self.temperature = float(temperature)
        self.reorg_energy = float(reorg_energy)
        self.cutoff_freq = float(cutoff_freq)
        self.matsubara_cutoff = int(matsubara_cutoff)

    def __repr__(self):
        return 'DebyeBath(temperature={!r}, reorg_energy={!r}, cutoff_freq={!r})'.format(
            self.temperature, self.reorg_energy, self.cutoff_freq)

    def __eq__(self, other):
        return (isinstance(other, DebyeBath)
                and (self.temperature, self.reorg_energy, self.cutoff_freq)
                == (other.temperature, other.reorg_energy, other.cutoff_freq))

    def spectral_density_func(self, x):
        return (2 * self.reorg_energy * self.cutoff_freq * x
                / (self.cutoff_freq ** 2 + x ** 2))

    @property
    def spectral_density_limit_at_zero(self):
        return 2 * self.reorg_energy / self.cutoff_freq

    def _corr(self, x, real_only, matsubara_cutoff=None):
        scalar = np.ndim(x) == 0
        xs = torch.as_tensor(np.atleast_1d(np.asarray(x, float)),
                             dtype=torch.float64).cuda()
        out = _native.debye_corr(xs, self.temperature, self.reorg_energy,
                                 self.cutoff_freq,
                                 matsubara_cutoff or self.matsubara_cutoff,
                                 real_only).cpu().numpy()
        if real_only:
            out = out.real
        return out[0] if scalar else out

    def corr_func_complex(self, x, matsubara_cutoff=1000):
        """One-sided C(x) with the truncated Matsubara sum (bath.py:84-102)."""
        return self._corr(x, False, matsubara_cutoff)

    def corr_func_real(self, x):
        """(n(x)+1) J_anti(x) (bath.py:17-31)."""
        return self._corr(x, True)


class PseudomodeBath:
    """Bath given by pseudomodes, Lorentzians in the bath correlation spectrum
    (bath.py:105-146): frequencies ``Omega``, widths ``gamma`` and couplings
    ``huang``, each (numb_pm, n_sites) when the sites have separate baths.
    Used by the ZOFE master equation."""

    def __init__(self, numb_pm, Omega, gamma, huang):
        self.numb_pm = numb_pm
        self.Omega = Omega
        self.gamma = gamma
        self.huang = huang

    def __repr__(self):
        return 'PseudomodeBath(numb_pm={!r})'.format(self.numb_pm)
