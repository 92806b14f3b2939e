"""Seeded synthetic Hamiltonians for the benchmark workloads.

The reference publishes no input files for these workloads, so every input is
generated here from a fixed seed.  The recipes are plain NumPy on the host;
nothing in this module touches the GPU.

Workloads
---------
``fmo7``      7-site Frenkel exciton: E_i ~ U(12000, 12600) cm^-1, J_ij ~ N(0, 50^2)
              (i < j, symmetric), seed 1234; Debye bath λ=35, γ=106 cm^-1, T=77 K;
              unit x dipoles on every site.  Redfield, non-secular, 'ge' Hilbert
              space, dt = 1 fs.  The batched form adds Gaussian static disorder
              with SD 80 cm^-1 on the site energies (16384 samples).
``chain24``   24-site chain: E_i ~ N(12300, 100^2), nearest neighbour -80,
              next-nearest +15 cm^-1; λ=40, γ=100 cm^-1, T=300 K; dt = 2 fs;
              disorder SD 60 cm^-1 (256 samples).
``ring8``     8-site ring: E_i ~ N(12400, 80^2), ring coupling -100 cm^-1;
              λ=35, γ=106 cm^-1, T=300 K; HEOM K=0, level_cutoff=5 (495 nodes);
              dt = 0.5 fs; disorder SD 50 cm^-1 (64 samples).
"""
import numpy as np

from .constants import CM_FS, CM_K, GAUSSIAN_SD_FWHM


def fmo7_hamiltonian(n_sites=7, seed=1234):
    """E_i ~ U(12000, 12600); J_ij ~ N(0, 50^2) on the upper triangle."""
    rng = np.random.RandomState(seed)
    E = rng.uniform(12000.0, 12600.0, n_sites)
    J = np.triu(rng.normal(0.0, 50.0, (n_sites, n_sites)), 1)
    return J + J.T + np.diag(E)


def chain_hamiltonian(n_sites=24, seed=2024, mean=12300.0, sd=100.0,
                      nn=-80.0, nnn=15.0):
    """Linear chain with nearest and next-nearest neighbour couplings."""
    rng = np.random.RandomState(seed)
    H = np.diag(rng.normal(mean, sd, n_sites))
    for i in range(n_sites - 1):
        H[i, i + 1] = H[i + 1, i] = nn
    for i in range(n_sites - 2):
        H[i, i + 2] = H[i + 2, i] = nnn
    return H


def ring_hamiltonian(n_sites=8, seed=4321, mean=12400.0, sd=80.0,
                     coupling=-100.0):
    """Ring with equal nearest-neighbour couplings."""
    rng = np.random.RandomState(seed)
    H = np.diag(rng.normal(mean, sd, n_sites))
    for i in range(n_sites):
        j = (i + 1) % n_sites
        H[i, j] = H[j, i] = coupling
    return H


def pseudomode_parameters(n_sites=7, numb_pm=16, seed=77):
    """Seeded pseudomode bath (Omega, gamma, huang), each (numb_pm, n_sites):
    Lorentzians at Omega in [-500, 1500] cm^-1 with widths 40..500 cm^-1 and
    couplings Omega^2 huang of 20..400 cm^-1, one low-frequency mode near
    zero; the same set on every site."""
    rng = np.random.RandomState(seed)
    Om = np.sort(rng.uniform(-500.0, 1500.0, numb_pm))
    Om[np.argmin(np.abs(Om))] = 1.0
    ga = rng.uniform(40.0, 500.0, numb_pm)
    hu = rng.uniform(20.0, 400.0, numb_pm) / (Om ** 2 + 100.0)
    on = np.ones(n_sites, complex)
    return tuple(np.array([x * on for x in v]) for v in (Om, ga, hu))


def unit_dipoles(n_sites=7, seed=99):
    """Random unit transition dipoles."""
    d = np.random.RandomState(seed).randn(n_sites, 3)
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def fwhm_for_sd(sd):
    """Disorder argument (a FWHM) that gives Gaussian SD ``sd`` (hamiltonian.py:458-461)."""
    return sd / GAUSSIAN_SD_FWHM


def energy_spread_for_dt(H1, dt, unit_convert=CM_FS, rw_freq=None):
    """``energy_spread_extra`` that makes the Nyquist time step exactly ``dt``.

    The reference picks its time step from the spread of the rotating-frame
    energies plus ``energy_spread_extra`` (hamiltonian.py:382-412); this
    solves for the extra and nudges it by ulps until the step is exact.
    """
    import scipy.linalg
    from .operator_tools import operator_extend
    H1 = np.asarray(H1, float)
    if rw_freq is None:
        rw_freq = float(np.mean(scipy.linalg.eigh(H1)[0]))
    E, _ = scipy.linalg.eigh(operator_extend(H1, 'gef'))
    n = len(H1)
    E[1:1 + n] -= rw_freq
    E[1 + n:] -= 2 * rw_freq
    emax = max(E.max(), -E.min())

    def step(extra):
        return 1.0 / (2 * (emax + extra)) / unit_convert

    extra = 1.0 / (2 * dt * unit_convert) - emax
    for _ in range(64):
        s = step(extra)
        if s == dt:
            return extra
        extra = np.nextafter(extra, np.inf if s > dt else -np.inf)
    return extra


WORKLOADS = {
    'fmo7': dict(n_sites=7, temperature_K=77.0, reorg=35.0, cutoff=106.0,
                 dt=1.0, disorder_sd=80.0, n_samples=16384,
                 dynamics_time=1000.0, absorption_time=2048.0),
    'chain24': dict(n_sites=24, temperature_K=300.0, reorg=40.0, cutoff=100.0,
                    dt=2.0, disorder_sd=60.0, n_samples=256,
                    coherence_time=256.0, population_times=(0.0, 200.0, 500.0)),
    'ring8': dict(n_sites=8, temperature_K=300.0, reorg=35.0, cutoff=106.0,
                  dt=0.5, disorder_sd=50.0, n_samples=64, duration=1000.0,
                  K=0, level_cutoff=5),
}


def temperature_cm(kelvin):
    return CM_K * kelvin
