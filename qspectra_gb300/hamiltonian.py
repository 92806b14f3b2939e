"""Electronic (Frenkel exciton) Hamiltonian: host-side system description.

Mirrors ElectronicHamiltonian (qspectra/hamiltonian.py:464-631).  The object
holds the small matrices a model is built from (H, dipoles, number operators,
disorder draws) and the scalar set-up quantities (rotating-wave frequency,
Nyquist time step, thermal state).  The per-sample numerics (eigensolve,
Redfield build, propagation) run on the GPU in the models and drivers.
"""
import warnings
from numbers import Number

import numpy as np
import scipy.linalg

from .constants import GAUSSIAN_SD_FWHM
from .operator_tools import (SubspaceError, basis_transform_operator,
                             basis_transform_vector, hilbert_subspace_index,
                             occupation_table, operator_extend,
                             transition_operator, unit_vec)
from .polarization import polarization_vector


class HamiltonianError(Exception):
    """hamiltonian.py:90-93."""


def check_hermitian(matrix):
    m = np.asarray(matrix)
    if not np.allclose(m.conj().T, m):
        raise ValueError('matrix input must to be Hermitian')
    return m


def ground_state(H):
    """Average of the lowest eigenprojectors (hamiltonian.py:25-46)."""
    E, U = scipy.linalg.eigh(H)
    rho = np.mean([np.outer(U[:, i], U[:, i]) for i in range(len(U))
                   if E[i] == E[0]], axis=0)
    return rho.astype(complex)


def thermal_state(H, temperature):
    """exp(-H/T)/Z, or the ground state at T = 0 (hamiltonian.py:49-78)."""
    if temperature > 0:
        rho = scipy.linalg.expm(-np.asarray(H) / float(temperature))
        tr = np.trace(rho)
        if tr == 0 or np.isnan(rho).any():
            raise OverflowError('temperature=%s too low to reliably calculate '
                                'thermal_state; raise it or set it to zero' % temperature)
        rho = rho / tr
    else:
        rho = ground_state(H)
    return rho.astype(complex)


def random_rotation_matrix(random_state):
    """Uniform random rotation (Arvo 1992; polarization.py:87-102)."""
    x1, x2, x3 = random_state.rand(3)
    th, ph = 2 * np.pi * x1, 2 * np.pi * x2
    R = np.array([[np.cos(th), np.sin(th), 0], [-np.sin(th), np.cos(th), 0],
                  [0, 0, 1]])
    v = np.array([np.cos(ph) * np.sqrt(x3), np.sin(ph) * np.sqrt(x3),
                  np.sqrt(1 - x3)])
    return -(np.eye(3) - 2 * np.outer(v, v)).dot(R)


class ElectronicHamiltonian:
    """Electronic system with one identical, independent bath per site.

    Parameters follow the reference (hamiltonian.py:513-522): ``H_1exc``
    (1-exciton matrix), ``bath``, ``dipoles`` (n x 3), ``disorder`` (FWHM of
    diagonal Gaussian disorder, or a callable of a RandomState),
    ``random_seed``, ``energy_spread_extra``.
    """

    n_vibrational_states = 1

    def __init__(self, H_1exc, bath=None, dipoles=None, disorder=None,
                 random_seed=0, energy_spread_extra=None, site_labels=None):
        self.H_1exc = check_hermitian(H_1exc)
        self.bath = bath
        self.dipoles = np.asarray(dipoles) if dipoles is not None else None
        self.disorder = disorder
        self.random_seed = random_seed
        self.energy_spread_extra = energy_spread_extra
        self.site_labels = site_labels
        self._not_sampled = self
        self._not_rotating = self
        self.rw_freq = 0
        self._cache = {}

    def __repr__(self):
        return 'ElectronicHamiltonian(n_sites={}, rw_freq={!r})'.format(
            self.n_sites, self.rw_freq)

    # ---- identity --------------------------------------------------------
    @property
    def _original(self):
        return self._not_rotating._not_sampled

    def _key(self):
        return (self.H_1exc.tobytes(), self.bath, None if self.dipoles is None
                else self.dipoles.tobytes(), self.disorder,
                repr(self.random_seed), self.energy_spread_extra, self.rw_freq)

    def __eq__(self, other):
        return isinstance(other, ElectronicHamiltonian) and self._key() == other._key()

    def __ne__(self, other):
        return not self == other

    def __hash__(self):
        return hash(self._key())

    def _memo(self, key, fn):
        if key not in self._cache:
            self._cache[key] = fn()
        return self._cache[key]

    # ---- matrices ----------------------------------------------------------
    @property
    def n_sites(self):
        return len(self.H_1exc)

    def H(self, subspace):
        """Hamiltonian on the requested manifolds (hamiltonian.py:539-544)."""
        return self._memo(('H', subspace),
                          lambda: operator_extend(self.H_1exc, subspace))

    def n_states(self, subspace):
        return len(self.H(subspace))

    def hilbert_subspace_index(self, subspace, all_subspaces):
        return hilbert_subspace_index(subspace, all_subspaces, self.n_sites,
                                      self.n_vibrational_states)

    def number_operator(self, site, subspace='gef'):
        return operator_extend(np.diag(unit_vec(site, self.n_sites, dtype=float)),
                               subspace)

    def system_bath_couplings(self, subspace='gef'):
        """Number operators n_i (hamiltonian.py:600-608)."""
        if self.bath is None:
            raise HamiltonianError('bath undefined')
        return np.array([self.number_operator(n, subspace)
                         for n in range(self.n_sites)])

    def occupation_table(self, subspace='gef'):
        """Diagonals of the number operators, the form the GPU kernels take."""
        if self.bath is None:
            raise HamiltonianError('bath undefined')
        return occupation_table(self.n_sites, subspace)

    def dipole_operator(self, subspace='gef', polarization='x',
                        transitions='-+'):
        """Σ_n T_n (d_n · e) (hamiltonian.py:580-591)."""
        if self.dipoles is None:
            raise HamiltonianError('transition dipole moments undefined')
        proj = self.dipoles @ polarization_vector(polarization)
        return sum(proj[n] * transition_operator(n, self.n_sites, subspace,
                                                 transitions)
                   for n in range(self.n_sites))

    # ---- eigen-structure (host set-up) -----------------------------------
    def eig(self, subspace):
        """eigh of the non-rotating H, e/f shifted by rw (hamiltonian.py:310-328)."""
        def run():
            E, U = scipy.linalg.eigh(self._not_rotating.H(subspace))
            if 'e' in subspace:
                E[self.hilbert_subspace_index('e', subspace)] -= self.rw_freq
            if 'f' in subspace:
                E[self.hilbert_subspace_index('f', subspace)] -= 2 * self.rw_freq
            return E, U
        return self._memo(('eig', subspace), run)

    def E(self, subspace):
        return self.eig(subspace)[0]

    def U(self, subspace):
        return self.eig(subspace)[1]

    def transform_vector_to_eigenbasis(self, rho, subspace):
        return basis_transform_vector(rho, self.U(subspace))

    def transform_vector_from_eigenbasis(self, rho, subspace):
        return basis_transform_vector(rho, self.U(subspace).T.conj())

    def transform_operator_to_eigenbasis(self, op, subspace):
        return basis_transform_operator(op, self.U(subspace))

    def transform_operator_from_eigenbasis(self, op, subspace):
        return basis_transform_operator(op, self.U(subspace).T.conj())

    @property
    def transition_energy(self):
        """mean E_e (hamiltonian.py:375-380)."""
        return np.mean(self.E('e'))

    @property
    def freq_step(self):
        """Nyquist frequency step, fixed under sampling (hamiltonian.py:382-399)."""
        energies = self._not_sampled.E('gef')
        if self.energy_spread_extra is None:
            extra = 0.01 * self._original.transition_energy
        else:
            extra = self.energy_spread_extra
        return 2 * (max(energies.max(), -energies.min()) + extra)

    @property
    def time_step(self):
        return 1.0 / self.freq_step

    def ground_state(self, subspace):
        return ground_state(self._not_rotating.H(subspace))

    def thermal_state(self, subspace):
        try:
            T = self._not_rotating.bath.temperature
        except AttributeError:
            T = 0
        return self._memo(('thermal', subspace),
                          lambda: thermal_state(self._not_rotating.H(subspace), T))

    # ---- rotating frame and disorder -------------------------------------
    def _copy(self, H_1exc, dipoles, random_seed):
        return type(self)(H_1exc, self.bath, dipoles, self.disorder,
                          random_seed, self.energy_spread_extra,
                          self.site_labels)

    def in_rotating_frame(self, rw_freq=None):
        """Shift the e manifold by -rw (hamiltonian.py:177-209); idempotent."""
        if rw_freq is None:
            rw_freq = self._original.transition_energy
        base = self._not_rotating
        ham = base._copy(base.H_1exc - rw_freq * np.identity(base.n_sites),
                         base.dipoles, base.random_seed)
        ham._not_rotating = base
        if self._not_sampled is not self:
            ham._not_sampled = self._not_sampled.in_rotating_frame(rw_freq)
        ham.rw_freq = rw_freq
        return ham

    def _disorder_for(self, random_state):
        if self.disorder is None:
            return 0
        if isinstance(self.disorder, Number):
            return np.diag((self.disorder * GAUSSIAN_SD_FWHM)
                           * random_state.randn(self.n_sites))
        return self.disorder(random_state)

    def _seed_for(self, n):
        return list(np.atleast_1d(self.random_seed)) + [n]

    def _sample(self, n, random_orientations):
        if self.disorder is None and not random_orientations:
            warnings.warn('called sample with `disorder=None` and '
                          '`random_orientations=False`: sampled Hamiltonian '
                          'is identical to original', RuntimeWarning,
                          stacklevel=3)
        seed = self._seed_for(n)
        rs = np.random.RandomState(seed)
        H = self.H_1exc + self._disorder_for(rs)
        dip = self.dipoles
        if random_orientations:
            dip = np.einsum('mn,in->im', random_rotation_matrix(rs), self.dipoles)
        return self._copy(H, dip, seed)

    def sample(self, n=None, random_orientations=False):
        """n-th static-disorder sample (hamiltonian.py:233-274)."""
        if n is None:
            n = np.random.randint(2 ** 30)
        ham = self._not_sampled._sample(n, random_orientations)
        if self._not_rotating is not self:
            ham._not_rotating = self._not_rotating.sample(n, random_orientations)
        ham._not_sampled = self._not_sampled
        ham.rw_freq = self.rw_freq
        return ham

    def sample_ensemble(self, ensemble_size=1, random_orientations=False):
        for n in range(ensemble_size):
            yield self.sample(n, random_orientations)

    def disorder_offsets(self, ensemble_size, start=0):
        """Diagonal site-energy offsets of samples start..start+ensemble_size-1.

        The same draws as ``sample(n)`` (RandomState(list(seed) + [n]).randn,
        scaled by disorder * GAUSSIAN_SD_FWHM), returned as an
        (ensemble_size, n_sites) array for the batched GPU path.
        """
        base = self._not_sampled
        if base.disorder is None:
            return np.zeros((ensemble_size, self.n_sites))
        if not isinstance(base.disorder, Number):
            out = []
            for n in range(start, start + ensemble_size):
                d = base.disorder(np.random.RandomState(base._seed_for(n)))
                d = np.asarray(d)
                if d.ndim != 2 or np.count_nonzero(d - np.diag(np.diag(d))):
                    raise NotImplementedError('batched path needs diagonal disorder')
                out.append(np.diag(d))
            return np.array(out)
        scale = base.disorder * GAUSSIAN_SD_FWHM
        out = np.empty((ensemble_size, self.n_sites))
        for k, n in enumerate(range(start, start + ensemble_size)):
            out[k] = scale * np.random.RandomState(base._seed_for(n)).randn(self.n_sites)
        return out

    def orientation_rotations(self, ensemble_size, start=0):
        """(ensemble_size, 3, 3) rotations applied to the dipoles of samples
        start..start+ensemble_size-1 when ``random_orientations`` is set.

        The same draws as ``sample(n, random_orientations=True)``
        (hamiltonian.py:552-575): RandomState(list(seed) + [n]) draws the
        disorder first, then the three uniforms of the rotation.  Sample n's
        dipoles are R_n d_i, so its response to lab polarization e equals the
        unrotated system's response to R_n^T e.
        """
        base = self._not_sampled
        out = np.empty((ensemble_size, 3, 3))
        for k, n in enumerate(range(start, start + ensemble_size)):
            rs = np.random.RandomState(base._seed_for(n))
            base._disorder_for(rs)
            out[k] = random_rotation_matrix(rs)
        return out
