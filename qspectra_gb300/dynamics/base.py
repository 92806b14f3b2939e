"""Dynamical-model plugin API (qspectra/dynamics/base.py:7-181).

The abstract interface every model implements.  Spectroscopy drivers only
talk to a model through it: thermal_state, equation_of_motion,
map_between_subspaces and dipole_operator.
"""
import copy
from abc import ABCMeta, abstractmethod


class DynamicalModel(metaclass=ABCMeta):
    """Abstract base class of dynamical models (base.py:7-140)."""

    def __init__(self, hamiltonian, rw_freq=None, hilbert_subspace='gef',
                 unit_convert=1):
        self.hamiltonian = hamiltonian.in_rotating_frame(rw_freq)
        self.rw_freq = self.hamiltonian.rw_freq
        self.hilbert_subspace = hilbert_subspace
        self.unit_convert = unit_convert

    def density_matrix_to_state_vector(self, rho, liouville_subspace=None):
        return rho

    def state_vector_to_density_matrix(self, rho):
        return rho

    @abstractmethod
    def thermal_state(self, liouville_subspace):
        """Thermal state for this model on a Liouville subspace."""

    @abstractmethod
    def equation_of_motion(self, liouville_subspace, heisenberg_picture=False):
        """Callable eom(t, state) -> d state / dt on a Liouville subspace.

        Raises NotImplementedError when the model has no Heisenberg picture.
        """

    @abstractmethod
    def map_between_subspaces(self, state, from_subspace, to_subspace):
        """Map a state vector between Liouville subspaces (zeros where new)."""

    def dipole_operator(self, liouv_subspace_map, polarization, transitions='-+'):
        op = self.hamiltonian.dipole_operator(self.hilbert_subspace,
                                              polarization, transitions)
        return self.system_operator(op, liouv_subspace_map, self)

    def dipole_destroy(self, liouville_subspace_map, polarization):
        return self.dipole_operator(liouville_subspace_map, polarization, '-')

    def dipole_create(self, liouville_subspace_map, polarization):
        return self.dipole_operator(liouville_subspace_map, polarization, '+')

    def sample_ensemble(self, *args, **kwargs):
        """Copies of this model with the Hamiltonian's disorder samples (base.py:120-128)."""
        for ham in self.hamiltonian.sample_ensemble(*args, **kwargs):
            new = copy.copy(self)
            new.hamiltonian = ham
            new._cache = {}
            yield new

    @property
    def time_step(self):
        """Default sampling step of the equation of motion (base.py:130-136)."""
        return self.hamiltonian.time_step / self.unit_convert

    def hilbert_subspace_index(self, subspace):
        return self.hamiltonian.hilbert_subspace_index(subspace,
                                                       self.hilbert_subspace)


class SystemOperator(metaclass=ABCMeta):
    """System-field operator API (base.py:143-181)."""

    def commutator(self, state):
        return self.left_multiply(state) - self.right_multiply(state)

    @abstractmethod
    def left_multiply(self, state):
        """Operator times state."""

    @abstractmethod
    def right_multiply(self, state):
        """State times operator."""

    @abstractmethod
    def expectation_value(self, state):
        """tr(operator · state)."""
