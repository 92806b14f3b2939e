"""Liouville-space conventions, operators and the model base class.

Conventions follow qspectra/dynamics/liouville_space.py: density matrices are
column-stacked (vec index a + n*b for element (a, b)); a Liouville subspace
such as 'eg,ee' selects, in ascending vec order, the elements whose row and
column lie in the named manifolds.  Operators and equations of motion hold
their matrices as CUDA tensors and apply them on the GPU.
"""
import itertools

import numpy as np
import torch

from .. import _native
from ..operator_tools import (SubspaceError, full_liouville_subspace,
                              n_excitations)
from .base import DynamicalModel, SystemOperator


def liouville_subspace_index(liouville_subspace, full_subspace, n_sites,
                             n_vibrational_states=1):
    """Column-stacked indices of the blocks in ``liouville_subspace`` (liouville_space.py:9-29)."""
    sizes = n_excitations(n_sites, n_vibrational_states)
    cuts, total = {}, 0
    for letter, size in zip('gef', sizes):
        if letter in full_subspace:
            cuts[letter] = np.arange(size) + total
            total += size
    keep = np.zeros((total, total), dtype=bool)
    for block in liouville_subspace.split(','):
        row, col = block
        if row not in cuts or col not in cuts:
            raise SubspaceError("{}{} not in subspace '{}'".format(
                row, col, full_subspace))
        keep[np.ix_(cuts[row], cuts[col])] = True
    return np.flatnonzero(keep.reshape(-1, order='F'))


def all_liouville_subspaces(hilbert_subspace):
    """'ge' -> 'gg,ge,eg,ee' (liouville_space.py:32-43)."""
    return ','.join(''.join(s) for s in itertools.product(hilbert_subspace, repeat=2))


def matrix_to_ket_vec(matrix):
    return np.asarray(matrix).reshape(-1, order='F')


def ket_vec_to_matrix(ket_vec):
    ket_vec = np.asarray(ket_vec)
    n = int(np.sqrt(np.prod(ket_vec.shape)))
    return ket_vec.reshape((n, n), order='F')


def matrix_to_bra_vec(matrix):
    return np.asarray(matrix).reshape(-1, order='C')


def tensor_to_super(tensor_operator):
    """S[i + N j, k + N l] = T[i, j, k, l] (liouville_space.py:68-90)."""
    t = np.asarray(tensor_operator)
    n = t.shape[0]
    return np.ascontiguousarray(t.transpose(1, 0, 3, 2)).reshape(n * n, n * n)


def super_left_matrix(operator):
    return np.kron(np.identity(len(operator)), operator)


def super_right_matrix(operator):
    return np.kron(np.asarray(operator).T, np.identity(len(operator)))


def super_commutator_matrix(operator):
    return super_left_matrix(operator) - super_right_matrix(operator)


def _device():
    _native.require_gpu()
    return torch.device('cuda', torch.cuda.current_device())


def _as_device(x):
    if isinstance(x, torch.Tensor):
        return x.to(device=_device(), dtype=torch.complex128), True
    return torch.as_tensor(np.asarray(x, dtype=complex), device=_device()), False


class LinearMap:
    """A fixed matrix applied along the last axis of a state, on the GPU.

    Stands in for the bound ``ndarray.dot`` methods that the reference's
    operators expose; numpy inputs give numpy outputs.
    """

    def __init__(self, matrix, scalar=False):
        self.matrix = torch.as_tensor(np.asarray(matrix, dtype=complex),
                                      device=_device())
        self.scalar = scalar  # one output row returned as a scalar (expectation)

    @property
    def shape(self):
        return tuple(self.matrix.shape)

    def __call__(self, state):
        x, is_tensor = _as_device(state)
        y = x @ self.matrix.T
        if self.scalar:
            y = y[..., 0]
        return y if is_tensor else y.cpu().numpy()

    dot = __call__


class EquationOfMotion:
    """Linear equation of motion eom(t, y) = L y with L resident on the GPU.

    ``matrix`` is the (M, M) complex128 generator (already transposed for the
    Heisenberg picture).  Calling it performs one GPU matrix-vector product,
    for API parity with the reference's closures (liouville_space.py:339-341);
    ``integrate`` recognises it and runs the whole RK4 loop on the GPU.
    """

    def __init__(self, matrix, liouville_subspace=None, heisenberg_picture=False,
                 model=None):
        self.matrix = matrix
        self.liouville_subspace = liouville_subspace
        self.heisenberg_picture = heisenberg_picture
        self.model = model

    @property
    def dim(self):
        return int(self.matrix.shape[-1])

    def __call__(self, t, rho):
        x, is_tensor = _as_device(rho)
        y = x @ self.matrix.T
        return y if is_tensor else y.cpu().numpy()


class LiouvilleSpaceOperator(SystemOperator):
    """Dipole-type operator restricted to from/to Liouville subspaces (liouville_space.py:151-209)."""

    def __init__(self, operator, liouv_subspace_map, dynamical_model):
        self.operator = operator
        parts = (liouv_subspace_map.split('->') if '->' in liouv_subspace_map
                 else [liouv_subspace_map, liouv_subspace_map])
        self.from_indices, self.to_indices = [
            dynamical_model.liouville_subspace_index(s) for s in parts]
        self.super_op_mesh = np.ix_(self.to_indices, self.from_indices)
        self._maps = {}

    @property
    def bra_vector(self):
        op = np.asanyarray(self.operator, dtype=complex)
        return matrix_to_bra_vec(op)[self.from_indices]

    def _map(self, key, build, scalar=False):
        if key not in self._maps:
            self._maps[key] = LinearMap(build(), scalar)
        return self._maps[key]

    def _restricted(self, side):
        """kron(I, V) (side 'left') or kron(V^T, I) ('right') restricted to
        to x from indices, without forming the n^2 x n^2 super-operator:
        element (a + n b, c + n d) is V[a, c] [b == d] or V[d, b] [a == c]."""
        V = np.asarray(self.operator)
        n = len(V)
        ta, tb = self.to_indices % n, self.to_indices // n
        fc, fd = self.from_indices % n, self.from_indices // n
        if side == 'left':
            return V[np.ix_(ta, fc)] * (tb[:, None] == fd[None, :])
        return V[np.ix_(fd, tb)].T * (ta[:, None] == fc[None, :])

    def _left(self):
        return self._restricted('left')

    @property
    def left_multiply(self):
        return self._map('left', self._left)

    @property
    def right_multiply(self):
        return self._map('right', lambda: self._restricted('right'))

    @property
    def commutator(self):
        return self._map('comm', lambda: self.commutator_matrix)

    @property
    def commutator_matrix(self):
        """Host (to x from) matrix of the restricted commutator [V, .]."""
        return self._restricted('left') - self._restricted('right')

    @property
    def expectation_row(self):
        n = len(self.operator)
        tr = (self.to_indices % n == self.to_indices // n).astype(float)
        return tr.dot(self._left())

    @property
    def expectation_value(self):
        return self._map('expect', lambda: self.expectation_row[None, :], scalar=True)


class LiouvilleSpaceModel(DynamicalModel):
    """Base class of Liouville-space models (liouville_space.py:212-349).

    Subclasses provide ``_block(idx, transpose)``: the dense generator on the
    given column-stacked indices as a CUDA complex128 tensor.
    ``sparse_matrix`` is accepted for API parity; the GPU path always uses
    the dense block.
    """
    system_operator = LiouvilleSpaceOperator

    def __init__(self, hamiltonian, rw_freq=None, hilbert_subspace='gef',
                 unit_convert=1, evolve_basis='site', sparse_matrix=False):
        super().__init__(hamiltonian, rw_freq, hilbert_subspace, unit_convert)
        self.evolve_basis = evolve_basis
        self.sparse_matrix = sparse_matrix
        self._cache = {}

    @property
    def evolve_basis(self):
        return self._evolve_basis

    @evolve_basis.setter
    def evolve_basis(self, val):
        if val not in ('site', 'eigen'):
            raise ValueError('invalid basis')
        self._evolve_basis = val

    def liouville_subspace_index(self, subspace):
        return liouville_subspace_index(subspace, self.hilbert_subspace,
                                        self.hamiltonian.n_sites,
                                        self.hamiltonian.n_vibrational_states)

    def density_matrix_to_state_vector(self, rho0, liouville_subspace):
        state0 = matrix_to_ket_vec(rho0)
        return self.map_between_subspaces(
            state0, full_liouville_subspace(liouville_subspace), liouville_subspace)

    def state_vector_to_density_matrix(self, rho):
        n = int(np.sqrt(rho.shape[-1]))
        if isinstance(rho, torch.Tensor):
            return rho.reshape(rho.shape[:-1] + (n, n)).transpose(-1, -2)
        return rho.reshape(-1, n, n, order='F')

    def dipole_operator(self, liouv_subspace_map, polarization, transitions='-+'):
        op = self.hamiltonian.dipole_operator(self.hilbert_subspace,
                                              polarization, transitions)
        if self.evolve_basis == 'eigen':
            op = self.hamiltonian.transform_operator_to_eigenbasis(
                op, self.hilbert_subspace)
        return self.system_operator(op, liouv_subspace_map, self)

    def thermal_state(self, liouville_subspace):
        rho0 = self.hamiltonian.thermal_state(liouville_subspace)
        rho = self.map_between_subspaces(
            matrix_to_ket_vec(rho0), full_liouville_subspace(liouville_subspace),
            liouville_subspace)
        if self.evolve_basis == 'eigen':
            rho = self.hamiltonian.transform_vector_to_eigenbasis(rho, liouville_subspace)
        return rho

    def map_between_subspaces(self, state, from_subspace, to_subspace):
        from_idx = self.liouville_subspace_index(from_subspace)
        to_idx = self.liouville_subspace_index(to_subspace)
        n = self.hamiltonian.n_states(self.hilbert_subspace)
        full = np.zeros(n * n, dtype=complex)
        full[from_idx] = state
        return full[to_idx]

    def _block(self, idx, transpose):
        raise NotImplementedError('subclass must provide the Liouvillian')

    @property
    def evolution_super_operator_device(self):
        """Full generator on the model's Hilbert subspace (CUDA complex128)."""
        key = ('full',)
        if key not in self._cache:
            n = self.hamiltonian.n_states(self.hilbert_subspace)
            self._cache[key] = self._block(np.arange(n * n), False)
        return self._cache[key]

    @property
    def evolution_super_operator(self):
        return self.evolution_super_operator_device.cpu().numpy()

    def equation_of_motion(self, liouville_subspace, heisenberg_picture=False):
        """Generator restricted to a subspace, transposed in the Heisenberg
        picture (liouville_space.py:316-341), as a GPU-resident callable."""
        key = ('eom', liouville_subspace, bool(heisenberg_picture))
        if key not in self._cache:
            idx = self.liouville_subspace_index(liouville_subspace)
            self._cache[key] = EquationOfMotion(
                self._block(idx, heisenberg_picture), liouville_subspace,
                heisenberg_picture, self)
        return self._cache[key]
