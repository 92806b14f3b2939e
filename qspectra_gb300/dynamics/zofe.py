"""ZOFE master equation (qspectra/dynamics/zofe.py).

The zeroth-order functional expansion couples the density matrix to one
auxiliary operator O[pm][s] per pseudomode and site; the equation of motion
is quadratic in the state, so it is integrated stage by stage on the GPU
(``qsx_zofe_rk4``, one thread-block cluster per sample) rather than through
a propagator matrix.  States use the reference's vector layout: rho in
column-major order followed by O (numb_pm, n_sites, n, n) in column-major
order.
"""
import numpy as np
import torch

from .. import _native
from ..bath import PseudomodeBath
from .base import DynamicalModel, SystemOperator


def _split(state, n, oop_shape):
    """(..., M) state -> rho (..., n, n) and O (..., npm, N, n, n) views."""
    lead = state.shape[:-1]
    n2 = n * n
    rho = state[..., :n2].reshape(lead + (n, n)).swapaxes(-1, -2)
    npm, N = oop_shape[0], oop_shape[1]
    O = state[..., n2:].reshape(lead + (n, n, N, npm))
    axes = tuple(range(len(lead))) + tuple(len(lead) + k for k in (3, 2, 1, 0))
    return rho, O.transpose(axes) if isinstance(O, np.ndarray) else O.permute(axes)


def _join(rho, O):
    """Inverse of _split."""
    lib = np if isinstance(rho, np.ndarray) else torch
    lead = rho.shape[:-2]
    k = len(lead)
    r = rho.swapaxes(-1, -2).reshape(lead + (-1,))
    axes = tuple(range(k)) + tuple(k + a for a in (3, 2, 1, 0))
    o = (O.transpose(axes) if lib is np else O.permute(axes)).reshape(lead + (-1,))
    return lib.concatenate([r, o], axis=-1) if lib is np else torch.cat([r, o], dim=-1)


class ZOFESpaceOperator(SystemOperator):
    """An operator acting on rho and on every auxiliary operator
    (zofe.py:8-42).  States may be numpy arrays or CUDA tensors (..., M)."""

    def __init__(self, operator, liouv_subspace_map, dynamical_model):
        self.operator = np.asarray(operator)
        self.dynamical_model = dynamical_model

    def _op(self, like):
        if isinstance(like, np.ndarray):
            return self.operator
        return torch.as_tensor(self.operator, dtype=torch.complex128, device=like.device)

    def _parts(self, state):
        m = self.dynamical_model
        x = state if isinstance(state, torch.Tensor) else np.asarray(state, dtype=complex)
        return _split(x, m.n_states, m.oop_shape)

    def left_multiply(self, state):
        rho, O = self._parts(state)
        A = self._op(rho)
        return _join(A @ rho, A @ O)

    def right_multiply(self, state):
        rho, O = self._parts(state)
        A = self._op(rho)
        return _join(rho @ A, O @ A)

    def commutator(self, state):
        return self.left_multiply(state) - self.right_multiply(state)

    def expectation_value(self, state):
        """tr(operator rho) (zofe.py:38-41)."""
        rho, _ = self._parts(state)
        A = self._op(rho)
        return (A * rho.swapaxes(-1, -2)).sum((-1, -2))

    @property
    def expectation_row(self):
        """(n*n,) row over column-major rho with row . vec(rho) = tr(A rho)."""
        return self.operator.reshape(-1)


class ZOFEEquationOfMotion:
    """The ZOFE right-hand side on the GPU; ``integrate`` runs its RK4 loop in
    one kernel.  ``H`` is (n, n) or per sample (S, n, n)."""

    def __init__(self, model, H):
        self.model = model
        self.H = H
        self.heisenberg_picture = False

    @property
    def dim(self):
        return self.model.state_size

    def __call__(self, t, state):
        x = state if isinstance(state, torch.Tensor) else torch.as_tensor(
            np.asarray(state, dtype=complex))
        x = x.to(device='cuda', dtype=torch.complex128)
        Ld, G, w = self.model.zofe_tables()
        out = _native.zofe_rk4(self.H, Ld, G, w, x, 0, 1.0, self.model.unit_convert,
                               hermit=self.model.zofe_hermit,
                               mode=1)['rhs']
        out = out[0] if x.dim() == 1 else out
        return out if isinstance(state, torch.Tensor) else out.cpu().numpy()


class ZOFEModel(DynamicalModel):
    """ZOFE master equation with one pseudomode bath per site (zofe.py:44-229).

    ``rho_hermit`` takes rho^H in place of rho in the last term of rho's
    right-hand side (the conjugate transpose of the second term), and with
    ``ham_hermit`` in the third as well (zofe.py:179-192); both are exact for
    a Hermitian rho.  ``ham_hermit`` alone selects an algebraically equal form
    for Hermitian Hamiltonians (always the case here).
    """
    system_operator = ZOFESpaceOperator

    def __init__(self, hamiltonian, rw_freq=None, hilbert_subspace='gef',
                 unit_convert=1, ham_hermit=False, rho_hermit=False):
        super().__init__(hamiltonian, rw_freq, hilbert_subspace, unit_convert)
        if not isinstance(self.hamiltonian.bath, PseudomodeBath):
            raise NotImplementedError('ZOFE only implemented for baths of type '
                                      'PseudomodeBath')
        numb_pm = self.hamiltonian.bath.numb_pm
        n_sit = self.hamiltonian.n_sites
        n_stat = self.hamiltonian.n_states(self.hilbert_subspace)
        self.oop_shape = (numb_pm, n_sit, n_stat, n_stat)
        self.ham_hermit = ham_hermit
        self.rho_hermit = rho_hermit
        self._tables = None

    @property
    def n_states(self):
        return self.oop_shape[2]

    @property
    def zofe_hermit(self):
        """The kernel's form flags for rho_hermit / ham_hermit."""
        if not self.rho_hermit:
            return 0
        return _native.QSX_ZOFE_RHO_HERMIT | (_native.QSX_ZOFE_HAM_HERMIT if self.ham_hermit
                                              else 0)

    @property
    def state_size(self):
        n = self.n_states
        return n * n + int(np.prod(self.oop_shape))

    def zofe_tables(self):
        """(Ld, Gamma, w) on the GPU: the diagonals of L_n = -(site number
        operators) (zofe.py:219-222) and the pseudomode parameters
        Gamma = Omega^2 huang, w = i Omega + gamma (zofe.py:224-229)."""
        if self._tables is None:
            ham = self.hamiltonian
            couplings = -np.asanyarray(ham.system_bath_couplings(self.hilbert_subspace))
            diag = np.array([np.diag(c) for c in couplings])
            if np.abs(couplings - np.array([np.diag(d) for d in diag])).max() > 0:
                raise NotImplementedError('the GPU ZOFE path needs diagonal couplings')
            bath = ham.bath
            shape = self.oop_shape[:2]
            Om = np.broadcast_to(np.asarray(bath.Omega, dtype=complex), shape)
            ga = np.broadcast_to(np.asarray(bath.gamma, dtype=complex), shape)
            hu = np.broadcast_to(np.asarray(bath.huang, dtype=complex), shape)
            dev = torch.device('cuda', torch.cuda.current_device())
            self._tables = (torch.as_tensor(diag.real.copy(), dtype=torch.float64, device=dev),
                            torch.as_tensor(Om ** 2 * hu, device=dev),
                            torch.as_tensor(1j * Om + ga, device=dev))
        return self._tables

    def density_matrix_to_state_vector(self, rho0, liouville_subspace=None):
        state0 = np.asarray(rho0).reshape(-1, order='F')
        return np.append(state0, np.zeros(int(np.prod(self.oop_shape)), dtype=complex))

    def state_vec_to_operators(self, rho_oop_vec):
        n = self.n_states
        v = np.asarray(rho_oop_vec)
        rho = v[:n * n].reshape((n, n), order='F')
        oop = v[n * n:].reshape(self.oop_shape, order='F')
        return rho, oop

    def operators_to_state_vec(self, rho, oop):
        return np.append(np.asarray(rho).reshape(-1, order='F'),
                         np.asarray(oop).reshape(-1, order='F'))

    def state_vector_to_density_matrix(self, rhos):
        return np.array([self.state_vec_to_operators(k)[0] for k in rhos])

    def thermal_state(self, _=None):
        rho0 = self.hamiltonian.thermal_state(self.hilbert_subspace)
        return self.density_matrix_to_state_vector(rho0)

    def map_between_subspaces(self, state, from_subspace, to_subspace):
        return state

    def equation_of_motion(self, liouville_subspace=None, heisenberg_picture=False):
        if heisenberg_picture:
            raise NotImplementedError('ZOFE not implemented in the Heisenberg picture')
        H = torch.as_tensor(self.hamiltonian.H(self.hilbert_subspace), dtype=torch.float64,
                            device=torch.device('cuda', torch.cuda.current_device()))
        return ZOFEEquationOfMotion(self, H)


def excitation_numbers(model):
    """Excitations of each basis state of the model's Hilbert subspace."""
    from ..operator_tools import hilbert_subspace_index
    N = model.hamiltonian.n_sites
    out = np.zeros(model.n_states)
    for k, manifold in enumerate('gef'):
        if manifold in model.hilbert_subspace:
            sl = hilbert_subspace_index(manifold, model.hilbert_subspace, N)
            out[sl] = k
    return out


def ensemble_inputs(model, ensemble_size, start=0):
    """(H (S, n, n) float64 CUDA rotating-frame Hamiltonians, thermal states
    (S, M) complex128 CUDA) of the disorder samples start..start+S-1.

    A pseudomode bath defines no temperature, so each sample's thermal state
    is its ground state: the mean of the lowest eigenprojectors of the
    non-rotating Hamiltonian (hamiltonian.py:25-46, 164-175).
    """
    from ..simulate.ensemble import SampleBatch
    batch = SampleBatch(model, ensemble_size, start)
    H = batch.H(model.hilbert_subspace)
    Hn = H.cpu().numpy() + np.diag(model.rw_freq * excitation_numbers(model))[None]
    E, U = np.linalg.eigh(Hn)
    n = model.n_states
    rhos = np.empty((ensemble_size, n, n), dtype=complex)
    for s in range(ensemble_size):
        low = np.nonzero(E[s] == E[s, 0])[0]
        rhos[s] = np.mean([np.outer(U[s][:, i], U[s][:, i]) for i in low], axis=0)
    M = model.state_size
    y = np.zeros((ensemble_size, M), dtype=complex)
    y[:, :n * n] = rhos.transpose(0, 2, 1).reshape(ensemble_size, n * n)
    return H, torch.as_tensor(y, device=H.device)
