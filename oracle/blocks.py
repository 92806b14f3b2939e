"""Block-restricted dense Redfield oracle for third-order response at large N.

TEST INFRASTRUCTURE ONLY (the oracle; never imported by ``qspectra_gb300``).

The dense oracle in ``restatement.py`` forms the whole 'gef' Redfield tensor
exactly as the reference does (qspectra/dynamics/redfield.py:9-74).  At 24
sites that tensor has 301^4 entries (131 GB), so neither the reference nor
that oracle can run the third-order configuration.  This module forms only
the Liouville blocks that the third-order pathways visit ('gg', 'ge', 'eg',
'ee', 'fe'), each as a dense matrix, from the same formulas:

* the system-bath couplings K_i (number operators, hamiltonian.py:593-608)
  and the Hamiltonian are block-diagonal over the g/e/f manifolds, so
  Gamma_abcd = sum_i K_i,ab K_i,cd C(E_d - E_c) (redfield.py:40-60) vanishes
  unless a, b share a manifold and c, d share a manifold;
* R_abcd = delta_ac conj(GS_bd) + delta_bd GS_ac - conj(Gamma_cabd)
  - Gamma_dbac with GS_ac = sum_b Gamma_abbc (redfield.py:62-70) therefore
  maps block XY (a in X, b in Y) into block XY and needs the eigenpairs of
  manifolds X and Y only;
* L = -i [H, .] - R (redfield.py:95-104), scaled by unit_convert
  (redfield.py:146-152).

Everything is evaluated in the eigenbasis of each manifold.  The reference's
site-basis generator is (U (x) U) L (U (x) U)^T with U block-diagonal, and
the RK4 step matrix commutes with that similarity, so propagating eigenbasis
states with eigenbasis dipoles gives the same signals (the signals are
traces).  The pathway logic is the reference's third_order_response
(qspectra/simulate/response.py:267-337): t1 propagation saving the second
commutator, t2 propagation saving the third, t3 in the Heisenberg picture
(the transposed generator, liouville_space.py:316-341) from the fourth
dipole's bra vector, and the contraction einsum('ci,abi').  The t2
trajectory of the states after the second interaction is shared by the
pathways that visit the same block with the same first two interactions
(ESE and ESA): the map is linear, so this changes no number.

Validated against the dense oracle at 4 sites and against reference-generated
fixtures on the 128 x 3 x 128 grids at 6 and 8 sites
(tests/test_oracle_golden.py).
"""
import itertools

import numpy as np
import scipy.linalg

from .restatement import (THIRD_ORDER_PATHWAYS, two_exciton_operator, polarization_vector,
                          time_grid)


def manifold_basis(H1, rw_freq):
    """Per-manifold eigenpairs of the non-rotating Hamiltonian, rotating-frame
    energies (hamiltonian.py:310-328): {'g': (E, U), 'e': ..., 'f': ...}."""
    H1 = np.asarray(H1, float)
    n = len(H1)
    Ee, Ue = scipy.linalg.eigh(H1)
    Hf = two_exciton_operator(H1)
    Ef, Uf = scipy.linalg.eigh(Hf)
    return {'g': (np.zeros(1), np.ones((1, 1))),
            'e': (Ee - rw_freq, Ue),
            'f': (Ef - 2 * rw_freq, Uf)}


def manifold_couplings(n_sites):
    """Number operators n_i restricted to each manifold, as diagonals
    {'g': (N, 1), 'e': (N, N), 'f': (N, N(N-1)/2)} (hamiltonian.py:593-608)."""
    pairs = list(itertools.combinations(range(n_sites), 2))
    occ_f = np.zeros((n_sites, len(pairs)))
    for p, (k, l) in enumerate(pairs):
        occ_f[k, p] = occ_f[l, p] = 1.0
    return {'g': np.zeros((n_sites, 1)), 'e': np.eye(n_sites), 'f': occ_f}


class BlockRedfield:
    """Eigenbasis Redfield blocks of one (sampled) Hamiltonian.

    ``H1`` is the non-rotating one-exciton Hamiltonian, ``corr`` the bath's
    complex correlation function C(omega) (bath.py:84-102) as a scalar
    callable, ``dipoles`` (N, 3).
    """

    def __init__(self, H1, rw_freq, corr, dipoles, unit_convert):
        self.n_sites = len(H1)
        self.uc = unit_convert
        self.basis = manifold_basis(H1, rw_freq)
        occ = manifold_couplings(self.n_sites)
        self.K, self.M, self.GS = {}, {}, {}
        for X, (E, U) in self.basis.items():
            # K_i in the eigenbasis: U^T diag(occ_i) U
            K = np.einsum('sa,is,sb->iab', U, occ[X], U)
            Cw = np.array([[corr(E[d] - E[c]) for d in range(len(E))]
                           for c in range(len(E))])
            self.K[X] = K
            self.M[X] = K * Cw[None]               # M_i,cd = K_i,cd C(E_d - E_c)
            self.GS[X] = np.einsum('iab,ibc->ac', K, self.M[X])
        self.dipoles = np.asarray(dipoles, float)

    def size(self, X):
        return len(self.basis[X][0])

    def generator(self, block):
        """Dense unit_convert * L on block XY, column-stacked local order
        (row a + nX b), a in X, b in Y."""
        X, Y = block
        EX, EY = self.basis[X][0], self.basis[Y][0]
        nX, nY = len(EX), len(EY)
        # arr[b, a, d, c] is L[(a, b), (c, d)]
        arr = np.zeros((nY, nX, nY, nX), complex)
        # R terms: - delta_ac conj(GS^Y_bd) - delta_bd GS^X_ac
        ia = np.arange(nX)
        ib = np.arange(nY)
        arr[:, ia, :, ia] -= np.conj(self.GS[Y])[None, :, :]
        arr[ib, :, ib, :] -= self.GS[X][None, :, :]
        # + conj(Gamma_cabd) = + sum_i K^X_i,ca conj(M^Y_i,bd)
        t3 = np.tensordot(self.K[X], np.conj(self.M[Y]), axes=(0, 0))   # [c, a, b, d]
        arr += t3.transpose(2, 1, 3, 0)
        del t3
        # + Gamma_dbac = + sum_i K^Y_i,db M^X_i,ac
        t4 = np.tensordot(self.K[Y], self.M[X], axes=(0, 0))            # [d, b, a, c]
        arr += t4.transpose(1, 2, 0, 3)
        del t4
        # -i [H, .]: -i (E_a - E_b) on the diagonal
        L = arr.reshape(nX * nY, nX * nY)
        L[np.diag_indices(nX * nY)] += -1j * (EX[None, :] - EY[:, None]).reshape(-1)
        L *= self.uc
        return L

    def dipole(self, polarization, transitions):
        """Eigenbasis dipole blocks {(X, Y): V[X, Y]} for the given
        polarization and transitions '-+' (hamiltonian.py:580-591,
        operator_tools.py:238-270): e <- g and f <- e creation, and their
        transposes for annihilation."""
        mu = self.dipoles @ polarization_vector(polarization)     # (N,)
        N = self.n_sites
        pairs = list(itertools.combinations(range(N), 2))
        up_eg = mu[:, None]                                      # e <- g
        up_fe = np.zeros((len(pairs), N))                        # f <- e
        for p, (k, l) in enumerate(pairs):
            up_fe[p, k] += mu[l]
            up_fe[p, l] += mu[k]
        Ue, Uf = self.basis['e'][1], self.basis['f'][1]
        up_eg = Ue.T @ up_eg
        up_fe = Uf.T @ up_fe @ Ue
        out = {}
        if '+' in transitions:
            out[('e', 'g')] = up_eg
            out[('f', 'e')] = up_fe
        if '-' in transitions:
            out[('g', 'e')] = up_eg.T
            out[('e', 'f')] = up_fe.T
        return out

    def _op(self, V, X, Y):
        if (X, Y) in V:
            return V[(X, Y)]
        return np.zeros((self.size(X), self.size(Y)))

    def commutator_matrix(self, V, frm, to):
        """[V, .] from block frm = X1Y1 to block to = X2Y2 as a dense matrix
        on column-stacked local vectors (liouville_space.py:93-99, 151-209):
        vec(A rho) = (I (x) A) vec rho, vec(rho B) = (B^T (x) I) vec rho."""
        X1, Y1 = frm
        X2, Y2 = to
        n_to, n_from = self.size(X2) * self.size(Y2), self.size(X1) * self.size(Y1)
        out = np.zeros((n_to, n_from), complex)
        if Y1 == Y2:
            out += np.kron(np.eye(self.size(Y1)), self._op(V, X2, X1))
        if X1 == X2:
            out -= np.kron(self._op(V, Y1, Y2).T, np.eye(self.size(X1)))
        return out

    def bra_vector(self, V, block):
        """tr(V rho) as a row over block XY: V[b, a] at (a, b)
        (liouville_space.py:176-181)."""
        X, Y = block
        return self._op(V, Y, X).T.reshape(-1, order='F').astype(complex)


def _rk4_steps(L, y, nsteps, h):
    for _ in range(nsteps):
        k1 = y @ L.T
        k2 = (y + 0.5 * h * k1) @ L.T
        k3 = (y + 0.5 * h * k2) @ L.T
        k4 = (y + h * k3) @ L.T
        y = y + (h / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
    return y


def rk4_trajectory(L, y0, times, h, t0=0.0):
    """States at ``times`` (whole numbers of steps from t0), fixed-step RK4
    (simulate/utils.py:16-109 with zvode replaced by RK4)."""
    y = np.array(y0, complex)
    out, cur = [], t0
    for t in times:
        n = int(round((t - cur) / h))
        y = _rk4_steps(L, y, n, h)
        cur += n * h
        out.append(y)
    return np.stack(out, axis=-2)


def third_order_response(model, coherence_time_max, population_times, dt,
                         geometry='-++', polarization='xxxx', include_signal=None):
    """response.py:267-337 on the eigenbasis blocks of ``model`` (a
    BlockRedfield).  Returns ((t1, t2, t3), response (T1, T2, T3))."""
    t1 = time_grid(coherence_time_max, dt)
    t3 = time_grid(coherence_time_max, dt)
    t2 = np.asarray(population_times, float)
    gens = {}

    def gen(block, heisenberg=False):
        if block not in gens:
            gens[block] = model.generator(block)
        return gens[block].T if heisenberg else gens[block]

    total = 0
    t2_cache = {}
    for name, path in THIRD_ORDER_PATHWAYS[geometry].items():
        if include_signal is not None and name not in include_signal:
            continue
        subs = path.split('->')
        V = [model.dipole(p, tr) for p, tr in zip(polarization, geometry + '-')]
        rho0 = np.ones(1, complex)                     # thermal 'gg' state
        v_rho0 = model.commutator_matrix(V[0], subs[0], subs[1]) @ rho0
        key = (subs[1], subs[2])
        if key not in t2_cache:
            L1 = gen(subs[1])
            S1 = model.commutator_matrix(V[1], subs[1], subs[2])
            v_rho1 = rk4_trajectory(L1, v_rho0, t1, dt) @ S1.T        # (T1, n2)
            t2_cache[key] = rk4_trajectory(gen(subs[2]), v_rho1, t2, dt)  # (T1, T2, n2)
        S2 = model.commutator_matrix(V[2], subs[2], subs[3])
        v_rho2 = t2_cache[key] @ S2.T                                  # (T1, T2, n3)
        bra = model.bra_vector(V[3], subs[3])
        v_gt3 = rk4_trajectory(gen(subs[3], heisenberg=True), bra, t3, dt)   # (T3, n3)
        total = total + np.einsum('ci,abi->abc', v_gt3, v_rho2)
    return (t1, t2, t3), total
