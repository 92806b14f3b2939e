"""Hilbert-space bookkeeping for electronic (Frenkel exciton) systems.

Host-side set-up code, the same role as qspectra/operator_tools.py: it builds
the small index tables and operator matrices that the GPU kernels consume.
States are hard-core boson occupations: the ground state, one excitation on a
site, or two excitations on a pair of sites i < j.
"""
import itertools

import numpy as np


class SubspaceError(Exception):
    """Raised for a Hilbert or Liouville subspace the model does not contain
    (operator_tools.py:273-276)."""


MANIFOLDS = 'gef'


def n_excitations(n_sites=1, n_vibrational_states=1):
    """Sizes of the 0-, 1- and 2-excitation manifolds (operator_tools.py:279-285)."""
    return np.array([1, n_sites, n_sites * (n_sites - 1) // 2]) \
        * n_vibrational_states


def unit_vec(n, N, dtype=complex):
    """n-th unit vector of length N (operator_tools.py:34-40)."""
    v = np.zeros(N, dtype=dtype)
    v[n] = 1
    return v


def all_states(N, subspace='gef'):
    """Excited-site lists of every state in ``subspace`` (operator_tools.py:122-152)."""
    states = []
    if 'g' in subspace:
        states.append([])
    if 'e' in subspace:
        states.extend([i] for i in range(N))
    if 'f' in subspace:
        states.extend(list(p) for p in itertools.combinations(range(N), 2))
    return states


def operator_1_to_2(operator1):
    """Representation of Σ A_nm a†_n a_m on the pair states (operator_tools.py:155-191)."""
    A = np.asarray(operator1)
    n = len(A)
    pairs = list(itertools.combinations(range(n), 2))
    out = np.zeros((len(pairs), len(pairs)), dtype=A.dtype)
    for r, (i, j) in enumerate(pairs):
        for c, (k, l) in enumerate(pairs):
            v = 0
            if i == k:
                v = v + A[j, l]
            if i == l:
                v = v + A[j, k]
            if j == k:
                v = v + A[i, l]
            if j == l:
                v = v + A[i, k]
            out[r, c] = v
    return out


def operator_extend(operator1, subspace='gef'):
    """Extend a 1-exciton operator over the requested manifolds (operator_tools.py:194-235)."""
    A = np.asarray(operator1)
    blocks = []
    if 'g' in subspace:
        blocks.append(np.zeros((1, 1), dtype=A.dtype))
    if 'e' in subspace:
        blocks.append(A)
    if 'f' in subspace:
        blocks.append(operator_1_to_2(A))
    size = sum(len(b) for b in blocks)
    out = np.zeros((size, size), dtype=A.dtype)
    pos = 0
    for b in blocks:
        out[pos:pos + len(b), pos:pos + len(b)] = b
        pos += len(b)
    return out


def transition_operator(n, n_sites, subspace='gef', include_transitions='-+'):
    """Create ('+') and/or annihilate ('-') an excitation on site n (operator_tools.py:238-270)."""
    states = all_states(n_sites, subspace)
    where = {tuple(st): k for k, st in enumerate(states)}
    out = np.zeros((len(states), len(states)))
    for c, sj in enumerate(states):
        # create: the state with site n added; destroy: the state with n removed
        if '+' in include_transitions and n not in sj:
            r = where.get(tuple(sorted(sj + [n])))
            if r is not None:
                out[r, c] = 1
        if '-' in include_transitions and n in sj:
            r = where.get(tuple(x for x in sj if x != n))
            if r is not None:
                out[r, c] = 1
    return out


def occupation_table(n_sites, subspace='gef'):
    """occ[i, s] = 1 when site i is excited in state s.

    The number operators a†_i a_i that couple each site to its bath
    (hamiltonian.py:593-608) are diag(occ[i]); the GPU kernels take this
    table instead of N dense n×n matrices.
    """
    states = all_states(n_sites, subspace)
    occ = np.zeros((n_sites, len(states)))
    for s, st in enumerate(states):
        occ[st, s] = 1.0
    return occ


def excitation_to_number(excitation):
    return {'g': 0, 'e': 1, 'f': 2}[excitation]


def extract_subspace(subspaces_string):
    """Smallest Hilbert subspace containing a Liouville subspace string (operator_tools.py:292-298)."""
    return sorted(set(subspaces_string) - {',', '-', '>'},
                  key=excitation_to_number)


def full_liouville_subspace(subspaces_string):
    """Tensor-product Liouville subspace of the contained manifolds (operator_tools.py:301-308)."""
    h = extract_subspace(subspaces_string)
    return ','.join(a + b for a in h for b in h)


def hilbert_subspace_index(subspace, all_subspaces, n_sites,
                           n_vibrational_states=1):
    """Slice of one manifold inside ``all_subspaces`` (operator_tools.py:311-335)."""
    sizes = n_excitations(n_sites, n_vibrational_states)
    if subspace not in all_subspaces:
        raise SubspaceError("{} not in set of all subspaces '{}'".format(
            subspace, all_subspaces))
    start = 0
    for letter in all_subspaces:
        size = int(sizes[MANIFOLDS.index(letter)])
        if letter == subspace:
            return slice(start, start + size)
        start += size


def _infer_kron(X, U):
    U = np.asarray(U)
    if U.ndim != 2 or U.shape[0] != U.shape[1]:
        raise ValueError('basis transformation must be a square matrix')
    N = len(U)
    if X.shape[-1] == N:
        return U
    if X.shape[-1] == N * N:
        return np.kron(U, U)
    raise ValueError('basis transformation incompatible with operator '
                     'dimensions')


def basis_transform_operator(X, U):
    """U† X U in Hilbert or Liouville space (operator_tools.py:59-87)."""
    X = np.asarray(X)
    if X.ndim != 2:
        raise ValueError('operator must have ndim=2')
    W = _infer_kron(X, U)
    return W.conj().T @ X @ W


def basis_transform_vector(rho, U):
    """State vector(s) into the basis U (operator_tools.py:90-119)."""
    rho = np.asarray(rho)
    W = _infer_kron(rho, U)
    return np.tensordot(rho, W.conj().T, axes=(-1, -1))
