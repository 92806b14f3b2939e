"""Host logic of the batched third-order engine (no GPU needed)."""
import numpy as np
import pytest
import torch

import qspectra_gb300 as qg
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from qspectra_gb300 import operator_tools as ot
from qspectra_gb300.dynamics import liouville_space as ls
from qspectra_gb300.simulate.third_order import pair_tables, powers_minus_identity, supports


def _transition_by_definition(n, n_sites, subspace, transitions):
    """transition_operator straight from its definition (operator_tools.py:238-270)."""
    states = ot.all_states(n_sites, subspace)
    out = np.zeros((len(states), len(states)))
    for r, si in enumerate(states):
        for c, sj in enumerate(states):
            create = '+' in transitions and si == sorted(sj + [n])
            destroy = '-' in transitions and sorted(si + [n]) == sj
            if create or destroy:
                out[r, c] = 1
    return out


@pytest.mark.parametrize('n_sites', [1, 2, 4])
def test_transition_operator_matches_definition(n_sites):
    for sub in ('g', 'e', 'ge', 'ef', 'gef'):
        for tr in ('-', '+', '-+'):
            for n in range(n_sites):
                assert np.array_equal(ot.transition_operator(n, n_sites, sub, tr),
                                      _transition_by_definition(n, n_sites, sub, tr))


def _chain_model(n_sites, secular=False, subspace='gef'):
    H = wl.chain_hamiltonian(n_sites=n_sites, seed=3)
    bath = qg.DebyeBath(qg.CM_K * 300, 40, 100)
    ham = qg.ElectronicHamiltonian(H, bath=bath, dipoles=[[1, 0, 0]] * n_sites)
    return qg.RedfieldModel(ham, hilbert_subspace=subspace, unit_convert=qg.CM_FS,
                            secular=secular)


@pytest.mark.parametrize('spec', ['gg->ge', 'ge->ee', 'eg->gg', 'ee->fe', 'fe->ee',
                                  'ee->eg', 'gg->eg', 'eg->fg', 'gef->gef'])
def test_restricted_maps_equal_sliced_kron(spec):
    """The restricted left/right/commutator maps equal slices of the full
    kron super-operators (liouville_space.py:93-148, 176-209)."""
    m = _chain_model(3)
    parts = spec.split('->')
    full = {'gef': ','.join(a + b for a in 'gef' for b in 'gef')}
    parts = [full.get(p, p) for p in parts]
    for tr in ('-', '+', '-+'):
        op = m.dipole_operator('->'.join(parts), 'x', tr)
        V = np.asarray(op.operator)
        mesh = np.ix_(op.to_indices, op.from_indices)
        left = ls.super_left_matrix(V)[mesh]
        right = ls.super_right_matrix(V)[mesh]
        assert np.array_equal(op._restricted('left'), left)
        assert np.array_equal(op._restricted('right'), right)
        assert np.array_equal(op.commutator_matrix, left - right)
        tr_full = np.identity(len(V)).reshape(-1)[op.to_indices]
        assert np.allclose(op.expectation_row, tr_full.dot(left), rtol=0, atol=0)


def test_pair_tables_follow_all_states():
    for n in (2, 3, 6, 24):
        pair_sites, site_pairs = pair_tables(n)
        f_states = [s for s in ot.all_states(n, 'f')]
        assert [list(p) for p in pair_sites] == f_states
        for i in range(n):
            listed = sorted(site_pairs[i])
            expect = [p for p, s in enumerate(f_states) if i in s]
            assert listed == expect


def test_powers_minus_identity():
    rng = np.random.RandomState(0)
    D = 0.05 * (rng.randn(3, 6, 6) + 1j * rng.randn(3, 6, 6))
    gaps = [0, 1, 7, 100, 150]
    out = powers_minus_identity(torch.as_tensor(D), gaps, mul_add=lambda A, B, C: A @ B + C)
    for k in gaps:
        ref = np.array([np.linalg.matrix_power(np.eye(6) + d, k) - np.eye(6) for d in D])
        assert np.max(np.abs(out[k].numpy() - ref)) < 1e-12 * max(1, np.abs(ref).max())


def test_csr_map_host_arrays():
    rng = np.random.RandomState(1)
    A = (rng.rand(9, 13) < 0.3) * (rng.randn(9, 13) + 1j * rng.randn(9, 13))
    A[4] = 0
    m = _native.CsrMap(A, device='cpu')
    rowptr, cols, vals = m.rowptr.numpy(), m.cols.numpy(), m.vals.numpy()
    back = np.zeros_like(A)
    for r in range(9):
        for k in range(rowptr[r], rowptr[r + 1]):
            back[r, cols[k]] += vals[k]
    assert np.array_equal(back, A)
    z = _native.CsrMap(np.zeros((3, 4)), device='cpu')
    assert z.rowptr.numpy().tolist() == [0, 0, 0, 0]


def test_engine_eligibility():
    assert supports(_chain_model(4), '-++')
    assert supports(_chain_model(4), '+-+')
    assert not supports(_chain_model(4), '++-')
    assert not supports(_chain_model(4, secular=True), '-++')
    assert not supports(_chain_model(3, subspace='ge'), '-++')
