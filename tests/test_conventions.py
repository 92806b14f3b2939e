"""The reference's own convention tests, restated against the host package (CPU only).

Sources: tests/test_liouville_space.py:11-138, tests/test_operator_tools.py:70-150,
tests/test_hamiltonian.py:19-125 and tests/test_simulate_utils.py:58-81 of the
reference.
"""
import numpy as np
import pytest
from numpy.testing import assert_allclose, assert_equal

import qspectra_gb300 as qg
from qspectra_gb300 import operator_tools as ot
from qspectra_gb300.dynamics import liouville_space as ls
from qspectra_gb300.simulate import utils


def test_liouville_subspace_index():
    assert_equal(ls.liouville_subspace_index('eg,ge', 'ge', 2), [1, 2, 3, 6])
    assert_equal(ls.liouville_subspace_index('eg,fe', 'gef', 2), [1, 2, 7, 11])
    assert_equal(ls.liouville_subspace_index('gg,ee,ff', 'gef', 2), [0, 5, 6, 9, 10, 15])
    with pytest.raises(ot.SubspaceError):
        ls.liouville_subspace_index('ef', 'ge', 2)
    assert_equal(ls.liouville_subspace_index('gg', 'ge', 1, 2), [0, 1, 4, 5])
    assert_equal(ls.liouville_subspace_index('eg', 'ge', 1, 2), [2, 3, 6, 7])


def test_all_liouville_subspaces():
    assert ls.all_liouville_subspaces('g') == 'gg'
    assert ls.all_liouville_subspaces('ge') == 'gg,ge,eg,ee'
    assert ls.all_liouville_subspaces('gef') == 'gg,ge,gf,eg,ee,ef,fg,fe,ff'


def test_tensor_to_super_and_vectorisation():
    rng = np.random.RandomState(0)
    R = rng.rand(2, 2, 2, 2)
    S = ls.tensor_to_super(R)
    for i, j, k, l in np.ndindex(2, 2, 2, 2):
        assert R[i, j, k, l] == S[i + 2 * j, k + 2 * l]
    rho_v = 0.25 * np.array([1., 2 + 2j, 2 - 2j, 3])
    rho_d = 0.25 * np.array([[1., 2 - 2j], [2 + 2j, 3]])
    assert_allclose(ls.matrix_to_ket_vec(rho_d), rho_v)
    assert_allclose(ls.ket_vec_to_matrix(rho_v), rho_d)
    assert_allclose(ls.matrix_to_bra_vec(rho_d), 0.25 * np.array([1, 2 - 2j, 2 + 2j, 3]))
    op = rng.rand(2, 2) + 1j * rng.rand(2, 2)
    assert_allclose(ls.super_left_matrix(op) @ rho_v, ls.matrix_to_ket_vec(op @ rho_d))
    assert_allclose(ls.super_right_matrix(op) @ rho_v, ls.matrix_to_ket_vec(rho_d @ op))
    assert_allclose(ls.super_commutator_matrix(op) @ rho_v,
                    ls.matrix_to_ket_vec(op @ rho_d - rho_d @ op))


def test_operator_tools():
    M = np.array([[1., 2 - 2j], [2 + 2j, 3]])
    assert ot.all_states(1) == [[], [0]]
    assert ot.all_states(2) == [[], [0], [1], [0, 1]]
    assert ot.all_states(2, 'ge') == [[], [0], [1]]
    assert_allclose(ot.operator_1_to_2(M), [[4]])
    assert_allclose(ot.operator_1_to_2(np.diag([1, 10, 100])), np.diag([11, 101, 110]))
    assert_allclose(ot.operator_extend(M, 'e'), M)
    assert_allclose(ot.operator_extend(M, 'g'), [[0]])
    assert_allclose(ot.operator_extend(M, 'f'), [[4]])
    assert_allclose(ot.operator_extend(M), [[0, 0, 0, 0], [0, 1, 2 - 2j, 0],
                                            [0, 2 + 2j, 3, 0], [0, 0, 0, 4]])
    assert_allclose(ot.transition_operator(0, 2, 'ge'), [[0, 1, 0], [1, 0, 0], [0, 0, 0]])
    assert_allclose(ot.transition_operator(0, 2), [[0, 1, 0, 0], [1, 0, 0, 0],
                                                  [0, 0, 0, 1], [0, 0, 1, 0]])
    assert_allclose(ot.transition_operator(0, 2, 'gef', ''), np.zeros((4, 4)))
    assert_allclose(ot.transition_operator(0, 2, 'gef', '-'),
                    [[0, 1, 0, 0], [0, 0, 0, 0], [0, 0, 0, 1], [0, 0, 0, 0]])
    assert_allclose(ot.transition_operator(0, 2, 'gef', '+'),
                    [[0, 0, 0, 0], [1, 0, 0, 0], [0, 0, 0, 0], [0, 0, 1, 0]])
    assert_equal(ot.n_excitations(1), [1, 1, 0])
    assert_equal(ot.n_excitations(3, 2), [2, 6, 6])
    assert ot.extract_subspace('gg,eg->gg') == ['g', 'e']
    assert ot.full_liouville_subspace('ge,ee') == 'gg,ge,eg,ee'
    assert ot.hilbert_subspace_index('e', 'gef', 3) == slice(1, 4)
    assert ot.hilbert_subspace_index('f', 'ef', 3) == slice(3, 6)
    occ = ot.occupation_table(3, 'gef')
    for i in range(3):
        H = qg.ElectronicHamiltonian(np.eye(3), bath=qg.DebyeBath(1, 1, 1))
        assert_allclose(np.diag(occ[i]), H.number_operator(i, 'gef'))


def construct_elec(M):
    return qg.ElectronicHamiltonian(M, bath=None, dipoles=[[1, 0, 0], [0, 1, 0]],
                                    disorder=1, energy_spread_extra=1.0)


def test_hamiltonian_properties():
    H = construct_elec(np.array([[1., 0], [0, 3]]))
    assert H.n_sites == 2 and H.n_states('gef') == 4
    assert H.freq_step == 10.0 and H.time_step == 0.1
    assert_allclose(H.E('gef'), [0, 1, 3, 4])
    assert H.transition_energy == 2
    assert_allclose(H.dipole_operator('gef', 'x', '-+'),
                    [[0, 1, 0, 0], [1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])
    with pytest.raises(qg.HamiltonianError):
        qg.ElectronicHamiltonian(np.eye(2)).dipole_operator()
    with pytest.raises(qg.HamiltonianError):
        H.system_bath_couplings()
    Hr = H.in_rotating_frame()
    assert_allclose(Hr.H('e'), [[-1, 0], [0, 1]])
    assert_allclose(Hr.E('gef'), [0, -1, 1, 0])
    assert Hr.freq_step == 4.0
    assert H.in_rotating_frame(2) == H.in_rotating_frame(2).in_rotating_frame(2)


def test_sampling_commutes_with_rotating_frame():
    H = construct_elec(np.array([[1., 0], [0, 3]]))
    s = H.sample(0)
    assert s != H
    assert s.time_step == H.time_step
    a = H.in_rotating_frame(10).sample(0)
    b = s.in_rotating_frame(10)
    assert_allclose(a.H('gef'), b.H('gef'))
    assert [h.H_1exc.tolist() for h in H.sample_ensemble(3)] == \
        [H.sample(n).H_1exc.tolist() for n in range(3)]
    off = H.disorder_offsets(3)
    for n in range(3):
        assert_allclose(np.diag(H.sample(n).H_1exc) - np.diag(H.H_1exc), off[n])


def test_liouville_model_thermal_and_mapping():
    class Example(ls.LiouvilleSpaceModel):
        @property
        def time_step(self):
            return 1.0
    m = Example(qg.ElectronicHamiltonian(np.eye(4)))
    assert_allclose(m.thermal_state('gg'), [1])
    assert_allclose(m.thermal_state('gg,eg,ge,ee'), ot.unit_vec(0, 25))
    assert_allclose(m.thermal_state('ee'), 0.25 * np.eye(4).reshape(-1))
    assert_allclose(m.map_between_subspaces(np.ones(25), 'gg,eg,ge,ee', 'gg'), [1])
    assert_allclose(m.map_between_subspaces(np.ones(25), 'gg,eg,ge,ee', 'gf'), np.zeros(6))


def test_symmetrize_and_constant():
    assert utils.is_constant([1, 1, 1])
    assert not utils.is_constant([1, 1, 1, 0])
    assert utils.is_constant([1, 1, 1, 1], positive=True)
    cases = [([0, 1, 2], [1, 1, 1], [-2, -1, 0, 1, 2], [0, 0, 1, 1, 1]),
             ([0.5, 1.5], [1, 1], [-1.5, -0.5, 0.5, 1.5], [0, 0, 1, 1]),
             ([-2, -1], [1, 1], [-2, -1, 0, 1, 2], [1, 1, 0, 0, 0]),
             ([-1.25, -0.25], [1, 1], [-1.25, -0.25, 0.75], [1, 1, 0])]
    for t, x, ts, xs in cases:
        a, b = utils._symmetrize(t, x)
        assert_allclose(a, ts)
        assert_allclose(b, xs)
