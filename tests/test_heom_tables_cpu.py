"""HEOM node tables (host set-up) reproduce the reference generator exactly (CPU)."""
import numpy as np
import pytest
import scipy.sparse as sps

import qspectra_gb300 as qg

CASES = [('K1lc3', dict(K=1, level_cutoff=3, low_temp_corr=True)),
         ('K0lc4', dict(K=0, level_cutoff=4, low_temp_corr=True)),
         ('K0lc3_nolt', dict(K=0, level_cutoff=3, low_temp_corr=False)),
         ('K1lc3_mod', dict(K=1, level_cutoff=3, low_temp_corr=True, modified_HEOM=True))]


def reference_L(golden, tag):
    return sps.coo_matrix((golden['heom2_{}_val'.format(tag)],
                           (golden['heom2_{}_row'.format(tag)],
                            golden['heom2_{}_col'.format(tag)])),
                          shape=tuple(golden['heom2_{}_n'.format(tag)])).toarray()


@pytest.mark.parametrize('tag,kw', CASES)
def test_heom_tables_match_reference(golden, tag, kw):
    ham = qg.ElectronicHamiltonian(golden['heom2_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106))
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, **kw)
    order = np.array([a.reshape(-1) for a in m.ado_indices])
    np.testing.assert_array_equal(order, golden['heom2_{}_order'.format(tag)])
    ref = reference_L(golden, tag)
    L = m.HEOM_tensor('ee').toarray()
    assert np.max(np.abs(L - ref)) <= 1e-13 * np.max(np.abs(ref))
    LT = m.HEOM_tensor('ee', heisenberg_picture=True).toarray()
    assert np.max(np.abs(LT - ref.T)) <= 1e-13 * np.max(np.abs(ref))


def test_ring8_depth4_node_count():
    """8 sites, K = 0, level_cutoff = 5: C(12, 4) = 495 nodes."""
    from qspectra_gb300 import workloads as wl
    ham = qg.ElectronicHamiltonian(wl.ring_hamiltonian(), bath=qg.DebyeBath(qg.CM_K * 300, 35, 106))
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=0, level_cutoff=5)
    assert m.ado_count == 495


@pytest.mark.parametrize('tag,sub,kw', [
    ('multi', 'gg,ge,eg,ee', dict(hilbert_subspace='ge')),
    ('multi2', 'ge,ee', dict(hilbert_subspace='ge')),
    ('aki', 'ee', dict(hilbert_subspace='e', aki_temp_corr=True, low_temp_corr=True)),
    ('aki_nolt', 'ee', dict(hilbert_subspace='e', aki_temp_corr=True, low_temp_corr=False))])
def test_heom_options_match_reference_generators(tag, sub, kw):
    """Multi-block Liouville subspaces and aki_temp_corr (heom.py:298-443):
    the host tables' sparse generator against the reference's own."""
    import os
    import scipy.sparse as sps
    import qspectra_gb300 as qg
    from conftest import ROOT
    with np.load(os.path.join(ROOT, 'tests', 'golden', 'reference_golden_drivers.npz')) as z:
        g = {k: z[k] for k in z.files}
    ham = qg.ElectronicHamiltonian(g['heomopt_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   dipoles=[[1, 0, 0]] * 2)
    m = qg.HEOMModel(ham, unit_convert=qg.CM_FS, K=1, level_cutoff=3, **kw)
    ref = sps.coo_matrix((g['heomopt_{}_val'.format(tag)],
                          (g['heomopt_{}_row'.format(tag)], g['heomopt_{}_col'.format(tag)])),
                         shape=tuple(g['heomopt_{}_n'.format(tag)])).toarray()
    got = m.HEOM_tensor(sub).toarray()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
