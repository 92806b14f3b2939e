"""The oracle's drivers against fixtures made by running the reference (CPU).

Pins, before any GPU comparison uses them:
* ``impulsive_probe`` and ``two_dimensional_spectra`` (response.py:174-244,
  430-455) on a 3-site 'gef' chain;
* the block-restricted third-order oracle (oracle/blocks.py) against the dense
  'gef' oracle at 4 sites and against the reference itself on the 128 x 3 x
  128 grids (t1 = t3 = 128 x 2 fs, t2 = 0 / 200 / 500 fs) at 6 and 8 sites;
* the HEOM oracle at the 8-site ring configuration (495 nodes, 200 RK4 steps
  of 0.5 fs) against the reference's own generator.
"""
import os

import numpy as np
import pytest

import oracle as orc
from oracle import blocks
from conftest import ROOT, rel_err
from qspectra_gb300 import workloads as wl


@pytest.fixture(scope='module')
def drivers():
    path = os.path.join(ROOT, 'tests', 'golden', 'reference_golden_drivers.npz')
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def probe_model(g):
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    ham = orc.ElectronicHamiltonianSpec(
        g['probe3_H'], dipoles=g['probe3_dipoles'], disorder=wl.fwhm_for_sd(30.0),
        random_seed=5, energy_spread_extra=float(g['probe3_extra']), bath=bath)
    return orc.RedfieldSpec(ham, bath, 'gef', orc.CM_FS, secular=False)


@pytest.mark.parametrize('sig', ['GSB', 'ESE', 'ESA', 'GSB,ESE,ESA'])
def test_impulsive_probe_matches_reference(drivers, sig):
    m = probe_model(drivers)
    f, X = orc.impulsive_probe(m, drivers['probe3_state'], 200.0, polarization='xy',
                               include_signal=sig)
    assert np.allclose(f, drivers['probe3_f'], rtol=0, atol=1e-9)
    assert rel_err(X, drivers['probe3_' + sig.replace(',', '_')]) < 1e-12


def test_impulsive_probe_ensemble_matches_reference(drivers):
    m = probe_model(drivers)
    _, X = orc.ensemble_average(m, 3, orc.impulsive_probe, drivers['probe3_state'], 200.0,
                                polarization='xx')
    assert rel_err(X, drivers['probe3_ens3']) < 1e-12


@pytest.mark.parametrize('geo', ['-++', '+-+'])
def test_two_dimensional_spectra_matches_reference(drivers, geo):
    m = probe_model(drivers)
    (f1, _, f3), X = orc.two_dimensional_spectra(m, 40.0, [0.0, 20.0, 50.0], geometry=geo)
    assert np.allclose(f1, drivers['twod3_f1'], rtol=0, atol=1e-9)
    assert np.allclose(f3, drivers['twod3_f3'], rtol=0, atol=1e-9)
    assert rel_err(X, drivers['twod3_' + geo]) < 1e-12


def block_model(H1, rw_freq, dipoles):
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    return blocks.BlockRedfield(H1, rw_freq, bath.corr_complex, dipoles, orc.CM_FS)


@pytest.mark.parametrize('geo,pol', [('-++', 'xxxx'), ('+-+', 'xyxz')])
def test_block_oracle_matches_dense_oracle(geo, pol):
    """4 sites, one disorder sample, non-parallel dipoles."""
    H = wl.chain_hamiltonian(n_sites=4, seed=11)
    dip = [[1.0, 0, 0], [0.3, 0.9, 0.1], [-0.5, 0.4, 0.7], [0.2, -0.6, 0.5]]
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    ham = orc.ElectronicHamiltonianSpec(H, dipoles=dip, disorder=wl.fwhm_for_sd(60.0),
                                        random_seed=5,
                                        energy_spread_extra=wl.energy_spread_for_dt(
                                            H, 2.0, orc.CM_FS), bath=bath).sample(2)
    dense = orc.RedfieldSpec(ham, bath, 'gef', orc.CM_FS, secular=False)
    _, ref = orc.third_order_response(dense, 30.0, [0.0, 10.0, 24.0], geometry=geo,
                                      polarization=pol)
    bm = block_model(ham.H1, ham.rw_freq, dip)
    _, got = blocks.third_order_response(bm, 30.0, [0.0, 10.0, 24.0], 2.0, geometry=geo,
                                         polarization=pol)
    assert rel_err(got, ref) < 1e-11


def chain_ensemble_block_oracle(g, N, geo, samples=2):
    base = orc.ElectronicHamiltonianSpec(g['chain{}_H'.format(N)], dipoles=[[1, 0, 0]] * N,
                                         disorder=wl.fwhm_for_sd(60.0), random_seed=3)
    total = 0
    for n in range(samples):
        h = base.sample(n)
        bm = block_model(h.H1, h.rw_freq, [[1, 0, 0]] * N)
        _, r = blocks.third_order_response(bm, 256.0, [0.0, 200.0, 500.0], 2.0, geometry=geo)
        total = total + r
    return total / samples


@pytest.mark.parametrize('N', [6, 8])
@pytest.mark.parametrize('geo', ['-++', '+-+'])
def test_block_oracle_matches_reference_full_grids(drivers, N, geo):
    got = chain_ensemble_block_oracle(drivers, N, geo)
    assert rel_err(got, drivers['chain{}_3rd_ens2_{}'.format(N, geo)]) < 1e-10


def test_heom_oracle_ring8_matches_reference(drivers):
    """The 8-site ring at its configuration size: K = 0, level_cutoff = 5
    (495 nodes x 64), sample 37 of the SD-50 disorder, 200 steps of 0.5 fs."""
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 35, 106)
    base = orc.ElectronicHamiltonianSpec(drivers['ring8_H'], disorder=wl.fwhm_for_sd(50.0),
                                         random_seed=7)
    ham = base.sample(int(drivers['ring8_sample']))
    assert np.allclose(ham.H1, drivers['ring8_sample_H'], rtol=0, atol=1e-9)
    hm = orc.HEOMSpec(ham, bath, 'e', orc.CM_FS, level_cutoff=5, K=0, low_temp_corr=True)
    assert hm.ado_count == 495
    L = hm.eom_matrix('ee')
    y0 = np.zeros(495 * 64, complex)
    y0[0] = 1.0
    traj = orc.rk4_integrate_sparse(L, y0, 200, 0.5)
    assert rel_err(traj[:, :64], drivers['ring8_traj_node0']) < 1e-12
    assert rel_err(traj[-1], drivers['ring8_final_state']) < 1e-12
