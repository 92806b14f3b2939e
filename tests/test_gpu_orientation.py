"""Orientation averages on the GPU path against the reference's own runs:
random ensemble orientations (decorators.py:40-64, hamiltonian.py:552-575)
and exact isotropic averages (decorators.py:67-125) of the absorption
spectrum, pumped dynamics and third-order response."""
import numpy as np
import pytest

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOLS = [('fp64', 1e-10), ('fp32', 1e-4)]


def ori4_model(golden):
    ham = qg.ElectronicHamiltonian(golden['ori4_H'], bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=golden['ori4_dipoles'],
                                   disorder=wl.fwhm_for_sd(40.0), random_seed=3,
                                   energy_spread_extra=float(golden['ori4_extra']))
    return qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)


def ori3_model(golden, secular=False):
    ham = qg.ElectronicHamiltonian(golden['chain3_H'], bath=qg.DebyeBath(qg.CM_K * 300, 40, 100),
                                   dipoles=golden['ori3_dipoles'],
                                   disorder=wl.fwhm_for_sd(30.0), random_seed=5,
                                   energy_spread_extra=float(golden['chain3_extra']))
    return qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS,
                            secular=secular)


def test_orientation_rotations_match_reference_draws(golden):
    ham = ori4_model(golden).hamiltonian
    R = ham.orientation_rotations(4)
    dips = np.einsum('smn,in->sim', R, golden['ori4_dipoles'])
    assert np.abs(dips - golden['ori4_sample_dipoles']).max() < 1e-14


@pytest.mark.parametrize('precision,tol', TOLS)
def test_absorption_random_orientations(golden, precision, tol):
    m = ori4_model(golden)
    f, X = qg.absorption_spectra(m, 512.0, ensemble_size=4, ensemble_random_orientations=True,
                                 precision=precision)
    assert np.allclose(f, golden['ori4_abs_f'], rtol=1e-12, atol=0)
    assert rel_err(X, golden['ori4_abs_rand']) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_absorption_isotropic(golden, precision, tol):
    m = ori4_model(golden)
    _, X = qg.absorption_spectra(m, 512.0, polarization=[0.3, 'x'],
                                 exact_isotropic_average=True, precision=precision)
    assert rel_err(X, golden['ori4_abs_iso']) < tol
    _, X = qg.absorption_spectra(m, 512.0, ensemble_size=3, ensemble_random_orientations=True,
                                 exact_isotropic_average=True, precision=precision)
    assert rel_err(X, golden['ori4_abs_iso_rand']) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_fields_orientation_averages(golden, precision, tol):
    m = ori4_model(golden)
    pump = qg.GaussianPulse(carrier_freq=float(np.mean(np.diag(golden['ori4_H']))), fwhm=20.0,
                            t_peak=0.0, scale=1e-2, freq_convert=qg.CM_FS)
    t, st = qg.simulate_pump(m, pump, polarization=0.5, time_extra=30.0,
                             exact_isotropic_average=True, precision=precision)
    assert np.allclose(t, golden['ori4_pump_iso_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['ori4_pump_iso']) < tol
    assert rel_err(st[:, 1:], golden['ori4_pump_iso'][:, 1:]) < 10 * tol
    p1 = qg.GaussianPulse(carrier_freq=12250.0, fwhm=15.0, t_peak=-10.0, scale=5e-3,
                          freq_convert=qg.CM_FS)
    p2 = qg.GaussianPulse(carrier_freq=12450.0, fwhm=25.0, t_peak=20.0, scale=8e-3,
                          freq_convert=qg.CM_FS)
    t, st = qg.simulate_with_fields(m, [p1, p2], geometry='-+', polarization='xy',
                                    time_extra=30.0, ensemble_size=3,
                                    ensemble_random_orientations=True, precision=precision)
    assert np.allclose(t, golden['ori4_fields_rand_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['ori4_fields_rand']) < tol
    assert rel_err(st[:, 1:], golden['ori4_fields_rand'][:, 1:]) < 10 * tol


CASES = [('ori3_3rd_iso_-++', '-++', [0, 0, 0.5, 0.5], None, False, True),
         ('ori3_3rd_isoxxyy_+-+', '+-+', 'xxyy', None, False, True),
         ('ori3_3rd_rand_-++', '-++', 'xyxz', 3, True, False),
         ('ori3_3rd_iso_rand_+-+', '+-+', 'xxxx', 2, True, True)]


@pytest.mark.parametrize('key,geo,pol,ens,rand,iso', CASES)
@pytest.mark.parametrize('precision,tol', TOLS)
def test_third_order_orientation_averages(golden, key, geo, pol, ens, rand, iso,
                                          precision, tol):
    """The engine evaluates the isotropic average from shared legs (3 t1 and
    3 t3 propagations, 9 t2 products) where the reference runs up to 21
    polarizations; random orientations become per-sample polarization
    vectors."""
    m = ori3_model(golden)
    _, S = qg.third_order_response(m, 40.0, population_times=[0.0, 20.0, 50.0],
                                   geometry=geo, polarization=pol, ensemble_size=ens,
                                   ensemble_random_orientations=rand,
                                   exact_isotropic_average=iso, precision=precision)
    assert rel_err(S, golden[key]) < tol


def test_third_order_isotropic_generic_path_matches_oracle(golden):
    """A secular model is not on the engine: the pathway loop runs each
    polarization of the invariants, as the reference does."""
    m = ori3_model(golden, secular=True)
    t2 = [0.0, 20.0]
    _, S = qg.third_order_response(m, 20.0, population_times=t2, geometry='-++',
                                   polarization='xxyy', exact_isotropic_average=True)
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    oham = orc.ElectronicHamiltonianSpec(golden['chain3_H'], dipoles=golden['ori3_dipoles'],
                                         energy_spread_extra=float(golden['chain3_extra']),
                                         bath=bath)
    om = orc.RedfieldSpec(oham, bath, 'gef', orc.CM_FS, secular=True)
    _, ref = orc.isotropic_average_4th(orc.third_order_response, 'xxyy', om, 20.0, t2,
                                       geometry='-++')
    assert rel_err(S, ref) < 1e-10
