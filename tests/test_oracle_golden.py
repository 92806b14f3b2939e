"""Pin the CPU oracle against fixtures produced by running the reference itself."""
import numpy as np
import pytest

import oracle as orc
from conftest import rel_err
from qspectra_gb300 import workloads as wl

CM_FS = orc.CM_FS


def fmo7_model(golden, sample=None):
    bath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    ham = orc.ElectronicHamiltonianSpec(
        golden['fmo7_H'], dipoles=[[1, 0, 0]] * 7, disorder=wl.fwhm_for_sd(80.0),
        random_seed=1, energy_spread_extra=float(golden['fmo7_extra']), bath=bath)
    m = orc.RedfieldSpec(ham, bath, 'ge', CM_FS, secular=False)
    return m if sample is None else m.sample(sample)


def test_constants_match_reference_values():
    assert orc.CM_FS == np.pi * 2 * 2.99792458e-5
    assert orc.CM_K == 0.69503476


@pytest.mark.parametrize('tag,TK,lam,gam', [('77K', 77, 35, 106),
                                            ('300K', 300, 40, 100),
                                            ('10K', 10, 35, 106)])
def test_debye_corr(golden, tag, TK, lam, gam):
    b = orc.DebyeBathSpec(orc.CM_K * TK, lam, gam)
    xs = golden['corr_x']
    c = np.array([b.corr_complex(x) for x in xs])
    r = np.array([b.corr_real(x) for x in xs])
    assert rel_err(c, golden['corr_complex_' + tag]) < 1e-14
    assert rel_err(r, golden['corr_real_' + tag]) < 1e-14


@pytest.mark.parametrize('sec', [0, 1])
@pytest.mark.parametrize('dic', [0, 1])
@pytest.mark.parametrize('basis', ['site', 'eigen'])
def test_redfield_dimer_all_options(golden, sec, dic, basis):
    bath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    ham = orc.ElectronicHamiltonianSpec(golden['dimer_H'],
                                        dipoles=golden['dimer_dipoles'])
    m = orc.RedfieldSpec(ham, bath, 'gef', CM_FS, secular=bool(sec),
                         discard_imag_corr=bool(dic), evolve_basis=basis)
    L = m.evolution_super_operator()
    ref = golden['dimer_L_sec{}_dic{}_{}'.format(sec, dic, basis)]
    if basis == 'eigen':
        # eigenvector signs are arbitrary; compare sign-invariant magnitudes
        assert rel_err(np.abs(L), np.abs(ref)) < 1e-12
    else:
        assert rel_err(L, ref) < 1e-12


def test_fmo7_blocks_and_time_step(golden):
    m = fmo7_model(golden)
    assert m.time_step == 1.0
    assert m.ham.rw_freq == pytest.approx(float(golden['fmo7_rw']), rel=1e-15)
    assert rel_err(m.eom_matrix('ee'), golden['fmo7_L_ee']) < 1e-12
    assert rel_err(m.eom_matrix('eg'), golden['fmo7_L_eg']) < 1e-12


def test_fmo7_rk4_dynamics_and_absorption(golden):
    m = fmo7_model(golden)
    psi = np.zeros(7)
    psi[0] = 1
    t, rhos = orc.simulate_dynamics(m, psi, 1000.0)
    pops = np.einsum('tii->ti', rhos).real
    assert rel_err(pops, golden['fmo7_dyn_pops']) < 1e-12
    assert rel_err(rhos[::10], golden['fmo7_dyn_rho_every10']) < 1e-12
    t, sig = orc.linear_response(m, 2048.0)
    assert rel_err(sig, golden['fmo7_abs_signal']) < 1e-12
    f, X = orc.absorption_spectra(m, 2048.0)
    assert rel_err(f, golden['fmo7_abs_f']) < 1e-14
    assert rel_err(X, golden['fmo7_abs_X']) < 1e-12
    # integrator gap to the reference's own tight zvode run (RK4 at 1 fs)
    assert rel_err(pops, golden['fmo7_dyn_pops_zvode']) < 1e-5
    assert rel_err(X, golden['fmo7_abs_X_zvode']) < 1e-5


def test_fmo7_disorder_and_small_ensemble(golden):
    m = fmo7_model(golden)
    draws = np.array([np.diag(m.sample(n).ham.H1) for n in range(8)])
    np.testing.assert_array_equal(draws, golden['fmo7_sample_diag'])
    _, X = orc.ensemble_average(m, 8, orc.absorption_spectra, 2048.0)
    assert rel_err(X, golden['fmo7_ens8_abs_X']) < 1e-12
    psi = np.zeros(7)
    psi[0] = 1
    _, rhos = orc.ensemble_average(m, 8, orc.simulate_dynamics, psi, 1000.0)
    pops = np.einsum('tii->ti', rhos).real
    assert rel_err(pops, golden['fmo7_ens8_pops']) < 1e-12


@pytest.mark.parametrize('geo', ['-++', '+-+'])
def test_third_order_chain3(golden, geo):
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    ham = orc.ElectronicHamiltonianSpec(
        golden['chain3_H'], dipoles=[[1, 0, 0]] * 3,
        energy_spread_extra=float(golden['chain3_extra']), bath=bath)
    m = orc.RedfieldSpec(ham, bath, 'gef', CM_FS, secular=False)
    assert m.time_step == 2.0
    _, S = orc.third_order_response(m, 40.0, [0.0, 20.0, 50.0], geometry=geo)
    assert rel_err(S, golden['chain3_3rd_' + geo]) < 1e-11


@pytest.mark.parametrize('tag,kw', [
    ('K1lc3', dict(K=1, level_cutoff=3, low_temp_corr=True)),
    ('K0lc4', dict(K=0, level_cutoff=4, low_temp_corr=True)),
    ('K0lc3_nolt', dict(K=0, level_cutoff=3, low_temp_corr=False)),
    ('K1lc3_mod', dict(K=1, level_cutoff=3, low_temp_corr=True,
                       modified_HEOM=True))])
def test_heom_generator(golden, tag, kw):
    import scipy.sparse as sps
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 35, 106)
    ham = orc.ElectronicHamiltonianSpec(golden['heom2_H'])
    hm = orc.HEOMSpec(ham, bath, 'e', 1.0, **kw)
    order = np.array([a.reshape(-1) for a in hm.ados])
    np.testing.assert_array_equal(order, golden['heom2_{}_order'.format(tag)])
    L = hm.heom_tensor('ee').toarray()
    n = tuple(golden['heom2_{}_n'.format(tag)])
    ref = sps.coo_matrix((golden['heom2_{}_val'.format(tag)],
                          (golden['heom2_{}_row'.format(tag)],
                           golden['heom2_{}_col'.format(tag)])), shape=n).toarray()
    assert rel_err(L, ref) < 1e-13


def test_heom_trajectory(golden):
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 35, 106)
    ham = orc.ElectronicHamiltonianSpec(golden['heom3_H'])
    hm = orc.HEOMSpec(ham, bath, 'e', CM_FS, K=0, level_cutoff=3)
    L = hm.eom_matrix('ee')
    y0 = np.zeros(L.shape[0], complex)
    y0[0] = 1
    traj = orc.rk4_integrate_sparse(L, y0, 199, 0.5)
    assert rel_err(traj[:, :9], golden['heom3_traj_node0']) < 1e-12


def test_fields_oracle_matches_reference(golden):
    """Field-driven propagation (eom.py:77-227) against the reference's own
    simulate_pump / simulate_with_fields driven by the RK4 harness."""
    H7 = golden['fmo7_H']
    bath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H7, dipoles=[[1, 0, 0]] * 7,
                                         disorder=wl.fwhm_for_sd(80.0), random_seed=1,
                                         energy_spread_extra=float(golden['fmo7_extra']),
                                         bath=bath)
    om = orc.RedfieldSpec(oham, bath, 'ge', orc.CM_FS, secular=False)
    pump = orc.GaussianPulseSpec(12350.0, 20.0, 0.0, 1e-2, orc.CM_FS)
    t, st = orc.simulate_with_fields(om, [pump, pump], '-+', 'xx', 60.0)
    assert np.allclose(t, golden['fields_pump_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['fields_pump_states']) < 1e-12
    p1 = orc.GaussianPulseSpec(12250.0, 15.0, -10.0, 5e-3, orc.CM_FS)
    p2 = orc.GaussianPulseSpec(12450.0, 25.0, 20.0, 8e-3, orc.CM_FS)
    ticks, st = orc.ensemble_average(om, 3, orc.simulate_with_fields, [p1, p2], '-+', 'xy',
                                     40.0)
    assert rel_err(st, golden['fields_two_states']) < 1e-12


def ori4_model(golden):
    bath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    ham = orc.ElectronicHamiltonianSpec(golden['ori4_H'], dipoles=golden['ori4_dipoles'],
                                        disorder=wl.fwhm_for_sd(40.0), random_seed=3,
                                        energy_spread_extra=float(golden['ori4_extra']),
                                        bath=bath)
    return orc.RedfieldSpec(ham, bath, 'ge', CM_FS, secular=False)


def test_random_orientation_draws(golden):
    """Sample n's dipoles are R_n d_i with R_n drawn after the disorder
    (hamiltonian.py:552-575, polarization.py:87-102)."""
    m = ori4_model(golden)
    dips = np.array([m.sample(n, True).ham.dipoles for n in range(4)])
    assert np.abs(dips - golden['ori4_sample_dipoles']).max() < 1e-14


def test_orientation_averaged_absorption(golden):
    """Random ensemble orientations and the exact second-order isotropic
    average of the absorption spectrum (decorators.py:40-64, 95-125)."""
    m = ori4_model(golden)

    def spectrum(x):
        t = orc.time_grid(512.0, m.time_step)
        return orc.fourier_transform(t, -x, rw_freq=m.ham.rw_freq,
                                     unit_convert=m.unit_convert)[1].real

    _, x = orc.ensemble_average(m, 4, orc.linear_response, 512.0, random_orientations=True)
    assert rel_err(spectrum(x), golden['ori4_abs_rand']) < 1e-11
    _, x = orc.isotropic_average_2nd(orc.linear_response, [0.3, 'x'], m, 512.0)
    assert rel_err(spectrum(x), golden['ori4_abs_iso']) < 1e-11

    def iso(model, time_max):
        return orc.isotropic_average_2nd(orc.linear_response, 'xx', model, time_max)
    _, x = orc.ensemble_average(m, 3, iso, 512.0, random_orientations=True)
    assert rel_err(spectrum(x), golden['ori4_abs_iso_rand']) < 1e-11


def test_orientation_averaged_fields(golden):
    m = ori4_model(golden)
    pump = orc.GaussianPulseSpec(float(np.mean(np.diag(golden['ori4_H']))), 20.0, 0.0,
                                 1e-2, orc.CM_FS)

    def pumped(model, polarization):
        return orc.simulate_with_fields(model, [pump, pump], '-+', polarization, 30.0)
    t, st = orc.isotropic_average_2nd(pumped, [0.5, 0.5], m)
    assert np.allclose(t, golden['ori4_pump_iso_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['ori4_pump_iso']) < 1e-12
    p1 = orc.GaussianPulseSpec(12250.0, 15.0, -10.0, 5e-3, orc.CM_FS)
    p2 = orc.GaussianPulseSpec(12450.0, 25.0, 20.0, 8e-3, orc.CM_FS)
    t, st = orc.ensemble_average(m, 3, orc.simulate_with_fields, [p1, p2], '-+', 'xy',
                                 30.0, random_orientations=True)
    assert np.allclose(t, golden['ori4_fields_rand_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['ori4_fields_rand']) < 1e-12


def ori3_model(golden):
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    ham = orc.ElectronicHamiltonianSpec(golden['chain3_H'], dipoles=golden['ori3_dipoles'],
                                        disorder=wl.fwhm_for_sd(30.0), random_seed=5,
                                        energy_spread_extra=float(golden['chain3_extra']),
                                        bath=bath)
    return orc.RedfieldSpec(ham, bath, 'gef', CM_FS, secular=False)


@pytest.mark.parametrize('key,geo,pol,ens,rand,iso', [
    ('ori3_3rd_iso_-++', '-++', [0, 0, 0.5, 0.5], None, False, True),
    ('ori3_3rd_isoxxyy_+-+', '+-+', 'xxyy', None, False, True),
    ('ori3_3rd_rand_-++', '-++', 'xyxz', 3, True, False),
    ('ori3_3rd_iso_rand_+-+', '+-+', 'xxxx', 2, True, True)])
def test_orientation_averaged_third_order(golden, key, geo, pol, ens, rand, iso):
    """Fourth-order isotropic average (decorators.py:67-92, invariants with
    weight <= 1e-8 dropped as there) and random ensemble orientations."""
    m = ori3_model(golden)
    t2 = [0.0, 20.0, 50.0]

    def one(model, polarization):
        if iso:
            return orc.isotropic_average_4th(orc.third_order_response, polarization, model,
                                             40.0, t2, geometry=geo)
        return orc.third_order_response(model, 40.0, t2, geometry=geo,
                                        polarization=polarization)
    if ens is None:
        _, S = one(m, pol)
    else:
        _, S = orc.ensemble_average(m, ens, one, pol, random_orientations=rand)
    assert rel_err(S, golden[key]) < 1e-11


def zofe3_model(golden, subspace='ge', sites=3):
    ham = orc.ElectronicHamiltonianSpec(golden['zofe3_H'][:sites, :sites],
                                        dipoles=golden['zofe3_dipoles'][:sites],
                                        disorder=wl.fwhm_for_sd(30.0) if sites == 3 else None,
                                        random_seed=9,
                                        energy_spread_extra=float(golden['zofe3_extra']))
    pm = [np.outer(golden['zofe3_' + k], np.ones(sites)) for k in ('Omega', 'gamma', 'huang')]
    return orc.ZOFESpec(ham, *pm, hilbert_subspace=subspace, unit_convert=CM_FS)


def test_zofe_oracle_matches_reference(golden):
    """ZOFE master equation (zofe.py:121-229): free dynamics on 'ge' and 'e',
    linear response, absorption with random orientations, a pump pulse."""
    m = zofe3_model(golden)
    assert m.time_step == 2.0
    t, rho = orc.zofe_dynamics(m, [0, 1, 0, 0], 400.0)
    assert np.allclose(t, golden['zofe3_dyn_t'])
    assert rel_err(rho, golden['zofe3_dyn_rho']) < 1e-12
    _, rho = orc.zofe_dynamics(zofe3_model(golden, 'e'), [1, 0, 0], 200.0)
    assert rel_err(rho, golden['zofe3e_dyn_rho']) < 1e-12
    t, x = orc.zofe_linear_response(m, 256.0)
    assert rel_err(x, golden['zofe3_lin']) < 1e-12

    def spectrum(x):
        return orc.fourier_transform(t, -x, rw_freq=m.ham.rw_freq,
                                     unit_convert=CM_FS)[1].real
    assert rel_err(spectrum(x), golden['zofe3_abs_X']) < 1e-12
    _, x = orc.ensemble_average(m, 3, orc.zofe_linear_response, 256.0,
                                random_orientations=True)
    assert rel_err(spectrum(x), golden['zofe3_abs_rand_X']) < 1e-12
    pump = orc.GaussianPulseSpec(float(np.mean(np.diag(golden['zofe3_H']))), 20.0, 0.0,
                                 1e-2, CM_FS)
    t, st = orc.zofe_with_fields(m, [pump, pump], '-+', 'xx', 60.0)
    assert np.allclose(t, golden['zofe3_pump_t'])
    assert rel_err(st, golden['zofe3_pump']) < 1e-12


@pytest.mark.parametrize('rh,hh', [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_zofe_hermit_forms_oracle_matches_reference(golden, golden_zofe_hermit, rh, hh):
    """ZOFEModel's rho_hermit / ham_hermit forms (zofe.py:179-192): the
    right-hand side at random non-Hermitian states."""
    m = zofe3_model(golden)
    m.rho_hermit, m.ham_hermit = bool(rh), bool(hh)
    got = np.array([m.rhs(y) for y in golden_zofe_hermit['zofeh_Y']])
    assert rel_err(got, golden_zofe_hermit['zofeh_rhs_{}{}'.format(rh, hh)]) < 1e-13


def test_zofe_hermit_drivers_oracle_matches_reference(golden, golden_zofe_hermit):
    g = golden_zofe_hermit
    m = zofe3_model(golden)
    m.rho_hermit = True
    _, x = orc.zofe_linear_response(m, 256.0)
    assert rel_err(x, g['zofeh_lin_rho_only']) < 1e-12
    m.ham_hermit = True
    _, x = orc.zofe_linear_response(m, 256.0)
    assert rel_err(x, g['zofeh_lin']) < 1e-12
    _, rho = orc.zofe_dynamics(m, [0, 1, 0, 0], 200.0)
    assert rel_err(rho, g['zofeh_dyn_rho']) < 1e-12
    # linear response and a Hermitian start cannot tell the forms apart (the
    # auxiliary operators stay inside the one-exciton block); a non-Hermitian
    # start inside that block does
    for rh, hh in ((0, 0), (1, 0), (1, 1)):
        m.rho_hermit, m.ham_hermit = bool(rh), bool(hh)
        _, rho = orc.zofe_dynamics(m, g['zofeh_rho0'], 200.0)
        assert rel_err(rho, g['zofeh_dyn_nh_{}{}'.format(rh, hh)]) < 1e-12
    assert rel_err(g['zofeh_dyn_nh_10'], g['zofeh_dyn_nh_00']) > 1e-3
    assert rel_err(g['zofeh_dyn_nh_11'], g['zofeh_dyn_nh_10']) > 1e-3
