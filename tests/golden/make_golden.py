"""Generate the golden fixtures in this folder by running the reference itself.

Run from the repository root in a container where the reference checkout is
available (read-only is fine), giving the checkout's path:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference-checkout> [base|drivers|zofe_hermit|all]

``base`` writes reference_golden.npz (generators, trajectories, spectra and
small third-order cases); ``drivers`` writes reference_golden_drivers.npz
(impulsive probe, 2D spectra, third order on the 128 x 3 x 128 grids at 6
and 8 sites, and the 8-site 495-node HEOM trajectory); ``zofe_hermit``
writes reference_golden_zofe_hermit.npz (ZOFE's rho_hermit / ham_hermit
forms).

Every fixture comes from the reference's own code path.  Its adaptive
``zvode`` integrator is swapped for a fixed-step RK4 harness that drives the
reference's own ``eom`` callables (the integrator the GPU path implements);
tight-tolerance ``zvode`` runs are stored beside them for the integrator gap.
The outputs are small ``.npz`` files committed next to this script; nothing
at test time reads the reference.
"""
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def rk4_harness(step):
    """Drop-in for qspectra.simulate.utils.integrate with a fixed-step RK4."""
    def integrate(f, y0, t, t0=None, method_name='zvode', f_params=None,
                  save_func=None, **kwargs):
        y0 = np.asarray(y0)
        if y0.ndim > 1:
            return np.array([integrate(f, yi, t, t0, method_name, f_params,
                                       save_func) for yi in y0])
        t = np.asarray(t, float)
        if t0 is None:
            t0 = t[0]
        save = (lambda x: x) if save_func is None else save_func
        y = np.array(y0, dtype=complex)
        out = []
        cur = t0
        h = step
        for ti in t:
            n = int(round((ti - cur) / h))
            for _ in range(n):
                k1 = f(cur, y)
                k2 = f(cur + h / 2, y + h / 2 * k1)
                k3 = f(cur + h / 2, y + h / 2 * k2)
                k4 = f(cur + h, y + h * k3)
                y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
                cur = cur + h
            out.append(save(y))
        return np.array(out)
    return integrate


def python3_shims():
    """The reference's decorators call inspect.getargspec, which Python 3.11
    removed; give it back as a view of getfullargspec (same fields, with
    ``keywords`` named ``varkw`` there) so the reference runs unmodified."""
    import inspect
    from collections import namedtuple
    if not hasattr(inspect, 'getargspec'):
        ArgSpec = namedtuple('ArgSpec', 'args varargs keywords defaults')

        def getargspec(func):
            spec = inspect.getfullargspec(func)
            return ArgSpec(spec.args, spec.varargs, spec.varkw, spec.defaults)
        inspect.getargspec = getargspec


def main(ref_root):
    python3_shims()
    sys.path.insert(0, ref_root)
    sys.path.insert(0, ROOT)
    warnings.simplefilter('ignore')
    import qspectra as qs
    import qspectra.simulate.response as qresp
    import qspectra.simulate.eom as qeom
    import qspectra.simulate.utils as qutils
    from qspectra.dynamics import heom as qheom
    from qspectra_gb300 import workloads as wl

    out = {}

    # ---- Debye correlation functions (bath.py:17-31, 84-102) -------------
    xs = np.concatenate([np.linspace(-900, 900, 37), [0.0, 1e-9, -3.5, 777.7]])
    for tag, (TK, lam, gam) in {'77K': (77, 35, 106), '300K': (300, 40, 100),
                                '10K': (10, 35, 106)}.items():
        b = qs.DebyeBath(qs.CM_K * TK, lam, gam)
        out['corr_x'] = xs
        out['corr_complex_' + tag] = np.array([b.corr_func_complex(x) for x in xs])
        out['corr_real_' + tag] = np.array([b.corr_func_real(x) for x in xs])

    # ---- Redfield Liouvillians on a dimer, every option ------------------
    dimer = np.array([[12881., 120], [120, 12719]])
    dip2 = [[1, 0, 0], [2 * np.cos(.3), 2 * np.sin(.3), 0]]
    bath77 = qs.DebyeBath(qs.CM_K * 77, 35, 106)
    ham = qs.ElectronicHamiltonian(dimer, bath=bath77, dipoles=dip2)
    for sec in (False, True):
        for dic in (False, True):
            for basis in ('site', 'eigen'):
                m = qs.RedfieldModel(ham, hilbert_subspace='gef',
                                     unit_convert=qs.CM_FS, secular=sec,
                                     discard_imag_corr=dic,
                                     evolve_basis=basis)
                key = 'dimer_L_sec{}_dic{}_{}'.format(int(sec), int(dic), basis)
                out[key] = m.evolution_super_operator
    out['dimer_H'] = dimer
    out['dimer_dipoles'] = np.array(dip2)

    # ---- 7-site workload: Liouvillian blocks, trajectories, spectra -------
    H7 = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H7, 1.0, qs.CM_FS)
    ham7 = qs.ElectronicHamiltonian(
        H7, bath=bath77, dipoles=[[1, 0, 0]] * 7,
        disorder=wl.fwhm_for_sd(80.0), random_seed=1, energy_spread_extra=extra)
    m7 = qs.RedfieldModel(ham7, hilbert_subspace='ge', unit_convert=qs.CM_FS,
                          secular=False)
    assert m7.time_step == 1.0, m7.time_step
    idx_ee = m7.liouville_subspace_index('ee')
    idx_eg = m7.liouville_subspace_index('eg')
    Lfull = m7.evolution_super_operator
    out['fmo7_H'] = H7
    out['fmo7_extra'] = extra
    out['fmo7_rw'] = m7.rw_freq
    out['fmo7_L_ee'] = Lfull[np.ix_(idx_ee, idx_ee)]
    out['fmo7_L_eg'] = Lfull[np.ix_(idx_eg, idx_eg)]
    out['fmo7_E'], out['fmo7_U'] = m7.hamiltonian.eig('ge')

    rk4 = rk4_harness(1.0)
    qeom.integrate = rk4
    qresp.integrate = rk4
    psi = np.zeros(7)
    psi[0] = 1.0
    t, rhos = qs.simulate_dynamics(m7, psi, duration=1000.0)
    out['fmo7_dyn_t'] = t
    out['fmo7_dyn_pops'] = np.einsum('tii->ti', rhos).real
    out['fmo7_dyn_rho_every10'] = rhos[::10]
    t, sig = qs.linear_response(m7, 'gg->eg->gg', 2048.0)
    out['fmo7_abs_t'] = t
    out['fmo7_abs_signal'] = sig
    f, X = qs.absorption_spectra(m7, 2048.0)
    out['fmo7_abs_f'] = f
    out['fmo7_abs_X'] = X

    # small ensemble: disorder draws and the averaged spectrum
    draws = np.array([np.diag(h.H_1exc) for h in ham7.sample_ensemble(8)])
    out['fmo7_sample_diag'] = draws
    f, X = qs.absorption_spectra(m7, 2048.0, ensemble_size=8)
    out['fmo7_ens8_abs_X'] = X
    t, rhos = qs.simulate_dynamics(m7, psi, duration=1000.0, ensemble_size=8)
    out['fmo7_ens8_pops'] = np.einsum('tii->ti', rhos).real

    # field-driven propagation (eom.py:77-227): a Gaussian pump, and two
    # different pulses with a 3-sample ensemble
    pump = qs.GaussianPulse(carrier_freq=12350.0, fwhm=20.0, t_peak=0.0, scale=1e-2,
                            freq_convert=qs.CM_FS)
    t, st = qs.simulate_pump(m7, pump, polarization='x', time_extra=60.0)
    out['fields_pump_t'] = t
    out['fields_pump_states'] = st
    p1 = qs.GaussianPulse(carrier_freq=12250.0, fwhm=15.0, t_peak=-10.0, scale=5e-3,
                          freq_convert=qs.CM_FS)
    p2 = qs.GaussianPulse(carrier_freq=12450.0, fwhm=25.0, t_peak=20.0, scale=8e-3,
                          freq_convert=qs.CM_FS)
    t, st = qs.simulate_with_fields(m7, [p1, p2], geometry='-+', polarization='xy',
                                    time_extra=40.0, ensemble_size=3)
    out['fields_two_t'] = t
    out['fields_two_states'] = st

    # orientation averages on a 4-site model with non-parallel dipoles:
    # random ensemble orientations (hamiltonian.py:552-575) and exact
    # isotropic averages (decorators.py:67-125)
    H4 = wl.chain_hamiltonian(n_sites=4, seed=11)
    extra4 = wl.energy_spread_for_dt(H4, 1.0, qs.CM_FS)
    dip4 = [[1.0, 0, 0], [0.3, 0.9, 0.1], [-0.5, 0.4, 0.7], [0.2, -0.6, 0.5]]
    ham4 = qs.ElectronicHamiltonian(H4, bath=bath77, dipoles=dip4,
                                    disorder=wl.fwhm_for_sd(40.0), random_seed=3,
                                    energy_spread_extra=extra4)
    m4 = qs.RedfieldModel(ham4, hilbert_subspace='ge', unit_convert=qs.CM_FS,
                          secular=False)
    assert m4.time_step == 1.0, m4.time_step
    out['ori4_H'] = H4
    out['ori4_extra'] = extra4
    out['ori4_dipoles'] = np.array(dip4)
    out['ori4_sample_dipoles'] = np.array(
        [h.dipoles for h in ham4.sample_ensemble(4, random_orientations=True)])
    f, X = qs.absorption_spectra(m4, 512.0, ensemble_size=4,
                                 ensemble_random_orientations=True)
    out['ori4_abs_f'] = f
    out['ori4_abs_rand'] = X
    f, X = qs.absorption_spectra(m4, 512.0, polarization=[0.3, 'x'],
                                 exact_isotropic_average=True)
    out['ori4_abs_iso'] = X
    f, X = qs.absorption_spectra(m4, 512.0, ensemble_size=3,
                                 ensemble_random_orientations=True,
                                 exact_isotropic_average=True)
    out['ori4_abs_iso_rand'] = X
    pump4 = qs.GaussianPulse(carrier_freq=float(np.mean(np.diag(H4))), fwhm=20.0,
                             t_peak=0.0, scale=1e-2, freq_convert=qs.CM_FS)
    t, st = qs.simulate_pump(m4, pump4, polarization=0.5, time_extra=30.0,
                             exact_isotropic_average=True)
    out['ori4_pump_iso_t'] = t
    out['ori4_pump_iso'] = st
    t, st = qs.simulate_with_fields(m4, [p1, p2], geometry='-+', polarization='xy',
                                    time_extra=30.0, ensemble_size=3,
                                    ensemble_random_orientations=True)
    out['ori4_fields_rand_t'] = t
    out['ori4_fields_rand'] = st

    # tight zvode for the integrator gap (reference as shipped)
    qeom.integrate = qutils.integrate
    qresp.integrate = qutils.integrate
    t, rhos = qs.simulate_dynamics(m7, psi, duration=1000.0, rtol=1e-12,
                                   atol=1e-14, nsteps=100000)
    out['fmo7_dyn_pops_zvode'] = np.einsum('tii->ti', rhos).real
    f, X = qs.absorption_spectra(m7, 2048.0, rtol=1e-12, atol=1e-14,
                                 nsteps=100000)
    out['fmo7_abs_X_zvode'] = X

    # ---- third-order response on a 3-site chain, 'gef' --------------------
    qeom.integrate = rk4_harness(2.0)
    qresp.integrate = rk4_harness(2.0)
    H3 = wl.chain_hamiltonian(n_sites=3, seed=7)
    bath300 = qs.DebyeBath(qs.CM_K * 300, 40, 100)
    extra3 = wl.energy_spread_for_dt(H3, 2.0, qs.CM_FS)
    ham3 = qs.ElectronicHamiltonian(H3, bath=bath300, dipoles=[[1, 0, 0]] * 3,
                                    energy_spread_extra=extra3)
    m3 = qs.RedfieldModel(ham3, hilbert_subspace='gef', unit_convert=qs.CM_FS,
                          secular=False)
    assert m3.time_step == 2.0
    out['chain3_H'] = H3
    out['chain3_extra'] = extra3
    for geo in ('-++', '+-+'):
        (t1, t2, t3), S = qs.third_order_response(
            m3, coherence_time_max=40.0, population_times=[0.0, 20.0, 50.0],
            geometry=geo)
        out['chain3_3rd_' + geo] = S
    out['chain3_t1'] = t1
    dip3 = [[1.0, 0, 0], [0.4, 0.8, 0.0], [-0.3, 0.5, 0.6]]
    ham3o = qs.ElectronicHamiltonian(H3, bath=bath300, dipoles=dip3,
                                     disorder=wl.fwhm_for_sd(30.0), random_seed=5,
                                     energy_spread_extra=extra3)
    m3o = qs.RedfieldModel(ham3o, hilbert_subspace='gef', unit_convert=qs.CM_FS,
                           secular=False)
    assert m3o.time_step == 2.0
    out['ori3_dipoles'] = np.array(dip3)
    t2s = [0.0, 20.0, 50.0]
    _, S = qs.third_order_response(m3o, coherence_time_max=40.0, population_times=t2s,
                                   geometry='-++', polarization=[0, 0, 0.5, 0.5],
                                   exact_isotropic_average=True)
    out['ori3_3rd_iso_-++'] = S
    _, S = qs.third_order_response(m3o, coherence_time_max=40.0, population_times=t2s,
                                   geometry='+-+', polarization='xxyy',
                                   exact_isotropic_average=True)
    out['ori3_3rd_isoxxyy_+-+'] = S
    _, S = qs.third_order_response(m3o, coherence_time_max=40.0, population_times=t2s,
                                   geometry='-++', polarization='xyxz', ensemble_size=3,
                                   ensemble_random_orientations=True)
    out['ori3_3rd_rand_-++'] = S
    _, S = qs.third_order_response(m3o, coherence_time_max=40.0, population_times=t2s,
                                   geometry='+-+', polarization='xxxx', ensemble_size=2,
                                   ensemble_random_orientations=True,
                                   exact_isotropic_average=True)
    out['ori3_3rd_iso_rand_+-+'] = S

    # ---- ZOFE master equation (dynamics/zofe.py) on a 3-site chain ---------
    Hz = wl.chain_hamiltonian(n_sites=3, seed=13)
    extraz = wl.energy_spread_for_dt(Hz, 2.0, qs.CM_FS)
    zpm = dict(Omega=[-200.0, 30.0, 250.0], gamma=[100.0, 50.0, 150.0],
               huang=[-5e-3, 0.8, 1e-2])
    on = np.ones(3, complex)
    pmb = qs.PseudomodeBath(3, np.array([x * on for x in zpm['Omega']]),
                            np.array([x * on for x in zpm['gamma']]),
                            np.array([x * on for x in zpm['huang']]))
    dipz = [[1.0, 0, 0], [0.4, 0.8, 0.0], [-0.3, 0.5, 0.6]]
    hamz = qs.ElectronicHamiltonian(Hz, bath=pmb, dipoles=dipz,
                                    disorder=wl.fwhm_for_sd(30.0), random_seed=9,
                                    energy_spread_extra=extraz)
    mz = qs.ZOFEModel(hamz, hilbert_subspace='ge', unit_convert=qs.CM_FS)
    assert mz.time_step == 2.0, mz.time_step
    out['zofe3_H'] = Hz
    out['zofe3_extra'] = extraz
    out['zofe3_dipoles'] = np.array(dipz)
    for k, v in zpm.items():
        out['zofe3_' + k] = np.array(v)
    qeom.integrate = rk4_harness(2.0)
    qresp.integrate = rk4_harness(2.0)
    t, rho = qs.simulate_dynamics(mz, [0, 1, 0, 0], 400.0)
    out['zofe3_dyn_t'] = t
    out['zofe3_dyn_rho'] = rho
    mze = qs.ZOFEModel(hamz, hilbert_subspace='e', unit_convert=qs.CM_FS)
    t, st = qs.simulate_dynamics(mze, [1, 0, 0], 200.0)
    out['zofe3e_dyn_rho'] = st
    t, x = qs.linear_response(mz, 'gg->eg->gg', 256.0)
    out['zofe3_lin'] = x
    f, X = qs.absorption_spectra(mz, 256.0)
    out['zofe3_abs_X'] = X
    f, X = qs.absorption_spectra(mz, 256.0, ensemble_size=3,
                                 ensemble_random_orientations=True)
    out['zofe3_abs_rand_X'] = X
    pumpz = qs.GaussianPulse(carrier_freq=float(np.mean(np.diag(Hz))), fwhm=20.0,
                             t_peak=0.0, scale=1e-2, freq_convert=qs.CM_FS)
    t, st = qs.simulate_pump(mz, pumpz, polarization='x', time_extra=60.0)
    out['zofe3_pump_t'] = t
    out['zofe3_pump'] = st
    mzf = qs.ZOFEModel(qs.ElectronicHamiltonian(Hz[:2, :2], bath=qs.PseudomodeBath(
        3, np.array([x * on[:2] for x in zpm['Omega']]),
        np.array([x * on[:2] for x in zpm['gamma']]),
        np.array([x * on[:2] for x in zpm['huang']])), dipoles=dipz[:2],
        energy_spread_extra=extraz), hilbert_subspace='gef', unit_convert=qs.CM_FS)
    out['zofe2f_time_step'] = np.array(mzf.time_step)
    qeom.integrate = rk4_harness(mzf.time_step)
    qresp.integrate = rk4_harness(mzf.time_step)
    _, S = qs.third_order_response(mzf, coherence_time_max=12 * mzf.time_step,
                                   population_times=[0.0, 4 * mzf.time_step],
                                   geometry='-++')
    out['zofe2f_3rd'] = S

    # ---- HEOM generators (heom.py:298-443) --------------------------------
    H2 = np.array([[12400., -100], [-100, 12480]])
    hamh = qs.ElectronicHamiltonian(H2, bath=qs.DebyeBath(qs.CM_K * 300, 35, 106),
                                    dipoles=[[1, 0, 0]] * 2)
    for tag, kw in {'K1lc3': dict(K=1, level_cutoff=3, low_temp_corr=True),
                    'K0lc4': dict(K=0, level_cutoff=4, low_temp_corr=True),
                    'K0lc3_nolt': dict(K=0, level_cutoff=3, low_temp_corr=False),
                    'K1lc3_mod': dict(K=1, level_cutoff=3, low_temp_corr=True,
                                      modified_HEOM=True)}.items():
        hm = qs.HEOMModel(hamh, hilbert_subspace='e', unit_convert=qs.CM_FS, **kw)
        L = hm.HEOM_tensor('ee').tocoo()
        out['heom2_{}_row'.format(tag)] = L.row
        out['heom2_{}_col'.format(tag)] = L.col
        out['heom2_{}_val'.format(tag)] = L.data
        out['heom2_{}_n'.format(tag)] = np.array(L.shape)
        out['heom2_{}_order'.format(tag)] = np.array(
            [a.reshape(-1) for a in hm.ado_indices])
    out['heom2_H'] = H2
    H3r = wl.ring_hamiltonian(n_sites=3, seed=5)
    hm = qs.HEOMModel(qs.ElectronicHamiltonian(
        H3r, bath=qs.DebyeBath(qs.CM_K * 300, 35, 106)),
        hilbert_subspace='e', unit_convert=qs.CM_FS, K=0, level_cutoff=3)
    L = hm.HEOM_tensor('ee').tocsr()
    out['heom3_H'] = H3r
    rho0 = np.zeros(9, complex)
    rho0[0] = 1
    y0 = np.zeros(L.shape[0], complex)
    y0[:9] = rho0
    eom = hm.equation_of_motion('ee')
    traj = rk4_harness(0.5)(eom, y0, np.arange(0, 100.0, 0.5))
    out['heom3_traj_node0'] = traj[:, :9]

    np.savez_compressed(os.path.join(HERE, 'reference_golden.npz'), **out)
    print('wrote', len(out), 'arrays')


def import_reference(ref_root):
    python3_shims()
    sys.path.insert(0, ref_root)
    sys.path.insert(0, ROOT)
    warnings.simplefilter('ignore')
    import qspectra as qs
    return qs


def second_order_state(n_sites, seed):
    """A Hermitian state on 'gg,ge,eg,ee' (column-stacked, the reference's
    state_vector layout): the ground state plus small seeded coherences and
    excited-state populations, as a pump would leave it."""
    rng = np.random.RandomState(seed)
    n = n_sites + 1
    rho = np.zeros((n, n), complex)
    rho[0, 0] = 0.9
    c = 0.05 * (rng.randn(n_sites) + 1j * rng.randn(n_sites))
    rho[1:, 0] = c
    rho[0, 1:] = c.conj()
    psi = rng.randn(n_sites) + 1j * rng.randn(n_sites)
    psi *= np.sqrt(0.1) / np.linalg.norm(psi)
    rho[1:, 1:] = np.outer(psi, psi.conj())
    return rho


def drivers_main(ref_root):
    """Fixtures for the pump-probe and 2D drivers and for the configuration-
    size third-order and HEOM checks."""
    qs = import_reference(ref_root)
    import qspectra.simulate.response as qresp
    import qspectra.simulate.eom as qeom
    from qspectra_gb300 import workloads as wl
    out = {}

    # ---- impulsive_probe (response.py:174-244) on a 3-site 'gef' chain -----
    rk4 = rk4_harness(2.0)
    qeom.integrate = rk4
    qresp.integrate = rk4
    H3 = wl.chain_hamiltonian(n_sites=3, seed=7)
    bath300 = qs.DebyeBath(qs.CM_K * 300, 40, 100)
    extra3 = wl.energy_spread_for_dt(H3, 2.0, qs.CM_FS)
    dip3 = [[1.0, 0, 0], [0.4, 0.8, 0.0], [-0.3, 0.5, 0.6]]
    ham3 = qs.ElectronicHamiltonian(H3, bath=bath300, dipoles=dip3,
                                    disorder=wl.fwhm_for_sd(30.0), random_seed=5,
                                    energy_spread_extra=extra3)
    m3 = qs.RedfieldModel(ham3, hilbert_subspace='gef', unit_convert=qs.CM_FS,
                          secular=False)
    assert m3.time_step == 2.0
    rho = second_order_state(3, seed=21)
    state = m3.density_matrix_to_state_vector(rho, 'gg,ge,eg,ee')
    out['probe3_H'] = H3
    out['probe3_extra'] = extra3
    out['probe3_dipoles'] = np.array(dip3)
    out['probe3_state'] = state
    for sig in ('GSB', 'ESE', 'ESA', 'GSB,ESE,ESA'):
        f, X = qs.impulsive_probe(m3, state, 200.0, polarization='xy',
                                  include_signal=sig)
        out['probe3_{}'.format(sig.replace(',', '_'))] = X
    out['probe3_f'] = f
    _, X = qs.impulsive_probe(m3, state, 200.0, polarization='xx', ensemble_size=3)
    out['probe3_ens3'] = X
    _, X = qs.impulsive_probe(m3, state, 200.0, polarization='xy', ensemble_size=3,
                              ensemble_random_orientations=True)
    out['probe3_ens3_rand'] = X
    _, X = qs.impulsive_probe(m3, state, 200.0, polarization=[0.4, 'x'],
                              exact_isotropic_average=True)
    out['probe3_iso'] = X

    # ---- two_dimensional_spectra (response.py:430-455) ---------------------
    for geo in ('-++', '+-+'):
        (f1, t2, f3), X = qs.two_dimensional_spectra(
            m3, coherence_time_max=40.0, population_times=[0.0, 20.0, 50.0], geometry=geo)
        out['twod3_{}'.format(geo)] = X
    out['twod3_f1'] = f1
    out['twod3_f3'] = f3
    (f1, t2, f3), X = qs.two_dimensional_spectra(
        m3, coherence_time_max=40.0, population_times=[0.0, 30.0], geometry='-++',
        polarization='xyxy', ensemble_size=2)
    out['twod3_ens2_xyxy'] = X

    # ---- third order on the 128 x 3 x 128 grids, chains of 6 and 8 sites ----
    for N in (6, 8):
        HN = wl.chain_hamiltonian(n_sites=N, seed=2024)
        extraN = wl.energy_spread_for_dt(HN, 2.0, qs.CM_FS)
        hamN = qs.ElectronicHamiltonian(HN, bath=bath300, dipoles=[[1, 0, 0]] * N,
                                        disorder=wl.fwhm_for_sd(60.0), random_seed=3,
                                        energy_spread_extra=extraN)
        mN = qs.RedfieldModel(hamN, hilbert_subspace='gef', unit_convert=qs.CM_FS,
                              secular=False)
        assert mN.time_step == 2.0
        out['chain{}_H'.format(N)] = HN
        out['chain{}_extra'.format(N)] = extraN
        for geo in ('-++', '+-+'):
            (t1, t2, t3), S = qs.third_order_response(
                mN, coherence_time_max=256.0, population_times=[0.0, 200.0, 500.0],
                geometry=geo, ensemble_size=2)
            out['chain{}_3rd_ens2_{}'.format(N, geo)] = S
        print('chain', N, 'done', flush=True)

    # ---- HEOM at the 8-site ring configuration: 495 nodes, 200 steps -------
    HR = wl.ring_hamiltonian()
    hamR = qs.ElectronicHamiltonian(HR, bath=qs.DebyeBath(qs.CM_K * 300, 35, 106),
                                    disorder=wl.fwhm_for_sd(50.0), random_seed=7)
    sample = 37
    hs = hamR.sample(sample)
    hm = qs.HEOMModel(hs, hilbert_subspace='e', unit_convert=qs.CM_FS, K=0,
                      level_cutoff=5, low_temp_corr=True)
    assert hm.ado_count == 495
    eom = hm.equation_of_motion('ee')
    y0 = np.zeros(495 * 64, complex)
    y0[0] = 1.0
    traj = rk4_harness(0.5)(eom, y0, np.arange(0, 100.5, 0.5))
    out['ring8_H'] = HR
    out['ring8_sample'] = np.array(sample)
    out['ring8_sample_H'] = hs.H_1exc
    out['ring8_traj_node0'] = traj[:, :64]
    out['ring8_final_state'] = traj[-1]

    # ---- HEOM options: a multi-block Liouville subspace, aki_temp_corr ------
    H2 = np.array([[12400., -100], [-100, 12480]])
    bathh = qs.DebyeBath(qs.CM_K * 300, 35, 106)
    hamh = qs.ElectronicHamiltonian(H2, bath=bathh, dipoles=[[1, 0, 0]] * 2)
    out['heomopt_H'] = H2
    hm = qs.HEOMModel(hamh, hilbert_subspace='ge', unit_convert=qs.CM_FS, K=1, level_cutoff=3)
    for tag, sub in (('multi', 'gg,ge,eg,ee'), ('multi2', 'ge,ee')):
        L = hm.HEOM_tensor(sub).tocoo()
        out['heomopt_{}_row'.format(tag)] = L.row
        out['heomopt_{}_col'.format(tag)] = L.col
        out['heomopt_{}_val'.format(tag)] = L.data
        out['heomopt_{}_n'.format(tag)] = np.array(L.shape)
    for tag, kw in (('aki', dict(low_temp_corr=True)), ('aki_nolt', dict(low_temp_corr=False))):
        hm = qs.HEOMModel(hamh, hilbert_subspace='e', unit_convert=qs.CM_FS, K=1,
                          level_cutoff=3, aki_temp_corr=True, **kw)
        L = hm.HEOM_tensor('ee').tocoo()
        out['heomopt_{}_row'.format(tag)] = L.row
        out['heomopt_{}_col'.format(tag)] = L.col
        out['heomopt_{}_val'.format(tag)] = L.data
        out['heomopt_{}_n'.format(tag)] = np.array(L.shape)
    np.savez_compressed(os.path.join(HERE, 'reference_golden_drivers.npz'), **out)
    print('wrote', len(out), 'arrays')


def zofe_hermit_main(ref_root):
    """Fixtures for ZOFEModel's rho_hermit / ham_hermit forms (zofe.py:179-192)
    on the 3-site chain of the base ZOFE fixtures: the right-hand side at
    random (non-Hermitian) states for every flag pair, and linear response and
    free dynamics with both flags set."""
    qs = import_reference(ref_root)
    import qspectra.simulate.response as qresp
    import qspectra.simulate.eom as qeom
    from qspectra_gb300 import workloads as wl
    out = {}
    Hz = wl.chain_hamiltonian(n_sites=3, seed=13)
    extraz = wl.energy_spread_for_dt(Hz, 2.0, qs.CM_FS)
    zpm = dict(Omega=[-200.0, 30.0, 250.0], gamma=[100.0, 50.0, 150.0],
               huang=[-5e-3, 0.8, 1e-2])
    on = np.ones(3, complex)
    pmb = qs.PseudomodeBath(3, np.array([x * on for x in zpm['Omega']]),
                            np.array([x * on for x in zpm['gamma']]),
                            np.array([x * on for x in zpm['huang']]))
    dipz = [[1.0, 0, 0], [0.4, 0.8, 0.0], [-0.3, 0.5, 0.6]]
    hamz = qs.ElectronicHamiltonian(Hz, bath=pmb, dipoles=dipz,
                                    disorder=wl.fwhm_for_sd(30.0), random_seed=9,
                                    energy_spread_extra=extraz)
    rng = np.random.RandomState(77)
    Y = None
    for rh, hh in ((False, False), (False, True), (True, False), (True, True)):
        m = qs.ZOFEModel(hamz, hilbert_subspace='ge', unit_convert=qs.CM_FS,
                         rho_hermit=rh, ham_hermit=hh)
        eom = m.equation_of_motion('gg,ge,eg,ee')
        if Y is None:
            M = 16 + int(np.prod(m.oop_shape))
            Y = rng.randn(3, M) + 1j * rng.randn(3, M)
            out['zofeh_Y'] = Y
        out['zofeh_rhs_{}{}'.format(int(rh), int(hh))] = np.array([eom(0.0, y) for y in Y])
    m = qs.ZOFEModel(hamz, hilbert_subspace='ge', unit_convert=qs.CM_FS, rho_hermit=True,
                     ham_hermit=True)
    assert m.time_step == 2.0, m.time_step
    qeom.integrate = rk4_harness(2.0)
    qresp.integrate = rk4_harness(2.0)
    _, x = qs.linear_response(m, 'gg->eg->gg', 256.0)
    out['zofeh_lin'] = x
    _, rho = qs.simulate_dynamics(m, [0, 1, 0, 0], 200.0)
    out['zofeh_dyn_rho'] = rho
    m = qs.ZOFEModel(hamz, hilbert_subspace='ge', unit_convert=qs.CM_FS, rho_hermit=True)
    _, x = qs.linear_response(m, 'gg->eg->gg', 256.0)
    out['zofeh_lin_rho_only'] = x
    # a non-Hermitian start inside the one-exciton block, where the forms differ
    rho0 = np.zeros((4, 4), complex)
    rho0[1, 1], rho0[2, 2], rho0[1, 2], rho0[2, 3] = 0.6, 0.4, 0.3 + 0.1j, -0.2j
    out['zofeh_rho0'] = rho0
    for rh, hh in ((False, False), (True, False), (True, True)):
        m = qs.ZOFEModel(hamz, hilbert_subspace='ge', unit_convert=qs.CM_FS,
                         rho_hermit=rh, ham_hermit=hh)
        _, rho = qs.simulate_dynamics(m, rho0, 200.0)
        out['zofeh_dyn_nh_{}{}'.format(int(rh), int(hh))] = rho
    np.savez_compressed(os.path.join(HERE, 'reference_golden_zofe_hermit.npz'), **out)
    print('wrote', len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) < 2:
        sys.exit('usage: make_golden.py <reference-checkout> [base|drivers|zofe_hermit|all]')
    what = sys.argv[2] if len(sys.argv) > 2 else 'all'
    if what in ('base', 'all'):
        main(sys.argv[1])
    if what in ('drivers', 'all'):
        drivers_main(sys.argv[1])
    if what in ('zofe_hermit', 'all'):
        zofe_hermit_main(sys.argv[1])
