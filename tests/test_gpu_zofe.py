"""ZOFE master equation (qspectra/dynamics/zofe.py) on the GPU through
qsx_zofe_rk4: the right-hand side against the oracle for several cluster
splits, and the drivers against the reference's own runs (RK4 harness)."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOLS = [('fp64', 1e-10), ('fp32', 1e-4)]


def zofe3(golden, subspace='ge'):
    on = np.ones(3, complex)
    pm = [np.array([x * on for x in golden['zofe3_' + k]]) for k in ('Omega', 'gamma', 'huang')]
    ham = qg.ElectronicHamiltonian(golden['zofe3_H'], bath=qg.PseudomodeBath(3, *pm),
                                   dipoles=golden['zofe3_dipoles'],
                                   disorder=wl.fwhm_for_sd(30.0), random_seed=9,
                                   energy_spread_extra=float(golden['zofe3_extra']))
    return qg.ZOFEModel(ham, hilbert_subspace=subspace, unit_convert=qg.CM_FS)


def oracle_zofe(n_sites, npm, subspace, seed):
    """Random pseudomode bath with couplings Omega^2 huang of 20..400 cm^-1."""
    rng = np.random.RandomState(seed)
    H1 = np.diag(12400 + 100 * rng.randn(n_sites)) + 40 * rng.randn(n_sites, n_sites)
    H1 = (H1 + H1.T) / 2
    ham = orc.ElectronicHamiltonianSpec(H1, dipoles=rng.randn(n_sites, 3))
    Om = rng.uniform(-500, 1500, (npm, 1)) * np.ones((1, n_sites))
    ga = rng.uniform(40, 300, (npm, 1)) * np.ones((1, n_sites))
    hu = rng.uniform(20, 400, (npm, 1)) / (Om ** 2 + 100) * np.ones((1, n_sites))
    return orc.ZOFESpec(ham, Om, ga, hu, subspace, orc.CM_FS)


def device_tables(om):
    L = -orc.occupations(om.ham.n_sites, om.hilbert_subspace)
    return (torch.as_tensor(L).cuda(), torch.as_tensor(om.Omega ** 2 * om.huang).cuda(),
            torch.as_tensor(1j * om.Omega + om.gamma).cuda(),
            torch.as_tensor(om.ham.H(om.hilbert_subspace)).cuda())


@pytest.mark.parametrize('n_sites,npm,subspace,clusters', [
    (3, 3, 'ge', (1, 2, 3)), (7, 16, 'ge', (0, 2, 4, 8)), (4, 5, 'gef', (0, 3, 5)),
    (7, 16, 'e', (0, 8))])
def test_rhs_matches_oracle(n_sites, npm, subspace, clusters):
    om = oracle_zofe(n_sites, npm, subspace, seed=n_sites + npm)
    rng = np.random.RandomState(1)
    M = om.n * om.n + int(np.prod(om.oop_shape))
    Y = rng.randn(3, M) + 1j * rng.randn(3, M)
    ref = np.array([om.rhs(y) for y in Y])
    Ld, G, w, H = device_tables(om)
    for c in clusters:
        for prec, tol in ((_native.QSX_FP64, 1e-13), (_native.QSX_FP32, 1e-5)):
            out = _native.zofe_rk4(H, Ld, G, w, torch.as_tensor(Y).cuda(), 0, 1.0, orc.CM_FS,
                                   precision=prec, mode=1, cluster=c)['rhs'].cpu().numpy()
            assert rel_err(out, ref) < tol, (c, prec)


@pytest.mark.parametrize('cluster', [0, 1, 4, 8])
def test_rk4_loop_matches_oracle_fmo_size(cluster):
    """16 pseudomodes on 7 sites ('ge', 7232 state elements) over 40 steps."""
    om = oracle_zofe(7, 16, 'ge', seed=3)
    rng = np.random.RandomState(2)
    rho0 = np.zeros((om.n, om.n), complex)
    rho0[1, 1] = 1.0
    y0 = om.join(rho0, 0.01 * (rng.randn(*om.oop_shape) + 1j * rng.randn(*om.oop_shape)))
    h = 2.0
    ref = orc.rk4_nonlinear(lambda _, y: om.rhs(y), y0, np.arange(0, 41 * h, 4 * h), h=h)
    Ld, G, w, H = device_tables(om)
    for prec, tol in ((_native.QSX_FP64, 1e-11), (_native.QSX_FP32, 1e-5)):
        st = _native.zofe_rk4(H, Ld, G, w, torch.as_tensor(y0).cuda(), 40, h, orc.CM_FS,
                              save_every=4, precision=prec, cluster=cluster)['state']
        assert rel_err(st[0].cpu().numpy(), ref) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_dynamics_matches_reference(golden, precision, tol):
    t, rho = qg.simulate_dynamics(zofe3(golden), [0, 1, 0, 0], 400.0, precision=precision)
    assert np.allclose(t, golden['zofe3_dyn_t'])
    assert rel_err(rho, golden['zofe3_dyn_rho']) < tol
    _, rho = qg.simulate_dynamics(zofe3(golden, 'e'), [1, 0, 0], 200.0, precision=precision)
    assert rel_err(rho, golden['zofe3e_dyn_rho']) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_linear_response_and_absorption_match_reference(golden, precision, tol):
    m = zofe3(golden)
    _, x = qg.linear_response(m, 'gg->eg->gg', 256.0, precision=precision)
    assert rel_err(x, golden['zofe3_lin']) < tol
    _, X = qg.absorption_spectra(m, 256.0, precision=precision)
    assert rel_err(X, golden['zofe3_abs_X']) < tol
    _, X = qg.absorption_spectra(m, 256.0, ensemble_size=3, ensemble_random_orientations=True,
                                 precision=precision)
    assert rel_err(X, golden['zofe3_abs_rand_X']) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_pump_matches_reference(golden, precision, tol):
    m = zofe3(golden)
    pump = qg.GaussianPulse(carrier_freq=float(np.mean(np.diag(golden['zofe3_H']))), fwhm=20.0,
                            t_peak=0.0, scale=1e-2, freq_convert=qg.CM_FS)
    t, st = qg.simulate_pump(m, pump, polarization='x', time_extra=60.0, precision=precision)
    assert np.allclose(t, golden['zofe3_pump_t'])
    assert rel_err(st, golden['zofe3_pump']) < tol


def test_third_order_matches_reference(golden):
    """No Heisenberg picture: the pathway loop integrates every t1 and t2
    state forward (response.py:297-336)."""
    on = np.ones(2, complex)
    pm = [np.array([x * on for x in golden['zofe3_' + k]]) for k in ('Omega', 'gamma', 'huang')]
    ham = qg.ElectronicHamiltonian(golden['zofe3_H'][:2, :2], bath=qg.PseudomodeBath(3, *pm),
                                   dipoles=golden['zofe3_dipoles'][:2],
                                   energy_spread_extra=float(golden['zofe3_extra']))
    m = qg.ZOFEModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS)
    dt = m.time_step
    assert abs(dt - float(golden['zofe2f_time_step'])) < 1e-12
    _, S = qg.third_order_response(m, 12 * dt, population_times=[0.0, 4 * dt],
                                   geometry='-++')
    assert rel_err(S, golden['zofe2f_3rd']) < 1e-10


def test_oversized_state_is_rejected():
    om = oracle_zofe(7, 16, 'gef', seed=1)
    Ld, G, w, H = device_tables(om)
    M = om.n * om.n + int(np.prod(om.oop_shape))
    with pytest.raises(_native.QsxError):
        _native.zofe_rk4(H, Ld, G, w, torch.zeros(M, dtype=torch.complex128).cuda(), 2, 1.0,
                         orc.CM_FS)


def zofe3_hermit(golden, rh, hh):
    m = zofe3(golden)
    m.rho_hermit, m.ham_hermit = bool(rh), bool(hh)
    return m


@pytest.mark.parametrize('rh,hh', [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_hermit_forms_rhs_match_reference(golden, golden_zofe_hermit, rh, hh):
    """rho_hermit / ham_hermit (zofe.py:179-192) at random non-Hermitian
    states, through the kernel's right-hand-side mode."""
    g = golden_zofe_hermit
    eom = zofe3_hermit(golden, rh, hh).equation_of_motion('gg,ge,eg,ee')
    got = eom(0.0, torch.as_tensor(g['zofeh_Y']).cuda()).cpu().numpy()
    assert rel_err(got, g['zofeh_rhs_{}{}'.format(rh, hh)]) < 1e-13


@pytest.mark.parametrize('precision,tol', TOLS)
def test_hermit_forms_drivers_match_reference(golden, golden_zofe_hermit, precision, tol):
    g = golden_zofe_hermit
    _, x = qg.linear_response(zofe3_hermit(golden, 1, 0), 'gg->eg->gg', 256.0,
                              precision=precision)
    assert rel_err(x, g['zofeh_lin_rho_only']) < tol
    m = zofe3_hermit(golden, 1, 1)
    _, x = qg.linear_response(m, 'gg->eg->gg', 256.0, precision=precision)
    assert rel_err(x, g['zofeh_lin']) < tol
    _, rho = qg.simulate_dynamics(m, [0, 1, 0, 0], 200.0, precision=precision)
    assert rel_err(rho, g['zofeh_dyn_rho']) < tol
    for rh, hh in ((0, 0), (1, 0), (1, 1)):
        _, rho = qg.simulate_dynamics(zofe3_hermit(golden, rh, hh), g['zofeh_rho0'], 200.0,
                                      precision=precision)
        assert rel_err(rho, g['zofeh_dyn_nh_{}{}'.format(rh, hh)]) < tol


@pytest.mark.parametrize('hermit', [1, 3])
def test_hermit_forms_under_fields_match_oracle(hermit):
    """Field terms a_p(t) [V_p, .] with the rho^H forms, from a non-Hermitian
    state: the field still acts on rho itself (eom.py:77-105 adds it beside
    the model's right-hand side)."""
    om = oracle_zofe(3, 4, 'ge', seed=5)
    om.rho_hermit, om.ham_hermit = True, hermit == 3
    rng = np.random.RandomState(3)
    n, M = om.n, om.n * om.n + int(np.prod(om.oop_shape))
    y0 = 0.1 * (rng.randn(M) + 1j * rng.randn(M))
    V = rng.randn(2, n, n) + 1j * rng.randn(2, n, n)
    nsteps, h = 12, 1.0
    coef = 1e-3 * (rng.randn(nsteps, 3, 2) + 1j * rng.randn(nsteps, 3, 2))

    def f(step, ci, y):
        d = om.rhs(y)
        for p in range(2):
            d = d + coef[step, ci, p] * om.commutator(V[p], y)
        return d
    y, ref = y0.copy(), [y0.copy()]
    for k in range(nsteps):
        k1 = f(k, 0, y)
        k2 = f(k, 1, y + h / 2 * k1)
        k3 = f(k, 1, y + h / 2 * k2)
        k4 = f(k, 2, y + h * k3)
        y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        ref.append(y.copy())
    Ld, G, w, H = device_tables(om)
    st = _native.zofe_rk4(H, Ld, G, w, torch.as_tensor(y0).cuda(), nsteps, h, orc.CM_FS,
                          V=torch.as_tensor(V).cuda(), coef=torch.as_tensor(coef).cuda(),
                          hermit=hermit)['state'][0].cpu().numpy()
    assert rel_err(st, np.array(ref)) < 1e-11
