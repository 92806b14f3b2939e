"""GPU parity of the Redfield path against the oracle and the reference fixtures."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # plain FP64 form vs the oracle (spec bar)
FP32_TOL = 1e-4    # split-word FP32 form vs the FP64 oracle


def fmo7_pair(golden):
    """(qspectra_gb300 model, oracle model) for the 7-site workload."""
    H7 = golden['fmo7_H']
    extra = float(golden['fmo7_extra'])
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    ham = qg.ElectronicHamiltonian(H7, bath=bath, dipoles=[[1, 0, 0]] * 7,
                                   disorder=wl.fwhm_for_sd(80.0), random_seed=1,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS,
                         secular=False)
    obath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H7, dipoles=[[1, 0, 0]] * 7,
                                         disorder=wl.fwhm_for_sd(80.0), random_seed=1,
                                         energy_spread_extra=extra, bath=obath)
    om = orc.RedfieldSpec(oham, obath, 'ge', orc.CM_FS, secular=False)
    return m, om


@pytest.mark.parametrize('tag,TK,lam,gam', [('77K', 77, 35, 106), ('300K', 300, 40, 100),
                                            ('10K', 10, 35, 106)])
def test_debye_corr_kernel(golden, tag, TK, lam, gam):
    b = qg.DebyeBath(qg.CM_K * TK, lam, gam)
    xs = golden['corr_x']
    assert rel_err(b.corr_func_complex(xs), golden['corr_complex_' + tag]) < 1e-13
    assert rel_err(b.corr_func_real(xs), golden['corr_real_' + tag]) < 1e-13


def test_eigh_jacobi_blocks():
    rng = np.random.RandomState(3)
    B, n = 9, 29
    A = rng.randn(B, n, n)
    A = A + A.transpose(0, 2, 1)
    bounds = [0, 1, 8, 29]
    mask = np.zeros((n, n))
    for a, b in zip(bounds[:-1], bounds[1:]):
        mask[a:b, a:b] = 1
    A = A * mask
    E, U = _native.eigh(torch.as_tensor(A).cuda(), bounds)
    E, U = E.cpu().numpy(), U.cpu().numpy()
    for k in range(B):
        for a, b in zip(bounds[:-1], bounds[1:]):
            ref = np.linalg.eigvalsh(A[k, a:b, a:b])
            assert np.max(np.abs(E[k, a:b] - ref)) < 1e-12 * max(1, np.abs(ref).max())
        assert np.max(np.abs(U[k].T @ U[k] - np.eye(n))) < 1e-13
        assert np.max(np.abs(U[k] @ np.diag(E[k]) @ U[k].T - A[k])) < 1e-12 * np.abs(A[k]).max()
        assert np.all(U[k] * (1 - mask) == 0)  # block structure is exact


@pytest.mark.parametrize('sec', [0, 1])
@pytest.mark.parametrize('dic', [0, 1])
@pytest.mark.parametrize('basis', ['site', 'eigen'])
def test_redfield_liouvillian_dimer_all_options(golden, sec, dic, basis):
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    ham = qg.ElectronicHamiltonian(golden['dimer_H'], bath=bath,
                                   dipoles=golden['dimer_dipoles'])
    m = qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS,
                         secular=bool(sec), discard_imag_corr=bool(dic),
                         evolve_basis=basis)
    L = m.evolution_super_operator
    ref = golden['dimer_L_sec{}_dic{}_{}'.format(sec, dic, basis)]
    if basis == 'eigen':
        assert rel_err(np.abs(L), np.abs(ref)) < 1e-12
    else:
        assert rel_err(L, ref) < 1e-12


def test_fmo7_blocks(golden):
    m, _ = fmo7_pair(golden)
    assert m.time_step == 1.0
    Lee = m.equation_of_motion('ee').matrix.cpu().numpy()
    Leg = m.equation_of_motion('eg').matrix.cpu().numpy()
    LegH = m.equation_of_motion('eg', heisenberg_picture=True).matrix.cpu().numpy()
    assert rel_err(Lee, golden['fmo7_L_ee']) < 1e-12
    assert rel_err(Leg, golden['fmo7_L_eg']) < 1e-12
    assert rel_err(LegH, golden['fmo7_L_eg'].T) < 1e-12


def test_fmo7_dynamics_fp64_and_fp32(golden):
    m, om = fmo7_pair(golden)
    psi = np.zeros(7)
    psi[0] = 1
    t, rhos = qg.simulate_dynamics(m, psi, duration=1000.0)
    _, orhos = orc.simulate_dynamics(om, psi, 1000.0)
    assert rel_err(rhos, orhos) < FP64_TOL
    pops = np.einsum('tii->ti', rhos).real
    assert rel_err(pops, golden['fmo7_dyn_pops']) < FP64_TOL
    _, r32 = qg.simulate_dynamics(m, psi, duration=1000.0, precision='fp32')
    assert rel_err(r32, orhos) < FP32_TOL


def test_fmo7_absorption_fp64_and_fp32(golden):
    m, om = fmo7_pair(golden)
    t, sig = qg.linear_response(m, 'gg->eg->gg', 2048.0)
    assert rel_err(sig, golden['fmo7_abs_signal']) < FP64_TOL
    f, X = qg.absorption_spectra(m, 2048.0)
    assert rel_err(f, golden['fmo7_abs_f']) < 1e-14
    assert rel_err(X, golden['fmo7_abs_X']) < FP64_TOL
    f, X32 = qg.absorption_spectra(m, 2048.0, precision='fp32')
    assert rel_err(X32, golden['fmo7_abs_X']) < FP32_TOL


def test_fmo7_small_ensemble_fp64(golden):
    m, _ = fmo7_pair(golden)
    f, X = qg.absorption_spectra(m, 2048.0, ensemble_size=8, precision='fp64')
    assert rel_err(X, golden['fmo7_ens8_abs_X']) < FP64_TOL
    psi = np.zeros(7)
    psi[0] = 1
    t, rhos = qg.simulate_dynamics(m, psi, duration=1000.0, ensemble_size=8,
                                   precision='fp64')
    pops = np.einsum('tii->ti', rhos).real
    assert rel_err(pops, golden['fmo7_ens8_pops']) < FP64_TOL
    t, r32 = qg.simulate_dynamics(m, psi, duration=1000.0, ensemble_size=8,
                                  precision='fp32')
    assert rel_err(np.einsum('tii->ti', r32).real, golden['fmo7_ens8_pops']) < FP32_TOL


@pytest.mark.parametrize('geo', ['-++', '+-+'])
def test_third_order_chain3(golden, geo):
    bath = qg.DebyeBath(qg.CM_K * 300, 40, 100)
    ham = qg.ElectronicHamiltonian(golden['chain3_H'], bath=bath, dipoles=[[1, 0, 0]] * 3,
                                   energy_spread_extra=float(golden['chain3_extra']))
    m = qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS, secular=False)
    assert m.time_step == 2.0
    _, S = qg.third_order_response(m, 40.0, population_times=[0.0, 20.0, 50.0], geometry=geo)
    assert rel_err(S, golden['chain3_3rd_' + geo]) < FP64_TOL


def test_fourier_transform_matches_oracle_fft():
    rng = np.random.RandomState(1)
    for t in [np.arange(0, 300.0, 1.0), np.linspace(-50, 120, 171), np.arange(0.5, 40.5, 1.0)]:
        x = rng.randn(len(t)) + 1j * rng.randn(len(t))
        for sign in (1, -1):
            f, X = qg.fourier_transform(t, x, rw_freq=3.0, unit_convert=0.7, sign=sign)
            of, oX = orc.fourier_transform(t, x, rw_freq=3.0, unit_convert=0.7, sign=sign)
            assert rel_err(f, of) < 1e-14
            assert rel_err(X, oX) < 1e-12


@pytest.mark.parametrize('nt', [1, 37, 2048, 4095])
def test_fp32_dft_matches_fp64_dft(nt):
    """qsx_dft_batched_f32 (FP32 rotation and sums between FP64 phase
    anchors) against the FP64 transform at the FP32 contract, on the
    workload's grid shape (1 fs steps, rotating-frame frequencies)."""
    rng = np.random.RandomState(nt)
    x = torch.as_tensor(rng.randn(2, nt) + 1j * rng.randn(2, nt)).cuda()
    f = torch.linspace(11800.0, 13000.0, 1024, dtype=torch.float64, device='cuda')
    args = (x, -0.5 * (nt - 1), 1.0, f, 12400.0, qg.CM_FS, 1)
    X64 = _native.dft(*args).cpu().numpy()
    X32 = _native.dft(*args, precision=_native.QSX_FP32).cpu().numpy()
    assert rel_err(X32, X64) < 2e-5


def test_fourier_transform_analytic():
    """Reference tests/test_simulate_utils.py:8-55 (analytic transforms)."""
    a = (1.0 + 0.3j) / 100
    fn = lambda x: (x > 0) * np.exp(-a * x)  # noqa: E731
    F = lambda v: 1.0 / (a - 1j * v)  # noqa: E731
    t = np.linspace(0, 1000, num=10000)
    v, X = qg.fourier_transform(t, fn(t))
    assert np.max(np.abs(X - F(v))) < 0.002 * abs(F(0))
    v, X = qg.fourier_transform(t, fn(t), sign=-1)
    assert np.max(np.abs(X - F(-v))) < 0.002 * abs(F(0))


def test_nonfinite_state_raises():
    L = torch.zeros((2, 3, 3), dtype=torch.complex128, device='cuda')
    L[1, 0, 0] = float('nan')
    y0 = torch.ones(3, dtype=torch.complex128, device='cuda')
    D = _native.rk4_propagator(L, 1.0, _native.QSX_FP64)
    with pytest.raises(_native.IntegratorError):
        _native.rk4(D, y0, 4, 1, state=True)


def test_invalid_arguments_raise():
    L = torch.zeros((1, 70, 70), dtype=torch.complex128, device='cuda')
    with pytest.raises(_native.QsxError, match='m <= 64'):
        _native.rk4_propagator(L, 1.0)
    with pytest.raises(ValueError):
        _native.rk4_propagator(L.cpu(), 1.0)
