"""Boundary cases through the C ABI: empty batches, zero steps, a single
disorder sample, and the no-work calls of the transforms and products."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision', [_native.QSX_FP64, _native.QSX_FP32])
def test_rk4_zero_steps_returns_the_initial_state(precision):
    rng = np.random.RandomState(1)
    m, B = 6, 3
    dt = torch.complex64 if precision == _native.QSX_FP32 else torch.complex128
    D = torch.as_tensor(0.01 * (rng.randn(B, m, m) + 1j * rng.randn(B, m, m))).to(dt).cuda()
    y0 = torch.as_tensor(rng.randn(B, m) + 1j * rng.randn(B, m)).cuda()
    out = _native.rk4(D, y0, 0, 1, state=True, precision=precision)['state']
    assert out.shape == (B, 1, m)
    assert rel_err(out[:, 0].cpu().numpy(), y0.cpu().numpy()) < 1e-7


def test_empty_batches_do_no_work():
    """batch = 0 returns at once from the entry points (no launch, no error)."""
    lib = _native.load()
    stream = _native._stream()
    assert lib.qsx_dft_batched(None, 16, 0, 0.0, 1.0, None, 8, 0.0, 1.0, 1, None, stream) == 0
    assert lib.qsx_dft2_batched(None, 8, 0, 8, 8, 8, 1, 0.0, 1.0, None, 4, -1, 0.0, 1.0,
                                None, 4, 1, 0.0, 1.0, None, stream) == 0
    assert lib.qsx_rk4_block_matrix_real_tc(None, 49, 0, 9, None, 7, None, None, stream) == 0
    A = torch.zeros((0, 4, 4), dtype=torch.float64, device='cuda')
    B = torch.zeros((0, 4, 4), dtype=torch.float64, device='cuda')
    out = _native.gemm(A, B)
    assert out.shape == (0, 4, 4)


def test_two_dimensional_transform_of_an_empty_population_axis():
    x = torch.zeros((8, 0, 8), dtype=torch.complex128, device='cuda')
    X = _native.dft2(x, 0.0, 1.0, np.arange(4.0), -1, 0.0, 1.0, np.arange(5.0), 1)
    assert X.shape == (4, 0, 5)


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('fp32', 1e-4)])
def test_single_sample_ensemble_workload_matches_oracle(precision, tol):
    """The benchmarked entry point on one disorder sample (the smallest
    ragged batch: one warp of one CTA does work in every kernel)."""
    from qspectra_gb300.simulate.ensemble import RedfieldEnsembleWorkload
    H = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H, 1.0, qg.CM_FS)
    fwhm = wl.fwhm_for_sd(80.0)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=fwhm, random_seed=1,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    psi = np.zeros(7)
    psi[0] = 1.0
    work = RedfieldEnsembleWorkload(m, 512.0, 300.0, psi)
    sample = 4321
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(1, start=sample)).cuda()
    X, pops, status = work.run(offs, precision)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    obath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H, dipoles=[[1, 0, 0]] * 7, disorder=fwhm,
                                         random_seed=1, energy_spread_extra=extra, bath=obath)
    om = orc.RedfieldSpec(oham, obath, 'ge', orc.CM_FS, secular=False).sample(sample)
    _, oX = orc.absorption_spectra(om, 512.0)
    _, rho = orc.simulate_dynamics(om, psi, 300.0)
    assert rel_err(X.cpu().numpy(), oX) < tol
    assert rel_err(pops.cpu().numpy(), np.einsum('tii->ti', rho).real) < tol


@pytest.mark.parametrize('n_sites', [3, 7])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('fp32', 1e-4)])
def test_drivers_with_one_sample_ensembles_match_oracle(n_sites, precision, tol):
    """absorption_spectra and simulate_dynamics with ensemble_size=1 (the
    batched pipelines on a batch of one) against the oracle's one-sample
    ensemble average (decorators.py:40-64)."""
    H = wl.fmo7_hamiltonian(n_sites)
    extra = wl.energy_spread_for_dt(H, 1.0, qg.CM_FS)
    fwhm = wl.fwhm_for_sd(80.0)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * n_sites, disorder=fwhm, random_seed=3,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    obath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H, dipoles=[[1, 0, 0]] * n_sites, disorder=fwhm,
                                         random_seed=3, energy_spread_extra=extra, bath=obath)
    om = orc.RedfieldSpec(oham, obath, 'ge', orc.CM_FS, secular=False)
    f, X = qg.absorption_spectra(m, 300.0, ensemble_size=1, precision=precision)
    _, oX = orc.ensemble_average(om, 1, orc.absorption_spectra, 300.0)
    assert rel_err(X, oX) < tol
    psi = np.zeros(n_sites)
    psi[-1] = 1.0
    _, rho = qg.simulate_dynamics(m, psi, 200.0, ensemble_size=1, precision=precision)
    _, orho = orc.ensemble_average(om, 1, orc.simulate_dynamics, psi, 200.0)
    assert rel_err(rho, orho) < tol


@pytest.mark.gpu
@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
def test_projected_mean_reports_a_non_finite_sample(dtype):
    """The absorption leg's loops check each sample's final state on the
    device: one sample whose step matrix holds a NaN sets QSX_ERR_NONFINITE
    in the status word, and raise_for_status raises IntegratorError, as
    integrate() does in the reference (simulate/utils.py:12-13).  A clean
    ensemble reports status 0."""
    from qspectra_gb300.simulate.ensemble import projected_mean, raise_for_status
    B, m, nsteps = 64, 7, 400
    g = torch.Generator().manual_seed(11)
    D = (torch.randn(B, m, m, dtype=torch.complex128, generator=g) * 1e-3).to(dtype).cuda()
    y0 = torch.randn(m, dtype=torch.complex128, generator=g).cuda()
    proj = torch.randn(1, m, dtype=torch.complex128, generator=g).cuda()
    clean = projected_mean(D, y0, proj, nsteps)
    assert int(clean['status'].item()) == 0
    raise_for_status(int(clean['status'].item()))
    D[5, 2, 3] = float('nan')
    bad = projected_mean(D, y0, proj, nsteps)
    assert int(bad['status'].item()) & _native.QSX_ERR_NONFINITE
    with pytest.raises(_native.IntegratorError):
        raise_for_status(int(bad['status'].item()))
