"""Field-driven propagation (simulate_with_fields / simulate_pump,
qspectra/simulate/eom.py:77-227) through qsx_rk4_field_batched, against the
reference's own runs (RK4 harness fixtures) and the oracle."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def fmo7_model(golden):
    ham = qg.ElectronicHamiltonian(golden['fmo7_H'], bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=wl.fwhm_for_sd(80.0),
                                   random_seed=1,
                                   energy_spread_extra=float(golden['fmo7_extra']))
    return qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('fp32', 1e-4)])
def test_simulate_pump_matches_reference(golden, precision, tol):
    m = fmo7_model(golden)
    pump = qg.GaussianPulse(carrier_freq=12350.0, fwhm=20.0, t_peak=0.0, scale=1e-2,
                            freq_convert=qg.CM_FS)
    t, st = qg.simulate_pump(m, pump, polarization='x', time_extra=60.0, precision=precision)
    assert np.allclose(t, golden['fields_pump_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['fields_pump_states']) < tol
    # the excited-state part alone (the pump moves about 1e-4 of the population)
    sel = slice(1, None)
    assert rel_err(st[:, sel], golden['fields_pump_states'][:, sel]) < tol * 10


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('fp32', 1e-4)])
def test_simulate_with_fields_ensemble_matches_reference(golden, precision, tol):
    m = fmo7_model(golden)
    p1 = qg.GaussianPulse(carrier_freq=12250.0, fwhm=15.0, t_peak=-10.0, scale=5e-3,
                          freq_convert=qg.CM_FS)
    p2 = qg.GaussianPulse(carrier_freq=12450.0, fwhm=25.0, t_peak=20.0, scale=8e-3,
                          freq_convert=qg.CM_FS)
    t, st = qg.simulate_with_fields(m, [p1, p2], geometry='-+', polarization='xy',
                                    time_extra=40.0, ensemble_size=3, precision=precision)
    assert np.allclose(t, golden['fields_two_t'], rtol=0, atol=1e-12)
    assert rel_err(st, golden['fields_two_states']) < tol


def test_field_kernel_without_pulses_is_the_plain_loop():
    """With no pulses the kernel is the stage-form RK4 of L."""
    rng = np.random.RandomState(0)
    L = 0.05 * (rng.randn(3, 9, 9) + 1j * rng.randn(3, 9, 9))
    y0 = rng.randn(9) + 1j * rng.randn(9)
    out = _native.rk4_field(torch.as_tensor(L).cuda(), None, None,
                            torch.as_tensor(y0).cuda(), 12, 0.7, 3).cpu().numpy()
    for s in range(3):
        ref = orc.rk4_integrate(L[s], y0, np.arange(5) * 3 * 0.7, h=0.7)
        assert rel_err(out[s], ref) < 1e-12


def test_field_kernel_rejects_oversized_maps():
    L = torch.zeros((1, 200, 200), dtype=torch.complex128, device='cuda')
    C = torch.zeros((2, 200, 200), dtype=torch.complex128, device='cuda')
    coef = torch.zeros((4, 3, 2), dtype=torch.complex128, device='cuda')
    y0 = torch.zeros(200, dtype=torch.complex128, device='cuda')
    with pytest.raises(_native.QsxError):
        _native.rk4_field(L, C, coef, y0, 4, 1.0)
