"""Parity at the benchmarked configurations' own sizes.

* The benchmarked entry point itself, ``RedfieldEnsembleWorkload.run`` (7-site
  model, 16384-sample disorder draws, absorption 2048 x 1 fs, populations
  1000 x 1 fs), in FP64 and FP32: against the reference's own 8-sample
  ensemble (``absorption_spectra`` / ``simulate_dynamics`` with
  ensemble_size=8, decorators.py:40-64) and against the oracle's serial
  ensemble over a 64-sample slice from the middle of the 16384 draws.
* The HEOM configuration: 8-site ring, K = 0, level_cutoff = 5 (495 nodes x
  64), one disorder sample, 200 RK4 steps of 0.5 fs, against the reference's
  own generator driven by the fixed-step RK4 (heom.py:298-443).
* The third-order configuration: one disorder sample of the 24-site chain
  (276 two-exciton states, 'fe' block 6624) through the batched engine, t1 =
  t3 = 128 x 2 fs, t2 = 0 / 200 / 500 fs, both geometries, against the
  block-restricted dense oracle (oracle/blocks.py).

FP64 must match to 1e-10 and FP32 to 1e-4 (max-abs relative).
"""
import os

import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import ROOT, rel_err
from oracle import blocks
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOLS = [('fp64', 1e-10), ('fp32', 1e-4)]


@pytest.fixture(scope='module')
def drivers():
    path = os.path.join(ROOT, 'tests', 'golden', 'reference_golden_drivers.npz')
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


# ------------------------------------------------------- benchmarked workload
def fmo7_models():
    H = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H, 1.0, qg.CM_FS)
    fwhm = wl.fwhm_for_sd(80.0)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=fwhm, random_seed=1,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    obath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H, dipoles=[[1, 0, 0]] * 7, disorder=fwhm,
                                         random_seed=1, energy_spread_extra=extra, bath=obath)
    om = orc.RedfieldSpec(oham, obath, 'ge', orc.CM_FS, secular=False)
    return m, om


@pytest.fixture(scope='module')
def fmo7():
    from qspectra_gb300.simulate.ensemble import RedfieldEnsembleWorkload
    m, om = fmo7_models()
    psi = np.zeros(7)
    psi[0] = 1.0
    return m, om, RedfieldEnsembleWorkload(m, 2048.0, 1000.0, psi)


@pytest.mark.parametrize('precision,tol', TOLS)
def test_benchmarked_workload_matches_reference_ensemble(golden, fmo7, precision, tol):
    m, _, work = fmo7
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(8)).cuda()
    X, pops, status = work.run(offs, precision)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert np.allclose(work.freqs_np, golden['fmo7_abs_f'], rtol=1e-13, atol=1e-9)
    assert rel_err(X.cpu().numpy(), golden['fmo7_ens8_abs_X']) < tol
    assert rel_err(pops.cpu().numpy(), golden['fmo7_ens8_pops']) < tol


@pytest.fixture(scope='module')
def fmo7_slice_oracle(fmo7):
    """The oracle's serial ensemble over samples 8160 .. 8223 of the draws
    (the middle of the 16384-sample benchmark)."""
    _, om, _ = fmo7
    start, S = 8160, 64
    psi = np.zeros(7)
    psi[0] = 1.0
    accX = accP = 0
    for n in range(start, start + S):
        o = om.sample(n)
        f, X = orc.absorption_spectra(o, 2048.0)
        _, rho = orc.simulate_dynamics(o, psi, 1000.0)
        accX = accX + X
        accP = accP + np.einsum('tii->ti', rho).real
    return start, S, accX / S, accP / S


@pytest.mark.parametrize('precision,tol', TOLS)
def test_benchmarked_workload_matches_oracle_slice(fmo7, fmo7_slice_oracle, precision, tol):
    m, _, work = fmo7
    start, S, refX, refP = fmo7_slice_oracle
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(S, start=start)).cuda()
    X, pops, status = work.run(offs, precision)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert rel_err(X.cpu().numpy(), refX) < tol
    assert rel_err(pops.cpu().numpy(), refP) < tol


@pytest.mark.parametrize('precision,tol', TOLS)
def test_benchmarked_workload_host_entry_matches_oracle_slice(fmo7, fmo7_slice_oracle,
                                                              precision, tol):
    """The end-to-end call (pinned host offsets in, numpy out), through the
    captured CUDA graph for FP32."""
    m, _, work = fmo7
    start, S, refX, refP = fmo7_slice_oracle
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(S, start=start)).pin_memory()
    if precision == 'fp32':
        assert work.capture(offs.cuda(), precision)
    X, P = work.run_host(offs, precision)
    assert rel_err(X, refX) < tol
    assert rel_err(P, refP) < tol


# --------------------------------------------------------------- HEOM ring 8
@pytest.mark.parametrize('variant', [0, 1, 2, 3, 4])
@pytest.mark.parametrize('precision,tol', TOLS)
def test_heom_ring8_config_size_matches_reference(drivers, precision, tol, variant):
    """variant 0: the library's choice (the persistent cluster kernel for
    one sample); 1: the per-stage kernels; 2: the cluster kernel forced; 3:
    the per-stage kernels with the node commutators on the tensor cores
    (FP32; FP64 takes variant 1); 4: the per-stage kernels with every term of
    a node visited by every element."""
    H = drivers['ring8_H']
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   disorder=wl.fwhm_for_sd(50.0), random_seed=7)
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=0, level_cutoff=5,
                     low_temp_corr=True)
    assert m.ado_count == 495
    sample = int(drivers['ring8_sample'])
    off = ham.disorder_offsets(1, start=sample)[0]
    Hs = m.hamiltonian.H('e') + np.diag(off)
    assert np.allclose(Hs + m.rw_freq * np.eye(8), drivers['ring8_sample_H'], rtol=0,
                       atol=1e-9)
    tb = m.tables('ee')
    Hb = torch.as_tensor(Hs[None]).cuda()
    y0 = torch.zeros(495 * 64, dtype=torch.complex128, device='cuda')
    y0[0] = 1.0
    prec = _native.QSX_FP32 if precision == 'fp32' else _native.QSX_FP64
    out = _native.heom_rk4(tb, Hb, Hb, y0, 200, 0.5, qg.CM_FS, batch=1, save_every=1,
                           save_nodes=495, precision=prec, variant=variant)
    st = out['state'][0].cpu().numpy()            # (201, 495 * 64)
    assert rel_err(st[:, :64], drivers['ring8_traj_node0']) < tol
    assert rel_err(st[-1], drivers['ring8_final_state']) < tol


# ------------------------------------------------------- third order, 24 sites
@pytest.fixture(scope='module')
def chain24():
    H = wl.chain_hamiltonian(n_sites=24, seed=2024)
    extra = wl.energy_spread_for_dt(H, 2.0, qg.CM_FS)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 40, 100),
                                   dipoles=[[1, 0, 0]] * 24, disorder=wl.fwhm_for_sd(60.0),
                                   random_seed=3, energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS, secular=False)
    sample = 100
    base = orc.ElectronicHamiltonianSpec(H, dipoles=[[1, 0, 0]] * 24,
                                         disorder=wl.fwhm_for_sd(60.0), random_seed=3)
    h = base.sample(sample)
    bath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    bm = blocks.BlockRedfield(h.H1, h.rw_freq, bath.corr_complex, [[1, 0, 0]] * 24, orc.CM_FS)
    ref = {}
    for geo in ('-++', '+-+'):
        _, ref[geo] = blocks.third_order_response(bm, 256.0, [0.0, 200.0, 500.0], 2.0,
                                                  geometry=geo)
    return m, sample, ref


@pytest.mark.parametrize('precision,tol', TOLS)
def test_third_order_chain24_matches_block_oracle(chain24, precision, tol):
    from qspectra_gb300.simulate.third_order import ThirdOrderEngine
    m, sample, ref = chain24
    eng = ThirdOrderEngine(m, 256.0, [0.0, 200.0, 500.0], precision=precision)
    out = eng.run(m.hamiltonian.disorder_offsets(1, start=sample))
    for geo in ('-++', '+-+'):
        got = out[geo].cpu().numpy()
        assert got.shape == (128, 3, 128)
        assert rel_err(got, ref[geo]) < tol
