"""GPU parity of the batched third-order engine against the oracle.

The oracle builds the dense 'gef' Redfield generator and integrates every
pathway (response.py:267-337); the engine never forms that generator (f
manifold in operator form, t2 by propagator powers, dipoles as CSR maps).
"""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from qspectra_gb300.dynamics.redfield import RedfieldBuild
from qspectra_gb300.operator_tools import occupation_table
from qspectra_gb300.simulate.ensemble import SampleBatch
from qspectra_gb300.simulate.third_order import ThirdOrderEngine

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4
DT = 2.0


def chain_pair(n_sites, seed=11, sd=60.0):
    """(model, oracle model) for a disordered chain whose time step is 2 fs."""
    H = wl.chain_hamiltonian(n_sites=n_sites, seed=seed)
    extra = wl.energy_spread_for_dt(H, DT, qg.CM_FS)
    bath = qg.DebyeBath(qg.CM_K * 300, 40, 100)
    ham = qg.ElectronicHamiltonian(H, bath=bath, dipoles=[[1, 0, 0]] * n_sites,
                                   disorder=wl.fwhm_for_sd(sd), random_seed=5,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS, secular=False)
    obath = orc.DebyeBathSpec(orc.CM_K * 300, 40, 100)
    oham = orc.ElectronicHamiltonianSpec(H, dipoles=[[1, 0, 0]] * n_sites,
                                         disorder=wl.fwhm_for_sd(sd), random_seed=5,
                                         energy_spread_extra=extra, bath=obath)
    om = orc.RedfieldSpec(oham, obath, 'gef', orc.CM_FS, secular=False)
    assert m.time_step == DT and om.time_step == DT
    return m, om


@pytest.mark.parametrize('precision,tol', [('fp64', FP64_TOL), ('fp32', FP32_TOL)])
def test_fe_heisenberg_rk4_matches_dense_block(precision, tol):
    """Operator-form 'fe' RK4 (qsx_fblock_tensor -> qsx_fe_generator ->
    qsx_fe_heisenberg_rk4) against RK4 on the oracle's dense transposed
    'fe' block (liouville_space.py:316-341)."""
    N, S, nsteps = 5, 3, 6
    m, om = chain_pair(N)
    eng = ThirdOrderEngine(m, 40.0, [0.0], precision=precision)
    offsets = m.hamiltonian.disorder_offsets(S)
    batch = SampleBatch(m, S, offsets=offsets)
    uc = m.unit_convert
    Hge = batch.H('ge')
    build = RedfieldBuild(Hge, N, 'ge', occupation_table(N, 'ge'), m.hamiltonian.bath, uc,
                          False, False, 'site')
    cdt = torch.complex64 if precision == 'fp32' else torch.complex128
    Q = eng._f_operators(batch, build, cdt)
    Me = build.M[:, :, 1:, 1:].to(cdt).contiguous()
    Ae = (build.G[:, 1:, 1:] + 1j * uc * Hge[:, 1:, 1:]).to(cdt).contiguous()
    rng = np.random.RandomState(2)
    P = N * (N - 1) // 2
    y0 = rng.randn(S, P * N) + 1j * rng.randn(S, P * N)
    out = _native.fe_heisenberg_rk4(Q, Ae, Me, eng._pair_sites,
                                    torch.as_tensor(y0).cuda(), nsteps, DT,
                                    eng.prec).cpu().numpy()
    t = np.arange(nsteps + 1) * DT
    for s in range(S):
        LH = om.sample(s).eom_matrix('fe', heisenberg_picture=True)
        ref = orc.rk4_integrate(LH, y0[s], t, h=DT)
        assert rel_err(out[s], ref) < tol


def test_csr_map_kernel_matches_dense():
    rng = np.random.RandomState(4)
    A = (rng.rand(40, 70) < 0.1) * (rng.randn(40, 70) + 1j * rng.randn(40, 70))
    x = rng.randn(5, 3, 70) + 1j * rng.randn(5, 3, 70)
    y = _native.CsrMap(A)(torch.as_tensor(x).cuda()).cpu().numpy()
    assert rel_err(y, x @ A.T) < 1e-14


@pytest.mark.parametrize('n_sites', [4, 5])
@pytest.mark.parametrize('geo', ['-++', '+-+'])
def test_engine_ensemble_matches_oracle(n_sites, geo):
    m, om = chain_pair(n_sites)
    S = 3
    ticks, ref = orc.ensemble_average(om, S, orc.third_order_response, 40.0,
                                      [0.0, 20.0, 50.0], geometry=geo)
    (t1, t2, t3), X64 = qg.third_order_response(m, 40.0, population_times=[0.0, 20.0, 50.0],
                                                geometry=geo, ensemble_size=S)
    assert np.array_equal(t1, ticks[0]) and np.array_equal(t3, ticks[2])
    assert X64.shape == ref.shape == (20, 3, 20)
    assert rel_err(X64, ref) < FP64_TOL
    _, X32 = qg.third_order_response(m, 40.0, population_times=[0.0, 20.0, 50.0],
                                     geometry=geo, ensemble_size=S, precision='fp32')
    assert rel_err(X32, ref) < FP32_TOL


@pytest.mark.parametrize('signals', ['ESA', 'GSB,ESE', 'GSB'])
def test_engine_pathway_selection(signals):
    m, om = chain_pair(4)
    om0 = om.sample(0)
    _, ref = orc.third_order_response(om0, 30.0, [10.0, 30.0], geometry='-++',
                                      include_signal=signals.split(','))
    _, X = qg.third_order_response(m.sample_ensemble(1).__next__(), 30.0,
                                   population_times=[10.0, 30.0], geometry='-++',
                                   include_signal=signals)
    assert rel_err(X, ref) < FP64_TOL


def test_engine_both_geometries_in_one_pass():
    """One run returns both geometries, equal to two single-geometry runs."""
    m, _ = chain_pair(4)
    offsets = m.hamiltonian.disorder_offsets(2)
    both = ThirdOrderEngine(m, 20.0, [0.0, 10.0], precision='fp64').run(offsets)
    for geo in ('-++', '+-+'):
        one = ThirdOrderEngine(m, 20.0, [0.0, 10.0], precision='fp64',
                               geometries=(geo,)).run(offsets)[geo]
        assert rel_err(both[geo].cpu().numpy(), one.cpu().numpy()) < 1e-14


@pytest.mark.parametrize('n,B', [(1, 3), (2, 4), (3, 2), (17, 5), (64, 3), (276, 2)])
def test_eigh_large_matches_numpy(n, B):
    """Householder + QL kernel against numpy.linalg.eigh (scipy.linalg.eigh
    stands behind the reference's Hamiltonian.eig, hamiltonian.py:310-328)."""
    rng = np.random.RandomState(n)
    A = rng.randn(B, n, n) * 50
    A = A + A.transpose(0, 2, 1)
    if n >= 3:
        A[0, 0, 2:] = A[0, 2:, 0] = 0.0   # a column already in tridiagonal form
        A[-1] += np.diag(np.arange(n) * 1e3)
    E, U = _native.eigh_large(torch.as_tensor(A).cuda())
    E, U = E.cpu().numpy(), U.cpu().numpy()
    for k in range(B):
        ref = np.linalg.eigvalsh(A[k])
        scale = np.abs(ref).max()
        assert np.max(np.abs(E[k] - ref)) < 1e-13 * n * scale
        rec = U[k] @ np.diag(E[k]) @ U[k].T
        assert np.max(np.abs(rec - A[k])) < 1e-13 * n * scale
        assert np.max(np.abs(U[k].T @ U[k] - np.eye(n))) < 1e-13 * n


def test_eigh_large_two_exciton_block():
    """f block of the 24-site chain (degenerate-free but densely spaced)."""
    H = wl.chain_hamiltonian(n_sites=24, seed=2024) - 12300 * np.eye(24)
    from qspectra_gb300.operator_tools import operator_1_to_2
    Hf = operator_1_to_2(H)
    E, U = _native.eigh_large(torch.as_tensor(Hf[None]).cuda())
    ref = np.linalg.eigvalsh(Hf)
    assert np.max(np.abs(E[0].cpu().numpy() - ref)) < 1e-11
    U = U[0].cpu().numpy()
    assert np.max(np.abs(U @ np.diag(E[0].cpu().numpy()) @ U.T - Hf)) < 1e-10


@pytest.mark.parametrize('dtype,tol', [(torch.complex128, 1e-13), (torch.complex64, 1e-5)])
def test_hermitian_rows_round_trip_and_real_form_action(dtype, tol):
    """qsx_hermitian_rows splits rows into the coordinates of their Hermitian
    and anti-Hermitian parts and merges them back; on those coordinates the
    real form of a Hermiticity-preserving map acts as the map itself."""
    from qspectra_gb300 import _native
    rng = np.random.RandomState(5)
    n, S, R = 5, 3, 7
    v = rng.randn(S, R, n * n) + 1j * rng.randn(S, R, n * n)
    x = torch.as_tensor(v).to(dtype).cuda()
    back = _native.hermitian_rows(_native.hermitian_rows(x, n), n, merge=True)
    assert rel_err(back.cpu().numpy(), x.cpu().numpy()) < tol
    # a Hermiticity-preserving map: X -> K X K^H + X B with K complex,
    # B Hermitian, as a matrix on column-stacked vectors
    K = rng.randn(n, n) + 1j * rng.randn(n, n)
    Bh = rng.randn(n, n) + 1j * rng.randn(n, n)
    Bh = Bh + Bh.conj().T
    I = np.eye(n)
    A = np.kron(K.conj(), K) + np.kron(Bh.T, I) + np.kron(I, Bh)
    At = torch.as_tensor(np.broadcast_to(A, (S,) + A.shape).copy()).to(dtype).cuda()
    Ar = _native.hermitian_real_form(At, n)
    ref = np.einsum('kl,srl->srk', A, v)
    y = torch.einsum('skl,srl->srk', Ar, _native.hermitian_rows(x, n))
    got = _native.hermitian_rows(y.contiguous(), n, merge=True).cpu().numpy()
    assert rel_err(got, ref) < 10 * tol
