"""The precision form's FP64 build: FP64 eigenpairs (FP32 Jacobi as the
preconditioner of FP64 Jacobi sweeps) and FP64 Redfield operators
(qsx_redfield_build_w64), against numpy's FP64 eigh and the plain FP64 build
(FP64 Jacobi + FP64 operator kernel), and the benchmarked workload with the
FP64 build and with the FP32 build against the oracle."""
import numpy as np
import pytest
import torch

import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from qspectra_gb300.dynamics.redfield import RedfieldBuild
from qspectra_gb300.operator_tools import occupation_table

pytestmark = pytest.mark.gpu


def ge_hamiltonians(N, B, seed, degenerate=True):
    """(B, N + 1, N + 1) rotating-frame 'ge' Hamiltonians: ground state 0,
    disordered one-exciton block; ``degenerate`` plants equal and nearly
    equal eigenvalues in a few of them."""
    rng = np.random.RandomState(seed)
    H = np.zeros((B, N + 1, N + 1))
    J = np.triu(rng.normal(0, 50, (B, N, N)), 1)
    H[:, 1:, 1:] = J + J.transpose(0, 2, 1)
    idx = np.arange(1, N + 1)
    H[:, idx, idx] = rng.uniform(-300, 300, (B, N))
    # exactly and nearly degenerate eigenvalues in a random eigenbasis, and
    # an exactly diagonal block
    for k, gap in zip(range(1, min(B, 6) if degenerate else 1), (0.0, 1e-9, 1e-5, 1e-3, 1.0)):
        lam = np.sort(rng.uniform(-300, 300, N))
        lam[1] = lam[0] + gap
        Q, _ = np.linalg.qr(rng.randn(N, N))
        blk = Q @ np.diag(lam) @ Q.T
        H[k, 1:, 1:] = 0.5 * (blk + blk.T)
    if B > 6 and degenerate:
        H[6, 1:, 1:] = np.diag(np.diag(H[6, 1:, 1:]))
    return H


@pytest.mark.parametrize('N', [2, 3, 5, 7, 8])
def test_refined_eigenpairs_are_fp64_accurate(N):
    B = 257
    Hn = ge_hamiltonians(N, B, seed=N)
    H = torch.as_tensor(Hn).cuda()
    _, U32 = _native.eigh(H, [0, 1, N + 1], _native.QSX_FP32)
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    E, U, _, _ = _native.redfield_build_w64(H, U32, N, 1, bath, qg.CM_FS)
    E, U = E.cpu().numpy(), U.cpu().numpy()
    for b in range(B):
        A = Hn[b]
        scale = np.abs(A).max()
        # ascending inside each block: the ground state, then the one-exciton block
        assert E[b, 0] == 0.0
        assert np.max(np.abs(E[b, 1:] - np.linalg.eigvalsh(A[1:, 1:]))) < 1e-13 * scale
        assert np.max(np.abs(U[b] @ np.diag(E[b]) @ U[b].T - A)) < 1e-13 * scale
        assert np.max(np.abs(U[b].T @ U[b] - np.eye(N + 1))) < 1e-13


@pytest.mark.parametrize('N,discard', [(7, False), (4, False), (6, True)])
def test_fp64_build_matches_plain_fp64_build(N, discard):
    """Generic (non-degenerate) spectra: the reference's correlation function
    takes a separate value at exactly zero frequency (bath.py:84-102), so at
    an exact degeneracy the operators depend on whether a difference of two
    computed eigenvalues rounds to zero."""
    B = 300
    H = torch.as_tensor(ge_hamiltonians(N, B, seed=10 + N, degenerate=False)).cuda()
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    occ = occupation_table(N, 'ge')
    ref = RedfieldBuild(H, N, 'ge', occ, bath, qg.CM_FS, discard_imag_corr=discard,
                        precision=_native.QSX_FP64)
    got = RedfieldBuild(H, N, 'ge', occ, bath, qg.CM_FS, discard_imag_corr=discard,
                        precision=_native.QSX_FP32)
    assert got.refined and not ref.refined
    assert rel_err(got.G.cpu().numpy(), ref.G.cpu().numpy()) < 1e-12
    assert rel_err(got.M.cpu().numpy(), ref.M.cpu().numpy()) < 1e-12
    assert rel_err(got.E.cpu().numpy(), ref.E.cpu().numpy()) < 1e-13


@pytest.mark.parametrize('build_precision', ['fp64', 'fp32'])
def test_workload_fp32_propagation_with_either_build(golden, build_precision):
    """FP32 propagation against the reference's 8-sample ensemble, with the
    FP64 build (the precision form) and with the FP32 build."""
    from qspectra_gb300.simulate.ensemble import RedfieldEnsembleWorkload
    H = wl.fmo7_hamiltonian()
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=wl.fwhm_for_sd(80.0),
                                   random_seed=1,
                                   energy_spread_extra=wl.energy_spread_for_dt(H, 1.0, qg.CM_FS))
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    psi = np.zeros(7)
    psi[0] = 1.0
    work = RedfieldEnsembleWorkload(m, 2048.0, 1000.0, psi)
    offs = torch.as_tensor(ham.disorder_offsets(8)).cuda()
    X, P, status = work.run(offs, 'fp32', build_precision=build_precision)
    assert int(status.item()) == 0
    assert rel_err(X.cpu().numpy(), golden['fmo7_ens8_abs_X']) < 1e-4
    assert rel_err(P.cpu().numpy(), golden['fmo7_ens8_pops']) < 1e-4


@pytest.mark.parametrize('N,space,discard', [(7, 'ge', False), (3, 'e', False), (8, 'ge', True),
                                             (2, 'ge', False)])
def test_fp32_warp_operator_build_matches_cta_operator_build(N, space, discard):
    """The FP32 build of one-exciton spaces takes the warp-per-sample operator
    form (qsx_redfield_operators_w32): the same G and M as the general FP32
    operator kernel (qsx_redfield_operators_batched, QSX_FP32) on the same
    FP32 eigendecomposition, to FP32 rounding, and close to the FP64 build."""
    B = 300
    Hn = ge_hamiltonians(N, B, seed=30 + N, degenerate=False)
    if space == 'e':
        Hn = np.ascontiguousarray(Hn[:, 1:, 1:])
    H = torch.as_tensor(Hn).cuda()
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    occ = occupation_table(N, space)
    got = RedfieldBuild(H, N, space, occ, bath, qg.CM_FS, discard_imag_corr=discard,
                        precision=_native.QSX_FP32, build_precision=_native.QSX_FP32)
    assert got.K is None and not got.refined
    occ_t = torch.as_tensor(np.asarray(occ, dtype=np.float64)).cuda()
    G32, M32, _ = _native.redfield_operators(got.E, got.U, occ_t, bath, qg.CM_FS, discard,
                                             site_basis=True, precision=_native.QSX_FP32)
    ref = RedfieldBuild(H, N, space, occ, bath, qg.CM_FS, discard_imag_corr=discard,
                        precision=_native.QSX_FP64)
    for a, b in ((got.G, G32), (got.M, M32)):
        assert rel_err(a.cpu().numpy(), b.cpu().numpy()) < 1e-5
    for a, b in ((got.G, ref.G), (got.M, ref.M)):
        assert rel_err(a.cpu().numpy(), b.cpu().numpy()) < 1e-4
    # zero outside the coupled block ('ge': the ground-state row and column)
    if space == 'ge':
        assert torch.count_nonzero(got.M[:, :, 0, :]) == 0
        assert torch.count_nonzero(got.M[:, :, :, 0]) == 0
        assert torch.count_nonzero(got.G[:, 0, :]) == 0
