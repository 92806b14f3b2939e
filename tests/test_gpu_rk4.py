"""Every RK4 kernel shape against the oracle's stage-form RK4 on random generators."""
import numpy as np
import pytest
import torch

import oracle as orc
from conftest import rel_err
from qspectra_gb300 import _native

pytestmark = pytest.mark.gpu


def random_generators(B, M, seed, scale=0.05):
    """Stable complex generators with |hL| ~ scale (like Redfield at dt = 1 fs)."""
    rng = np.random.RandomState(seed)
    A = (rng.randn(B, M, M) + 1j * rng.randn(B, M, M)) * scale / np.sqrt(M)
    A -= 0.5 * scale * np.eye(M)[None]  # damping keeps the trajectories bounded
    return A


def oracle_run(L, y0, nsteps, h, every):
    out = []
    for b in range(L.shape[0]):
        t = np.arange(0, nsteps + 1, every) * h
        out.append(orc.rk4_integrate(L[b], y0[b], t, h=h))
    return np.array(out)


CASES = [(1, 5), (3, 37), (7, 129), (8, 33), (9, 61), (16, 17), (25, 11), (36, 9),
         (49, 23), (64, 5), (10, 7), (70, 3)]


@pytest.mark.parametrize('M,B', CASES)
@pytest.mark.parametrize('prec', ['fp64', 'fp32'])
def test_kernels_state_and_means(M, B, prec):
    h, nsteps, every = 1.0, 40, 4
    L = random_generators(B, M, seed=M * 100 + B)
    rng = np.random.RandomState(M)
    y0 = rng.randn(B, M) + 1j * rng.randn(B, M)
    ref = oracle_run(L, y0, nsteps, h, every)
    Lt = torch.as_tensor(L).cuda()
    y0t = torch.as_tensor(y0).cuda()
    precision = _native.QSX_FP32 if prec == 'fp32' else _native.QSX_FP64
    tol = 1e-5 if prec == 'fp32' else 1e-12
    if M <= 64:
        mat = _native.rk4_propagator(Lt, h, precision)
        form = 0
    else:
        mat = Lt.to(torch.complex64 if prec == 'fp32' else torch.complex128)
        form = 1
    out = _native.rk4(mat, y0t, nsteps, every, form=form, h=h, state=True)
    assert rel_err(out['state'].cpu().numpy(), ref) < tol
    sel = sorted(set([0, M - 1, M // 2]))
    out = _native.rk4(mat, y0t, nsteps, every, form=form, h=h, select=sel, mean=True)
    assert rel_err(out['proj'].cpu().numpy(), ref[:, :, sel]) < tol
    assert rel_err(out['mean'].cpu().numpy(), ref[:, :, sel].mean(0)) < tol
    W = rng.randn(2, M) + 1j * rng.randn(2, M)
    if not (prec == 'fp32' and form == 0 and M in (9, 16, 25, 36, 49, 64)):
        out = _native.rk4(mat, y0t, nsteps, every, form=form, h=h,
                          proj=torch.as_tensor(W).cuda(), mean=True)
        want = np.einsum('pm,btm->btp', W, ref)
        assert rel_err(out['proj'].cpu().numpy(), want) < tol
        assert rel_err(out['mean'].cpu().numpy(), want.mean(0)) < tol


def test_stage_form_matches_propagator_form_fp64():
    B, M, h = 3, 12, 0.5
    L = random_generators(B, M, 5)
    y0 = np.ones((B, M), complex)
    Lt = torch.as_tensor(L).cuda()
    a = _native.rk4(_native.rk4_propagator(Lt, h), torch.as_tensor(y0).cuda(), 30, 1,
                    state=True)['state']
    b = _native.rk4(Lt, torch.as_tensor(y0).cuda(), 30, 1, form=1, h=h, state=True)['state']
    assert rel_err(a.cpu().numpy(), b.cpu().numpy()) < 1e-13


def test_zero_steps_and_shared_inputs():
    M = 7
    L = torch.as_tensor(random_generators(1, M, 2)[0]).cuda()
    y0 = torch.arange(M, dtype=torch.float64, device='cuda').to(torch.complex128)
    D = _native.rk4_propagator(L[None], 1.0, _native.QSX_FP32)[0]
    out = _native.rk4(D, y0.expand(5, M).contiguous(), 0, 1, state=True)
    assert torch.allclose(out['state'][:, 0], y0.expand(5, M))


def test_propagator_is_one_rk4_step():
    L = random_generators(2, 9, 8)
    Lt = torch.as_tensor(L).cuda()
    D = _native.rk4_propagator(Lt, 0.7).cpu().numpy()
    for b in range(2):
        hL = 0.7 * L[b]
        P = np.eye(9) + hL + hL @ hL / 2 + hL @ hL @ hL / 6 + hL @ hL @ hL @ hL / 24
        assert rel_err(D[b], P - np.eye(9)) < 1e-14


def test_fused_redfield_propagator_matches_two_step_path(golden):
    """qsx_redfield_propagator_batched == liouvillian block + rk4 propagator."""
    import qspectra_gb300 as qg
    from qspectra_gb300 import workloads as wl
    ham = qg.ElectronicHamiltonian(golden['fmo7_H'], bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=wl.fwhm_for_sd(80.0))
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    from qspectra_gb300.simulate.ensemble import SampleBatch
    build = m.build_batch(SampleBatch(m, 37).H('ge'))
    for sub, tr in [('ee', False), ('eg', True), ('gg,eg,ge,ee', False)]:
        idx = m.liouville_subspace_index(sub)
        for prec, tol in [(_native.QSX_FP64, 1e-13), (_native.QSX_FP32, 1e-5)]:
            fused = build.propagator(idx, 1.0, prec, transpose=tr).cpu().numpy()
            ref = _native.rk4_propagator(build.block(idx, tr), 1.0, prec).cpu().numpy()
            assert rel_err(fused, ref) < tol


@pytest.mark.parametrize('variant', [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize('M,B,K,nsteps', [(9, 13, 3, 30), (49, 11, 9, 54), (25, 7, 4, 40),
                                          (64, 5, 2, 10), (36, 40, 9, 27), (16, 33, 5, 25)])
def test_block_k_matches_step_by_step(M, B, K, nsteps, variant):
    """K-step blocking gives the same RK4 iterates as the step-by-step loop,
    for every kernel variant (one, two or four lanes per matrix row)."""
    L = random_generators(B, M, seed=M + K)
    rng = np.random.RandomState(K)
    y0 = rng.randn(B, M) + 1j * rng.randn(B, M)
    ref = oracle_run(L, y0, nsteps, 1.0, 1)
    D = _native.rk4_propagator(torch.as_tensor(L).cuda(), 1.0, _native.QSX_FP32)
    sel = [0, M // 3, M - 1, M // 2]
    blk = _native.rk4_block_matrix(D, K, sel)
    assert blk.shape == (B, M + len(sel) * (K - 1), M)
    out = _native.rk4(blk, torch.as_tensor(y0).cuda(), nsteps, 1, select=sel, mean=True,
                      block_k=K, variant=variant)
    assert rel_err(out['proj'].cpu().numpy(), ref[:, :, sel]) < 1e-5
    assert rel_err(out['mean'].cpu().numpy(), ref[:, :, sel].mean(0)) < 1e-5


def test_block_matrix_powers_fp64():
    L = random_generators(2, 16, 3)
    D = _native.rk4_propagator(torch.as_tensor(L).cuda(), 0.5, _native.QSX_FP64)
    sel = [1, 5]
    blk = _native.rk4_block_matrix(D, 5, sel).cpu().numpy()
    Dn = D.cpu().numpy()
    for b in range(2):
        P = np.eye(16) + Dn[b]
        assert rel_err(blk[b, :16], np.linalg.matrix_power(P, 5) - np.eye(16)) < 1e-13
        for k in range(1, 5):
            Pk = np.linalg.matrix_power(P, k) - np.eye(16)
            assert rel_err(blk[b, 16 + (k - 1) * 2:16 + k * 2], Pk[sel]) < 1e-13


def test_block_variant_too_wide_is_rejected():
    """A variant whose block would exceed its compiled size is refused (the
    planner's default and the autotuner fall back to the others)."""
    M, B, K = 49, 3, 3
    L = random_generators(B, M, seed=1)
    D = _native.rk4_propagator(torch.as_tensor(L).cuda(), 1.0, _native.QSX_FP32)
    sel = list(range(M))
    blk = _native.rk4_block_matrix(D, K, sel)
    y0 = torch.ones(M, dtype=torch.complex128, device='cuda')
    with pytest.raises(_native.QsxError):
        _native.rk4(blk, y0, 9, 1, select=sel, mean=True, block_k=K, variant=5)
    out = _native.rk4(blk, y0, 9, 1, select=sel, mean=True, block_k=K)
    assert torch.isfinite(out['mean'].real).all()
