"""Real (Hermitian) form of diagonal population blocks: the coordinate map,
the fused real propagator, the real K-step blocked matrix and loop, and the
ensemble drivers that use them, against the complex path and the oracle."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from qspectra_gb300.simulate import ensemble as ens

pytestmark = pytest.mark.gpu


def lindblad_maps(n, B, seed):
    """Random Hermiticity-preserving generators -i[H, .] + K . K^+ - {K^+K, .}/2."""
    rng = np.random.RandomState(seed)
    I = np.eye(n)
    out = []
    for _ in range(B):
        H = rng.randn(n, n)
        H = H + H.T
        K = rng.randn(n, n) + 1j * rng.randn(n, n)
        KK = K.conj().T @ K
        out.append(-1j * (np.kron(I, H) - np.kron(H.T, I)) + np.kron(K.conj(), K)
                   - 0.5 * (np.kron(I, KK) + np.kron(KK.T, I)))
    return np.array(out)


def real_form_np(L, n):
    x = np.eye(n * n)
    cols = ens.from_hermitian_coordinates(x, n)              # basis matrices as columns
    return np.array([ens.hermitian_coordinates((Lb @ cols.T).T, n).T for Lb in L])


@pytest.mark.parametrize('n', [3, 5, 7])
def test_real_form_kernel(n):
    L = lindblad_maps(n, 4, seed=n)
    ref = real_form_np(L, n)
    for dt, tol in ((torch.complex128, 1e-14), (torch.complex64, 1e-6)):
        R = _native.hermitian_real_form(torch.as_tensor(L).to(dt).cuda(), n).cpu().numpy()
        assert rel_err(R, ref) < tol


def fmo_build(S=6, nsites=7):
    H = wl.fmo7_hamiltonian(nsites)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * nsites, disorder=wl.fwhm_for_sd(80.0),
                                   random_seed=1,
                                   energy_spread_extra=wl.energy_spread_for_dt(H, 1.0, qg.CM_FS))
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    batch = ens.SampleBatch(m, S)
    return m, m.build_batch(batch.H('ge'))


@pytest.mark.parametrize('precision,tol', [(_native.QSX_FP64, 1e-12), (_native.QSX_FP32, 2e-5)])
def test_fused_real_propagator_matches_complex(precision, tol):
    m, build = fmo_build()
    idx = m.liouville_subspace_index('ee')
    D = build.propagator(idx, 1.0, _native.QSX_FP64)
    ref = _native.hermitian_real_form(D, 7).cpu().numpy()
    Dr = build.hermitian_propagator(idx, 7, 1.0, precision).cpu().numpy()
    assert rel_err(Dr, ref) < tol


def test_real_block_matrix_and_loop_match_numpy():
    rng = np.random.RandomState(3)
    n, B, K, nsteps = 4, 5, 4, 24
    m = n * n
    L = 0.05 * real_form_np(lindblad_maps(n, B, seed=9), n)
    P = np.array([np.eye(m) + Lb + Lb @ Lb / 2 for Lb in L])      # any real propagator
    D = P - np.eye(m)
    sel = [0, 5, 10, 15, 3]
    mat = _native.rk4_block_matrix_real(torch.as_tensor(D).cuda(), K, sel).cpu().numpy()
    for b in range(B):
        assert rel_err(mat[b, :m], np.linalg.matrix_power(P[b], K) - np.eye(m)) < 1e-13
        for k in range(1, K):
            Dk = np.linalg.matrix_power(P[b], k) - np.eye(m)
            assert rel_err(mat[b, m + (k - 1) * len(sel):m + k * len(sel)], Dk[sel]) < 1e-13
    mat32 = _native.rk4_block_matrix_real(torch.as_tensor(D).float().cuda(), K, sel)
    x0 = rng.randn(B, m)
    mean, _ = _native.rk4_real_block_mean(mat32, torch.as_tensor(x0).cuda(), nsteps, sel, K)
    xs = np.array([[np.linalg.matrix_power(P[b], t) @ x0[b] for t in range(nsteps + 1)]
                   for b in range(B)])
    assert rel_err(mean.cpu().numpy(), xs.mean(0)[:, sel]) < 2e-6


@pytest.mark.parametrize('n,K,nsteps,sel,group', [
    (4, 4, 24, [0, 5, 10, 15, 3], 0),     # two-pass: chain + tensor-core contraction
    (4, 2, 300, [0, 5, 10, 15], 0),       # 150 block-steps: fused warp-specialised loop
    (4, 4, 24, [0, 5, 10, 15, 3], 2),     # two samples per CTA: grouped loop
    (7, 9, 999, list(range(0, 49, 8)), 0),  # the fmo7 shape, two-pass
    (3, 3, 90, [0, 4, 8, 1], 0),          # m = 9, two-pass
])
def test_real_loop_paths_match_numpy(n, K, nsteps, sel, group):
    """Every execution path of qsx_rk4_real_block_mean against numpy powers
    of the same FP32 propagators."""
    rng = np.random.RandomState(n + K)
    B = 40
    m = n * n
    L = 0.02 * real_form_np(lindblad_maps(n, B, seed=n + 1), n)
    P = np.array([np.eye(m) + Lb + Lb @ Lb / 2 for Lb in L])
    D32 = torch.as_tensor(P - np.eye(m)).float().cuda()
    mat = _native.rk4_block_matrix_real(D32, K, sel)
    x0 = rng.randn(B, m)
    mean, st = _native.rk4_real_block_mean(mat, torch.as_tensor(x0).cuda(), nsteps, sel, K,
                                           group=group)
    assert int(st.item()) == 0
    Pd = (D32.cpu().numpy().astype(np.float64) + np.eye(m))
    ref = np.zeros((nsteps + 1, len(sel)))
    for b in range(B):
        x = x0[b].copy()
        for t in range(nsteps + 1):
            ref[t] += x[sel]
            x = Pd[b] @ x
    ref /= B
    assert rel_err(mean.cpu().numpy(), ref) < 2e-5


@pytest.mark.parametrize('full_state', [False, True])
def test_ensemble_populations_real_form_matches_complex_and_fp64(full_state):
    m, _ = fmo_build()
    psi = np.zeros(7)
    psi[2] = 1.0
    args = (m, psi, 600.0, 64, 'ee')
    t, r64 = ens.ensemble_populations(*args, precision='fp64', full_state=full_state)
    _, r32 = ens.ensemble_populations(*args, precision='fp32', full_state=full_state)
    ens.set_hermitian_form(False)
    try:
        _, c32 = ens.ensemble_populations(*args, precision='fp32', full_state=full_state)
    finally:
        ens.set_hermitian_form(True)
    r64, r32, c32 = (x.cpu().numpy() for x in (r64, r32, c32))
    assert rel_err(r32, r64) < 1e-5
    assert rel_err(c32, r64) < 1e-5


def test_workload_uses_real_form_and_matches_fp64():
    from qspectra_gb300.simulate.ensemble import RedfieldEnsembleWorkload
    m, _ = fmo_build()
    psi = np.zeros(7)
    psi[0] = 1.0
    work = RedfieldEnsembleWorkload(m, 512.0, 1000.0, psi)
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(256)).cuda()
    X64, P64, _ = work.run(offs, 'fp64')
    # K = 9 pinned: the tcgen05 build; K = 8 (1000 = 125 x 8 steps run, the
    # last dropped); then the measured choice of K
    for pin, variant in ((9, 'tcgen05'), (8, 'tcgen05'), (None, None)):
        ens.set_block_k_real(pin)
        try:
            ev = {}
            X32, P32, st = work.run(offs, 'fp32', ev)
        finally:
            ens.set_block_k_real(None)
        assert ev['dyn_variant'] == 'real'
        if pin is not None:
            assert ev['dyn_block_k'] == pin and ev['blockbuild_variant'] == variant
        else:
            assert 2 <= ev['dyn_block_k'] <= 64
        assert int(st.item()) == 0
        assert rel_err(P32.cpu().numpy(), P64.cpu().numpy()) < 1e-5
        assert rel_err(X32.cpu().numpy(), X64.cpu().numpy()) < 1e-5


def test_workload_graph_replay_matches_eager():
    """One captured step replayed (device input, then pinned host input
    through run_host) gives the eager step's results."""
    from qspectra_gb300.simulate.ensemble import RedfieldEnsembleWorkload
    m, _ = fmo_build()
    psi = np.zeros(7)
    psi[1] = 1.0
    work = RedfieldEnsembleWorkload(m, 512.0, 1000.0, psi)
    offs = torch.as_tensor(m.hamiltonian.disorder_offsets(192))
    X, P, st = work.run(offs.cuda(), 'fp32')
    X, P = X.cpu().numpy(), P.cpu().numpy()
    assert work.capture(offs.cuda(), 'fp32')
    Xg, Pg, stg = work.replay()
    assert int(stg.item()) == 0
    assert rel_err(Xg.cpu().numpy(), X) < 1e-12 and rel_err(Pg.cpu().numpy(), P) < 1e-12
    other = torch.as_tensor(m.hamiltonian.disorder_offsets(192, start=500)).pin_memory()
    Xh, Ph = work.run_host(other, 'fp32')
    X2, P2, _ = work.run(other.cuda(), 'fp32')
    assert rel_err(Xh, X2.cpu().numpy()) < 1e-12 and rel_err(Ph, P2.cpu().numpy()) < 1e-12


def test_tensor_core_and_cuda_core_block_builds_agree_in_the_ensemble(monkeypatch):
    """The ensemble populations through the tcgen05 block build equal those
    through the CUDA-core FP32 build to FP32 rounding."""
    m, _ = fmo_build()
    psi = np.zeros(7)
    psi[4] = 1.0
    args = (m, psi, 513.0, 300, 'ee')     # 512 steps
    calls = []
    real_tc = _native.rk4_block_matrix_real_tc

    def counting(D, K, select):
        res = real_tc(D, K, select)
        calls.append((K, res is not None))
        return res

    monkeypatch.setattr(_native, 'rk4_block_matrix_real_tc', counting)
    _, tc = ens.ensemble_populations(*args, precision='fp32')
    assert calls and all(ok for _, ok in calls)
    monkeypatch.setattr(ens, '_TENSOR_CORE_BLOCKS', False)
    _, cc = ens.ensemble_populations(*args, precision='fp32')
    assert len(calls) == 1 or all(ok for _, ok in calls)
    assert rel_err(tc.cpu().numpy(), cc.cpu().numpy()) < 2e-6


# (7, 1, 2047) and (4, 3, 679) fit one warp per sample (m + P K <= 32), the
# others take the CTA-wide loop
@pytest.mark.parametrize('m,P,nsteps', [(7, 1, 2047), (4, 3, 679), (3, 2, 120), (8, 1, 96),
                                        (5, 3, 64)])
def test_projection_blocked_loop_matches_stepwise(m, P, nsteps):
    """The K-step projection loop (qsx_rk4_proj_block_*) against the
    step-by-step batched loop and an FP64 NumPy recurrence."""
    rng = np.random.RandomState(m + P)
    B = 37
    A = 0.005 * (rng.randn(B, m, m) + 1j * rng.randn(B, m, m)) - 0.03 * np.eye(m)[None]
    D = torch.as_tensor(A).to(torch.complex64).cuda()
    y0 = torch.as_tensor(rng.randn(m) + 1j * rng.randn(m)).cuda()
    proj = torch.as_tensor(rng.randn(P, m) + 1j * rng.randn(P, m)).cuda()
    K = _native.proj_block_k(nsteps, m, P)
    assert K > 1
    blk, _ = _native.rk4_proj_block_mean(D, y0, proj, nsteps, K)
    ref = _native.rk4(D, y0, nsteps, 1, proj=proj, per_sample=False, mean=True)['mean']
    Pm = np.eye(m)[None] + D.cpu().numpy().astype(np.complex128)
    y = np.repeat(y0.cpu().numpy()[None], B, 0)
    exact = []
    for _ in range(nsteps + 1):
        exact.append((y @ proj.cpu().numpy().T).mean(0))
        y = np.einsum('bij,bj->bi', Pm, y)
    exact = np.array(exact)
    assert rel_err(blk.cpu().numpy(), exact) < 2e-6
    assert rel_err(ref.cpu().numpy(), exact) < 2e-6


@pytest.mark.parametrize('m,K,sel', [(49, 9, [i * 7 + i for i in range(7)]),
                                     (49, 8, [0, 8, 16, 24, 32, 40, 48]),
                                     (16, 5, [0, 5, 10, 15]),
                                     (25, 3, list(range(20))),
                                     (64, 2, [3, 9])])
def test_tensor_core_block_matrix_matches(m, K, sel):
    """3xTF32 tcgen05 form of the real blocked matrices against FP64 powers
    and the CUDA-core FP32 kernel."""
    rng = np.random.RandomState(m + K)
    B = 9
    D = 0.02 * rng.randn(B, m, m) - 0.01 * np.eye(m)[None]
    D32 = torch.as_tensor(D).float().cuda()
    res = _native.rk4_block_matrix_real_tc(D32, K, sel)
    assert res is not None
    tc, status = res
    assert int(status.item()) == 0
    ref32 = _native.rk4_block_matrix_real(D32, K, sel).cpu().numpy()
    tc = tc.cpu().numpy()
    Dd = D32.cpu().numpy().astype(np.float64)
    for b in range(B):
        P = np.eye(m) + Dd[b]
        exact = [np.linalg.matrix_power(P, K) - np.eye(m)]
        for k in range(1, K):
            exact.append((np.linalg.matrix_power(P, k) - np.eye(m))[sel])
        exact = np.concatenate(exact)
        assert rel_err(tc[b], exact) < 2e-6
        assert rel_err(tc[b], ref32[b]) < 2e-6


def test_tensor_core_block_matrix_unsupported_shapes():
    D = torch.zeros((2, 49, 49), dtype=torch.float32, device='cuda')
    assert _native.rk4_block_matrix_real_tc(D, 7, [0, 8]) is None      # K = 7
    assert _native.rk4_block_matrix_real_tc(D, 9, list(range(49))) is None  # 4 x 49 rows
