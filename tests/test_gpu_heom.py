"""GPU HEOM generator and RK4 loop against the oracle and the reference fixtures."""
import numpy as np
import pytest
import torch

import oracle as orc
import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from test_heom_tables_cpu import CASES, reference_L

pytestmark = pytest.mark.gpu


def model2(golden, **kw):
    ham = qg.ElectronicHamiltonian(golden['heom2_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106))
    return qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, **kw)


@pytest.mark.parametrize('tag,kw', CASES)
@pytest.mark.parametrize('heis', [False, True])
def test_heom_rhs_matches_reference_generator(golden, tag, kw, heis):
    m = model2(golden, **kw)
    ref = qg.CM_FS * reference_L(golden, tag)
    if heis:
        ref = ref.T
    eom = m.equation_of_motion('ee', heisenberg_picture=heis)
    rng = np.random.RandomState(3)
    x = rng.randn(3, ref.shape[0]) + 1j * rng.randn(3, ref.shape[0])
    got = eom(0.0, x)
    assert rel_err(got, x @ ref.T) < 1e-13


def test_heom_trajectory_fp64_matches_reference(golden):
    ham = qg.ElectronicHamiltonian(golden['heom3_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106))
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=0, level_cutoff=3)
    y0 = np.zeros(m.ado_count * 9, complex)
    y0[0] = 1
    traj = qg.integrate(m.equation_of_motion('ee'), y0, np.arange(0, 100.0, 0.5))
    assert traj.shape == (200, m.ado_count * 9)
    assert rel_err(traj[:, :9], golden['heom3_traj_node0']) < 1e-10
    t, rhos = qg.simulate_dynamics(m, np.array([1.0, 0, 0]), duration=100.0, step=0.5)
    assert rel_err(rhos.reshape(len(t), -1, order='C'),
                   golden['heom3_traj_node0'].reshape(200, 3, 3).transpose(0, 2, 1).reshape(200, -1)) < 1e-10


def test_heom_fp32_split_word_and_batch():
    H = wl.ring_hamiltonian(n_sites=4, seed=11)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   disorder=wl.fwhm_for_sd(50.0))
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=0, level_cutoff=4)
    tb = m.tables('ee')
    S = 5
    offs = m.hamiltonian.disorder_offsets(S)
    Hb = torch.as_tensor(np.array([m.hamiltonian.H('e') + np.diag(o) for o in offs])).cuda()
    Hx, Hy = Hb, Hb
    y0 = torch.zeros(m.ado_count * 16, dtype=torch.complex128, device='cuda')
    y0[0] = 1
    r64 = _native.heom_rk4(tb, Hx, Hy, y0, 400, 0.5, qg.CM_FS, batch=S, save_every=20,
                           precision=_native.QSX_FP64, mean=True)
    r32 = _native.heom_rk4(tb, Hx, Hy, y0, 400, 0.5, qg.CM_FS, batch=S, save_every=20,
                           precision=_native.QSX_FP32, mean=True)
    assert rel_err(r32['state'].cpu().numpy(), r64['state'].cpu().numpy()) < 1e-4
    assert rel_err(r64['mean'].cpu().numpy(), r64['state'].cpu().numpy().mean(0)) < 1e-14
    # every sample equals its own single-sample oracle run
    for s in range(S):
        om = orc.HEOMSpec(orc.ElectronicHamiltonianSpec(H + np.diag(offs[s]),
                                                        rw_freq=m.rw_freq),
                          orc.DebyeBathSpec(orc.CM_K * 300, 35, 106), 'e', orc.CM_FS,
                          level_cutoff=4, K=0, low_temp_corr=True)
        L = om.eom_matrix('ee')
        ref = orc.rk4_integrate_sparse(L, y0.cpu().numpy(), 400, 0.5, save_every=20)
        assert rel_err(r64['state'][s].cpu().numpy(), ref[:, :16]) < 1e-10


@pytest.mark.parametrize('tag,kw', CASES)
@pytest.mark.parametrize('heis', [False, True])
@pytest.mark.parametrize('precision,tol', [(_native.QSX_FP64, 1e-12), (_native.QSX_FP32, 1e-5)])
def test_heom_cluster_form_matches_per_stage_form(golden, tag, kw, heis, precision, tol):
    """The persistent cluster kernel (whole loop in one launch, node ranges
    over the cluster's CTAs, neighbours through distributed shared memory)
    and the per-stage kernels with the node commutators on the tensor cores
    (variant 3, FP32) against the per-stage kernels, on every generator case, both pictures,
    with per-sample Hamiltonians and all nodes saved."""
    m = model2(golden, **kw)
    tb = m.tables('ee', transpose=heis)
    S = 3
    base = m.hamiltonian.H('e')
    rng = np.random.RandomState(4)
    Hb = torch.as_tensor(np.array([base + np.diag(rng.randn(2) * 30) for _ in range(S)])).cuda()
    E = tb.nx * tb.ny
    y0 = torch.as_tensor(rng.randn(S, m.ado_count * E) + 1j * rng.randn(S, m.ado_count * E)).cuda()
    out = []
    for variant in (0, 1, 2, 3, 4):
        out.append(_native.heom_rk4(tb, Hb, Hb, y0, 60, 0.5, qg.CM_FS, batch=S, save_every=6,
                                    save_nodes=m.ado_count, precision=precision,
                                    variant=variant)['state'].cpu().numpy())
    assert rel_err(out[0], out[1]) < tol
    assert rel_err(out[2], out[1]) < tol
    assert rel_err(out[3], out[1]) < tol   # node commutators on the tensor cores (FP32)
    assert rel_err(out[4], out[1]) < tol   # per-stage, every term of the node per element


def _drivers():
    import os
    from conftest import ROOT
    with np.load(os.path.join(ROOT, 'tests', 'golden', 'reference_golden_drivers.npz')) as z:
        return {k: z[k] for k in z.files}


def _ref_sparse(g, tag):
    import scipy.sparse as sps
    return sps.coo_matrix((g['heomopt_{}_val'.format(tag)],
                           (g['heomopt_{}_row'.format(tag)], g['heomopt_{}_col'.format(tag)])),
                          shape=tuple(g['heomopt_{}_n'.format(tag)])).tocsr()


@pytest.mark.parametrize('tag,sub', [('multi', 'gg,ge,eg,ee'), ('multi2', 'ge,ee')])
@pytest.mark.parametrize('heis', [False, True])
def test_heom_multiblock_subspace_matches_reference(tag, sub, heis):
    """A Liouville subspace of several blocks (the reference builds the
    generator on their union): the composed GPU generator, applied and
    integrated, against the reference's HEOM_tensor."""
    g = _drivers()
    ham = qg.ElectronicHamiltonian(g['heomopt_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   dipoles=[[1, 0, 0]] * 2)
    m = qg.HEOMModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, K=1, level_cutoff=3)
    ref = qg.CM_FS * _ref_sparse(g, tag)
    if heis:
        ref = ref.T.tocsr()
    eom = m.equation_of_motion(sub, heisenberg_picture=heis)
    rng = np.random.RandomState(5)
    x = rng.randn(2, ref.shape[0]) + 1j * rng.randn(2, ref.shape[0])
    assert rel_err(eom(0.0, x), (ref @ x.T).T) < 1e-13
    t = np.arange(0, 20.0, 0.5)
    traj = qg.integrate(eom, x[0], t, step=0.5)
    oref = orc.rk4_integrate_sparse(ref, x[0], len(t) - 1, 0.5)
    assert rel_err(traj, oref) < 1e-10


@pytest.mark.parametrize('tag,low', [('aki', True), ('aki_nolt', False)])
@pytest.mark.parametrize('precision,tol', [(_native.QSX_FP64, 1e-10), (_native.QSX_FP32, 1e-4)])
def test_heom_aki_temp_corr_matches_reference(tag, low, precision, tol):
    """aki_temp_corr (heom.py:385-442): the generator against the reference's,
    and both RK4 forms (persistent cluster and per-stage kernels) against the
    oracle's RK4 over the reference matrix."""
    g = _drivers()
    ham = qg.ElectronicHamiltonian(g['heomopt_H'], bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   dipoles=[[1, 0, 0]] * 2)
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=1, level_cutoff=3,
                     aki_temp_corr=True, low_temp_corr=low)
    ref = qg.CM_FS * _ref_sparse(g, tag)
    rng = np.random.RandomState(6)
    x = rng.randn(ref.shape[0]) + 1j * rng.randn(ref.shape[0])
    if precision == _native.QSX_FP64:
        assert rel_err(m.equation_of_motion('ee')(0.0, x), ref @ x) < 1e-13
    oref = orc.rk4_integrate_sparse(ref, x, 60, 0.5)
    tb = m.tables('ee')
    Hx, Hy = m.block_hamiltonians('ee')
    for variant in (0, 1, 2, 3, 4):
        out = _native.heom_rk4(tb, Hx, Hy, torch.as_tensor(x).cuda(), 60, 0.5, qg.CM_FS,
                               batch=1, save_nodes=m.ado_count, precision=precision,
                               variant=variant)['state'][0].cpu().numpy()
        assert rel_err(out, oref) < tol


@pytest.mark.parametrize('block', ['ff', 'ef', 'ee'])
@pytest.mark.parametrize('precision,tol', [(_native.QSX_FP64, 1e-10), (_native.QSX_FP32, 1e-4)])
def test_heom_two_exciton_blocks_every_kernel_form(block, precision, tol):
    """A 'gef' hierarchy: two-exciton states couple to two sites each, so the
    site-grouped stage kernel takes its full term loop for those rows and
    columns.  Every kernel form against the oracle's generator (heom.py:
    298-443) driven by the fixed-step RK4."""
    H = wl.chain_hamiltonian(n_sites=3, seed=4)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 35, 106))
    m = qg.HEOMModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS, K=0, level_cutoff=3,
                     low_temp_corr=True)
    om = orc.HEOMSpec(orc.ElectronicHamiltonianSpec(H, rw_freq=m.rw_freq),
                      orc.DebyeBathSpec(orc.CM_K * 300, 35, 106), 'gef', orc.CM_FS,
                      level_cutoff=3, K=0, low_temp_corr=True)
    lsub = block
    L = om.eom_matrix(lsub)
    tb = m.tables(lsub)
    E = tb.nx * tb.ny
    assert L.shape[0] == m.ado_count * E
    rng = np.random.RandomState(8)
    y0 = rng.randn(L.shape[0]) + 1j * rng.randn(L.shape[0])
    ref = orc.rk4_integrate_sparse(L, y0, 80, 0.5, save_every=8)
    Hx, Hy = m.block_hamiltonians(lsub)
    out = []
    for variant in (1, 3, 4):
        r = _native.heom_rk4(tb, Hx, Hy, torch.as_tensor(y0).cuda(), 80, 0.5, qg.CM_FS,
                             batch=1, save_every=8, save_nodes=m.ado_count,
                             precision=precision, variant=variant)
        out.append(r['state'][0].cpu().numpy())
        assert rel_err(out[-1], ref) < tol, variant
