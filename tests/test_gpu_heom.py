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
    against the per-stage kernels, on every generator case, both pictures,
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
    for variant in (0, 1):
        out.append(_native.heom_rk4(tb, Hb, Hb, y0, 60, 0.5, qg.CM_FS, batch=S, save_every=6,
                                    save_nodes=m.ado_count, precision=precision,
                                    variant=variant)['state'].cpu().numpy())
    assert rel_err(out[0], out[1]) < tol
