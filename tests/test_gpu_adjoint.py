"""Adjoint gradients of the disorder-averaged absorption misfit (GPU).

The hand-written adjoint (qsx_rk4_adjoint_batched behind ProjectedMeanRK4)
is checked against torch autograd through an explicit FP64 RK4 loop and
against central finite differences of the forward path; the forward path
itself is checked against absorption_spectra and the dense CUDA build.
"""
import numpy as np
import pytest
import torch

import qspectra_gb300 as qg
from conftest import rel_err
from qspectra_gb300 import _native
from qspectra_gb300 import workloads as wl
from qspectra_gb300.simulate.adjoint import AbsorptionFit, ProjectedMeanRK4

pytestmark = pytest.mark.gpu


def fmo7_fit(S, nsteps=2047, nf=1024, seed=1):
    H7 = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H7, 1.0, qg.CM_FS)
    bath = qg.DebyeBath(qg.CM_K * 77, 35, 106)
    ham = qg.ElectronicHamiltonian(H7, bath=bath, dipoles=[[1, 0, 0]] * 7,
                                   disorder=wl.fwhm_for_sd(80.0), random_seed=seed,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    freqs = np.linspace(11800.0, 13000.0, nf)
    fit = AbsorptionFit(7, ham.disorder_offsets(S), freqs, rw_freq=m.rw_freq, dt=1.0,
                        nsteps=nsteps)
    return m, fit, fit.pack(H7, 35.0)


def test_forward_matches_absorption_spectra():
    S = 8
    m, fit, theta = fmo7_fit(S)
    assert m.time_step == 1.0
    f, X = qg.absorption_spectra(m, 2048.0, ensemble_size=S, freqs=fit.freqs,
                                 precision='fp64')
    spec = fit.spectrum(theta).cpu().numpy()
    assert rel_err(spec, X) < 1e-10


def test_generator_matches_cuda_build():
    S = 5
    m, fit, theta = fmo7_fit(S)
    from qspectra_gb300.simulate.ensemble import SampleBatch
    batch = SampleBatch(m, S)
    build = m.build_batch(batch.H('ge'))
    L = build.block(m.liouville_subspace_index('eg'), transpose=True)
    assert rel_err(fit.generator(theta).detach().cpu().numpy(), L.cpu().numpy()) < 1e-12


def test_adjoint_kernel_matches_autograd_loop():
    """ProjectedMeanRK4's backward vs autograd through the same loop in torch."""
    rng = np.random.RandomState(3)
    S, m, N = 6, 7, 300
    D0 = 0.02 * (rng.randn(S, m, m) + 1j * rng.randn(S, m, m))
    y0 = torch.as_tensor(rng.randn(m) + 1j * rng.randn(m)).cuda()
    c = torch.as_tensor(rng.randn(m) + 1j * rng.randn(m)).cuda()
    g = torch.as_tensor(rng.randn(N + 1) + 1j * rng.randn(N + 1)).cuda()
    for K in (1, 7, 64, 400):
        D = torch.as_tensor(D0).cuda().requires_grad_(True)
        x = ProjectedMeanRK4.apply(D, y0, c, N, K)
        (x * g.conj()).real.sum().backward()
        D2 = torch.as_tensor(D0).cuda().requires_grad_(True)
        y = y0.expand(S, m)
        out = [y @ c]
        for _ in range(N):
            y = y + (D2 @ y[..., None])[..., 0]
            out.append(y @ c)
        x2 = torch.stack(out, 1).mean(0)
        assert rel_err(x.detach().cpu().numpy(), x2.detach().cpu().numpy()) < 1e-12
        (x2 * g.conj()).real.sum().backward()
        assert rel_err(D.grad.cpu().numpy(), D2.grad.cpu().numpy()) < 1e-11


def test_gradient_matches_autograd_reference_and_fd():
    S = 16
    m, fit, theta_true = fmo7_fit(S)
    target = fit.spectrum(theta_true).detach()
    rng = np.random.RandomState(7)
    theta0 = theta_true.clone()
    theta0[:7] += torch.as_tensor(rng.randn(7) * 10.0).cuda()
    theta0[7:-1] += torch.as_tensor(rng.randn(21) * 5.0).cuda()
    theta0[-1] += 4.0
    th = theta0.clone().requires_grad_(True)
    fit.misfit(th, target).backward()
    g_adj = th.grad.detach().cpu().numpy()
    th2 = theta0.clone().requires_grad_(True)
    fit.misfit(th2, target, impl='autograd').backward()
    g_ref = th2.grad.detach().cpu().numpy()
    assert rel_err(g_adj, g_ref) < 1e-9
    h = 1e-3
    fd = np.zeros_like(g_adj)
    with torch.no_grad():
        for i in range(len(fd)):
            e = torch.zeros_like(theta0)
            e[i] = h
            fd[i] = ((fit.misfit(theta0 + e, target) - fit.misfit(theta0 - e, target))
                     / (2 * h)).item()
    assert rel_err(g_adj, fd) < 1e-5


def test_adjoint_checkpoint_validation():
    D = torch.zeros((2, 3, 3), dtype=torch.complex128, device='cuda')
    ck = torch.zeros((2, 2, 3), dtype=torch.complex128, device='cuda')
    c = torch.ones(3, dtype=torch.complex128, device='cuda')
    g = torch.ones(21, dtype=torch.complex128, device='cuda')
    with pytest.raises(_native.QsxError):
        _native.rk4_adjoint(D, ck, 4, 20, c, g, 0.5)  # 2 checkpoints x 4 < 20 steps


def test_symmetric_eigh_backward_matches_torch():
    """Jacobi eigensolver + analytic backward against torch.linalg.eigh on a
    sign-invariant function of the eigenpairs."""
    from qspectra_gb300.simulate.adjoint import SymmetricEigh
    rng = np.random.RandomState(5)
    A0 = rng.randn(6, 7, 7) * 40
    A0 = A0 + A0.transpose(0, 2, 1)
    wE = torch.as_tensor(rng.randn(6, 7)).cuda()
    R = torch.as_tensor(rng.randn(6, 7, 7)).cuda()

    def f(E, U):
        return (E * wE).sum() + ((U * U) * R).sum()

    A1 = torch.as_tensor(A0).cuda().requires_grad_(True)
    f(*SymmetricEigh.apply(A1)).backward()
    A2 = torch.as_tensor(A0).cuda().requires_grad_(True)
    f(*torch.linalg.eigh(A2)).backward()
    g2 = 0.5 * (A2.grad + A2.grad.transpose(1, 2))
    assert rel_err(A1.grad.cpu().numpy(), g2.cpu().numpy()) < 1e-10
