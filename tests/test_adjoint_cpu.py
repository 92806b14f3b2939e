"""Differentiable Redfield 'eg' generator of the adjoint path (CPU, torch)."""
import numpy as np
import torch

import oracle as orc
from conftest import rel_err
from qspectra_gb300 import workloads as wl
from qspectra_gb300.simulate.adjoint import (DebyeCorr, _debye_unit,
                                             eg_heisenberg_generator,
                                             rk4_step_minus_identity)


def test_debye_unit_matches_oracle_and_derivative():
    T, lam, gam = orc.CM_K * 77, 35.0, 106.0
    bath = orc.DebyeBathSpec(T, lam, gam)
    x = torch.tensor([-900.0, -250.5, -3.0, 0.0, 1e-3, 40.0, 600.0], dtype=torch.float64)
    val, der = _debye_unit(x, T, gam, 1000)
    ref = np.array([bath.corr_complex(v) for v in x.numpy()])
    assert rel_err(lam * val.numpy(), ref) < 1e-13
    h = 1e-4
    for i, v in enumerate(x.numpy()):
        if v == 0:
            continue
        fd = (bath.corr_complex(v + h) - bath.corr_complex(v - h)) / (2 * h)
        assert abs(lam * der[i].item() - fd) < 1e-7 * max(1, abs(fd))


def test_debye_autograd_function_gradients():
    T, gam = orc.CM_K * 300, 100.0
    x = torch.tensor([-120.0, 33.0, 410.0], dtype=torch.float64, requires_grad=True)
    lam = torch.tensor(40.0, dtype=torch.float64, requires_grad=True)
    w = torch.tensor([0.3 - 0.2j, -1.1 + 0.5j, 0.7 + 0.9j], dtype=torch.complex128)
    f = lambda x_, l_: (w * DebyeCorr.apply(x_, l_, T, gam, 1000)).real.sum()  # noqa: E731
    f(x, lam).backward()
    h = 1e-5
    for i in range(3):
        e = torch.zeros(3, dtype=torch.float64)
        e[i] = h
        fd = (f(x.detach() + e, lam.detach()) - f(x.detach() - e, lam.detach())) / (2 * h)
        assert abs(x.grad[i].item() - fd.item()) < 1e-7 * max(1, abs(fd.item()))
    fd = (f(x.detach(), lam.detach() + h) - f(x.detach(), lam.detach() - h)) / (2 * h)
    assert abs(lam.grad.item() - fd.item()) < 1e-8 * max(1, abs(fd.item()))


def test_eg_generator_matches_dense_oracle_block():
    H1 = wl.fmo7_hamiltonian()
    bath = orc.DebyeBathSpec(orc.CM_K * 77, 35, 106)
    oham = orc.ElectronicHamiltonianSpec(H1, dipoles=[[1, 0, 0]] * 7, bath=bath)
    om = orc.RedfieldSpec(oham, bath, 'ge', orc.CM_FS, secular=False)
    LH = om.eom_matrix('eg', heisenberg_picture=True)
    L = eg_heisenberg_generator(torch.as_tensor(H1)[None], torch.tensor(35.0, dtype=torch.float64),
                                orc.CM_K * 77, 106.0, oham.rw_freq, orc.CM_FS,
                                eigh=torch.linalg.eigh)
    assert rel_err(L[0].numpy(), LH) < 1e-12


def test_rk4_step_minus_identity_is_the_rk4_step():
    rng = np.random.RandomState(0)
    L = 0.1 * (rng.randn(7, 7) + 1j * rng.randn(7, 7))
    y = rng.randn(7) + 1j * rng.randn(7)
    D = rk4_step_minus_identity(torch.as_tensor(L), 0.7).numpy()
    step = orc.rk4_step_matrix(L, 0.7)
    assert rel_err(y + D @ y, step(y)) < 1e-14
