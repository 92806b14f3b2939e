"""Batched dense products (qsx_gemm_batched): the tensor-core 3xTF32 form
(FP32) and the CUDA-core FP64 form against FP64 torch products, for every
operand combination, shared operands, accumulation and ragged sizes."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from qspectra_gb300 import _native

pytestmark = pytest.mark.gpu


def rand(shape, cplx, rng):
    x = rng.randn(*shape)
    if cplx:
        x = x + 1j * rng.randn(*shape)
    return x


@pytest.mark.parametrize('ca,cb', [(False, False), (True, True), (True, False), (False, True)])
@pytest.mark.parametrize('S,M,K,N', [(3, 128, 64, 128), (2, 276, 276, 300), (4, 7, 33, 5),
                                     (2, 130, 576, 129)])
@pytest.mark.parametrize('single', [True, False])
def test_gemm_matches_fp64_product(ca, cb, S, M, K, N, single):
    rng = np.random.RandomState(M + K + N)
    A = rand((S, M, K), ca, rng)
    B = rand((S, K, N), cb, rng)
    C0 = rand((S, M, N), ca or cb, rng)
    ref = A @ B
    dt = {(True, True): torch.complex64, (True, False): torch.float32,
          (False, True): torch.complex128, (False, False): torch.float64}
    At = torch.as_tensor(A).to(dt[(single, ca)]).cuda()
    Bt = torch.as_tensor(B).to(dt[(single, cb)]).cuda()
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    out = _native.gemm(At, Bt, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    # 3xTF32 drops the lo*lo term (about 2^-22 of each product) and sums in
    # FP32: a few 1e-6 relative at K = 576 (FP32-level accuracy)
    tol = 1e-5 if single else 1e-13
    assert rel_err(out.cpu().numpy(), ref) < tol
    # accumulate in place: out = 0.5 A B + 2 C0
    Ct = torch.as_tensor(C0).to(out.dtype).cuda()
    _native.gemm(At, Bt, out=Ct, Cin=Ct, alpha=0.5, beta=2.0, status=status)
    assert rel_err(Ct.cpu().numpy(), 0.5 * ref + 2 * C0) < tol


@pytest.mark.parametrize('single', [True, False])
def test_gemm_shared_operand(single):
    rng = np.random.RandomState(9)
    A = rand((5, 64, 96), True, rng)
    B = rand((96, 40), True, rng)
    dt = torch.complex64 if single else torch.complex128
    out = _native.gemm(torch.as_tensor(A).to(dt).cuda(), torch.as_tensor(B).to(dt).cuda())
    assert rel_err(out.cpu().numpy(), A @ B) < (1e-5 if single else 1e-13)
    out = _native.gemm(torch.as_tensor(B.T.copy()).to(dt).cuda(),
                       torch.as_tensor(A.transpose(0, 2, 1).copy()).to(dt).cuda())
    assert rel_err(out.cpu().numpy(), B.T @ A.transpose(0, 2, 1)) < (1e-5 if single else 1e-13)
