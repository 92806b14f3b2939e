"""qsx_rk4_block_mean_noalloc: the ensemble-mean time loop that allocates nothing.

Callers that cannot call cudaMalloc (a plug-in inside a host application that
owns all device memory, an embedded runtime with a fixed budget) use this
entry point instead of qsx_rk4_batched: its partial sums live in a 16 MiB
array built into the library.  These tests call it through the C ABI and
check it against qsx_rk4_batched (caller workspace) on the same inputs, on
two calls in a row because every call shares and re-clears that array.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_err
from qspectra_gb300 import _native

pytestmark = pytest.mark.gpu


def generators(B, M, seed):
    rng = np.random.RandomState(seed)
    A = (rng.randn(B, M, M) + 1j * rng.randn(B, M, M)) * 0.05 / np.sqrt(M)
    return A - 0.025 * np.eye(M)[None]


def noalloc_mean(blk, y0, nsteps, select, K, variant=0, per_sample=False):
    """Fill qsx_rk4_args like the workspace path and call the no-alloc entry.
    Returns (status code, mean, device status word, per-sample outputs)."""
    lib = _native.load()
    B, rows, m = blk.shape
    sel = torch.as_tensor(select, dtype=torch.int32, device='cuda')
    out = torch.empty((nsteps + 1, len(select)), dtype=torch.complex128, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    proj = (torch.empty((B, nsteps + 1, len(select)), dtype=torch.complex128, device='cuda')
            if per_sample else None)
    a = _native.Rk4Args()
    a.precision, a.form, a.m, a.nsteps = _native.QSX_FP32, 0, m, nsteps
    a.batch = B
    a.matrix, a.matrix_stride = blk.data_ptr(), rows * m
    a.y0, a.y0_stride = y0.data_ptr(), 0
    a.save_every = 1
    a.nselect, a.block_k, a.select = len(select), K, sel.data_ptr()
    a.out_mean, a.mean_scale = out.data_ptr(), 1.0 / B
    a.status = status.data_ptr()
    a.variant = variant
    if proj is not None:
        a.out_proj = proj.data_ptr()
    st = lib.qsx_rk4_block_mean_noalloc(ctypes.byref(a),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, out, status, proj


@pytest.mark.parametrize('B,M,K,nsteps', [(37, 49, 9, 54),
                                          (700, 49, 9, 999),   # grid shrinks to fit
                                          (20, 16, 4, 40)])
def test_noalloc_matches_workspace_entry(B, M, K, nsteps):
    L = torch.as_tensor(generators(B, M, seed=B + M)).cuda()
    D = _native.rk4_propagator(L, 1.0, _native.QSX_FP32)
    select = list(range(0, M, max(1, M // 7)))[:7]
    blk = _native.rk4_block_matrix(D, K, select)
    y0 = torch.zeros(M, dtype=torch.complex128, device='cuda')
    y0[0] = 1.0
    ref = _native.rk4(blk, y0, nsteps, 1, select=select, per_sample=False, mean=True,
                      block_k=K)['mean'].cpu().numpy()
    for _ in range(2):
        st, out, status, _ = noalloc_mean(blk, y0, nsteps, select, K)
        torch.cuda.synchronize()
        assert st == 0, _native.load().qsx_last_error_string()
        assert int(status.item()) == 0
        assert rel_err(out.cpu().numpy(), ref) < 1e-12


def test_noalloc_rejects_oversized_request():
    M, K = 9, 9
    L = torch.as_tensor(generators(1, M, seed=1)).cuda()
    blk = _native.rk4_block_matrix(_native.rk4_propagator(L, 1.0, _native.QSX_FP32), K,
                                   list(range(7)))
    y0 = torch.ones(M, dtype=torch.complex128, device='cuda')
    st, _, _, _ = noalloc_mean(blk, y0, 150003, list(range(7)), K)
    assert st == 1
    assert b'built-in scratch' in _native.load().qsx_last_error_string()


@pytest.mark.parametrize('variant', [1, 2, 3, 4, 5])
def test_noalloc_kernel_variants_and_per_sample_outputs(variant):
    """Every blocked-loop variant an autotuner may pass, with the per-sample
    outputs (out_proj) requested beside the mean, on a batch large enough
    that the grid shrinks to fit the built-in array."""
    B, M, K, nsteps = 600, 49, 9, 999
    L = torch.as_tensor(generators(B, M, seed=variant)).cuda()
    D = _native.rk4_propagator(L, 1.0, _native.QSX_FP32)
    select = [0, 8, 16, 24, 32, 40, 48]
    blk = _native.rk4_block_matrix(D, K, select)
    y0 = torch.zeros(M, dtype=torch.complex128, device='cuda')
    y0[0] = 1.0
    try:
        ref = _native.rk4(blk, y0, nsteps, 1, select=select, per_sample=True, mean=True,
                          block_k=K, variant=variant)
    except _native.QsxError as e:
        pytest.skip('variant {} does not launch for this shape: {}'.format(variant, e))
    for _ in range(2):
        st, out, status, proj = noalloc_mean(blk, y0, nsteps, select, K, variant=variant,
                                             per_sample=True)
        torch.cuda.synchronize()
        assert st == 0, _native.load().qsx_last_error_string()
        assert int(status.item()) == 0
        assert rel_err(out.cpu().numpy(), ref['mean'].cpu().numpy()) < 1e-12
        assert rel_err(proj.cpu().numpy(), ref['proj'].cpu().numpy()) < 1e-12


@pytest.mark.parametrize('select', [[0, 3, 3, 5],      # repeated entry
                                    [0, 3, 16, 5],     # entry past the state
                                    [-1, 3, 4, 5]])    # negative entry
def test_noalloc_flags_bad_select_table(select):
    """The kernel checks the select table before using it: a bad table sets
    QSX_ERR_INVALID_ARG in the status word and no output is formed from it."""
    B, M, K, nsteps = 8, 16, 4, 40
    L = torch.as_tensor(generators(B, M, seed=3)).cuda()
    D = _native.rk4_propagator(L, 1.0, _native.QSX_FP32)
    blk = _native.rk4_block_matrix(D, K, [0, 1, 2, 3])
    y0 = torch.zeros(M, dtype=torch.complex128, device='cuda')
    y0[0] = 1.0
    st, out, status, _ = noalloc_mean(blk, y0, nsteps, select, K)
    torch.cuda.synchronize()
    assert st == 0
    assert int(status.item()) & _native.QSX_ERR_INVALID_ARG
