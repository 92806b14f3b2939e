"""ctypes binding of the qsx C ABI (include/qsx.h) plus thin torch wrappers.

Every wrapper takes CUDA tensors, checks dtype/shape/contiguity, launches on
torch's current stream and returns CUDA tensors.  There is no CPU fallback:
if the library is not built or no GPU is present the call raises.
"""
import ctypes
import os

import numpy as np
import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'libqsx.so')

QSX_FP64 = 0
QSX_FP32 = 1
# status-word bits set by the kernels (the QSX_ERR_* codes of include/qsx.h)
QSX_ERR_INVALID_ARG = 1
QSX_ZOFE_RHO_HERMIT = 1
QSX_ZOFE_HAM_HERMIT = 2
QSX_ERR_CUDA = 2
QSX_ERR_NONFINITE = 4

_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_dbl = ctypes.c_double
_c_vp = ctypes.c_void_p


class QsxError(RuntimeError):
    """A non-zero status returned by the qsx library."""


class IntegratorError(QsxError):
    """Non-finite state during integration (cf. simulate/utils.py:12-13)."""


class Rk4Args(ctypes.Structure):
    _fields_ = [
        ('precision', ctypes.c_int32), ('form', ctypes.c_int32),
        ('m', ctypes.c_int32), ('nsteps', ctypes.c_int32),
        ('batch', ctypes.c_int64),
        ('matrix', _c_vp), ('matrix_stride', ctypes.c_int64),
        ('h', ctypes.c_double),
        ('y0', _c_vp), ('y0_stride', ctypes.c_int64),
        ('save_every', ctypes.c_int32), ('nproj', ctypes.c_int32),
        ('proj', _c_vp), ('proj_stride', ctypes.c_int64),
        ('nselect', ctypes.c_int32), ('block_k', ctypes.c_int32),
        ('select', _c_vp),
        ('out_state', _c_vp), ('out_proj', _c_vp), ('out_mean', _c_vp),
        ('mean_scale', ctypes.c_double),
        ('workspace', _c_vp), ('workspace_bytes', ctypes.c_size_t),
        ('status', _c_vp),
        ('variant', ctypes.c_int32), ('reserved', ctypes.c_int32),
    ]


class HeomArgs(ctypes.Structure):
    _fields_ = [
        ('precision', ctypes.c_int32), ('nx', ctypes.c_int32), ('ny', ctypes.c_int32),
        ('nnodes', ctypes.c_int32), ('nterms', ctypes.c_int32), ('n_sites', ctypes.c_int32),
        ('nsteps', ctypes.c_int32), ('save_every', ctypes.c_int32),
        ('save_nodes', ctypes.c_int32), ('variant', ctypes.c_int32),
        ('batch', ctypes.c_int64), ('H_stride', ctypes.c_int64),
        ('Hx', _c_vp), ('Hy', _c_vp), ('occx', _c_vp), ('occy', _c_vp), ('W', _c_vp),
        ('shift', _c_vp), ('nbr', _c_vp), ('site', _c_vp), ('alpha', _c_vp), ('beta', _c_vp),
        ('unit_convert', ctypes.c_double), ('h', ctypes.c_double),
        ('y0', _c_vp), ('y0_stride', ctypes.c_int64),
        ('out_state', _c_vp), ('out_mean', _c_vp),
        ('workspace', _c_vp), ('workspace_bytes', ctypes.c_size_t),
        ('status', _c_vp), ('gamma', _c_vp), ('Wraw', _c_vp),
    ]


class ZofeArgs(ctypes.Structure):
    _fields_ = [
        ('precision', ctypes.c_int32), ('n', ctypes.c_int32), ('n_sites', ctypes.c_int32),
        ('npm', ctypes.c_int32), ('nsteps', ctypes.c_int32), ('save_every', ctypes.c_int32),
        ('npulses', ctypes.c_int32), ('nproj', ctypes.c_int32), ('mode', ctypes.c_int32),
        ('cluster', ctypes.c_int32), ('batch', ctypes.c_int64),
        ('H', _c_vp), ('H_stride', ctypes.c_int64), ('Ld', _c_vp), ('Gamma', _c_vp),
        ('w', _c_vp), ('V', _c_vp), ('V_stride', ctypes.c_int64), ('coef', _c_vp),
        ('proj', _c_vp), ('unit_convert', ctypes.c_double), ('h', ctypes.c_double),
        ('y0', _c_vp), ('y0_stride', ctypes.c_int64), ('out_state', _c_vp),
        ('out_proj', _c_vp), ('status', _c_vp), ('hermit', ctypes.c_int32),
        ('save_rho_only', ctypes.c_int32),
    ]


_PROTOS = {
    'qsx_last_error_string': (ctypes.c_char_p, []),
    'qsx_version': (_c_int, []),
    'qsx_debye_corr': (_c_int, [_c_vp, _c_i64, _c_dbl, _c_dbl, _c_dbl, _c_int,
                                _c_int, _c_vp, _c_vp]),
    'qsx_eigh_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_int,
                                  ctypes.POINTER(ctypes.c_int), _c_vp, _c_vp,
                                  _c_vp]),
    'qsx_eigh_batched_prec': (_c_int, [_c_vp, _c_int, _c_i64, _c_int,
                                       ctypes.POINTER(ctypes.c_int), _c_int, _c_vp, _c_vp,
                                       _c_vp]),
    'qsx_redfield_operators_batched': (_c_int, [
        _c_vp, _c_vp, _c_int, _c_i64, _c_vp, _c_int, _c_dbl, _c_dbl, _c_dbl,
        _c_int, _c_int, _c_dbl, _c_int, _c_int, _c_vp, _c_vp, _c_vp, _c_vp]),
    'qsx_redfield_liouvillian_batched': (_c_int, [
        _c_vp, _c_i64, _c_vp, _c_vp, _c_vp, _c_i64, _c_vp, _c_int, _c_int,
        _c_i64, _c_dbl, _c_vp, _c_int, _c_int, _c_int, _c_vp, _c_vp]),
    'qsx_redfield_propagator_batched': (_c_int, [
        _c_vp, _c_i64, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_i64, _c_dbl, _c_vp,
        _c_int, _c_int, _c_dbl, _c_int, _c_vp, _c_vp]),
    'qsx_rk4_block_matrix_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_int,
                                              _c_vp, _c_int, _c_vp, _c_vp]),
    'qsx_hermitian_real_form': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_vp, _c_vp]),
    'qsx_hermitian_rows': (_c_int, [_c_vp, _c_int, _c_i64, _c_i64, _c_int, _c_int, _c_vp,
                                    _c_vp]),
    'qsx_rk4_proj_block_build': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_vp, _c_int, _c_vp,
                                          _c_vp]),
    'qsx_rk4_proj_block_workspace_bytes': (ctypes.c_size_t, [_c_int, _c_i64, _c_int, _c_int,
                                                             _c_int]),
    'qsx_rk4_proj_block_mean': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_int, _c_vp, _c_i64,
                                         _c_int, _c_vp, _c_vp, ctypes.c_size_t, _c_vp, _c_vp]),
    'qsx_redfield_propagator_hermitian_batched': (_c_int, [
        _c_vp, _c_i64, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_i64, _c_dbl, _c_vp,
        _c_int, _c_vp, _c_dbl, _c_int, _c_vp, _c_vp]),
    'qsx_rk4_block_matrix_real_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_int,
                                                   _c_vp, _c_int, _c_vp, _c_vp]),
    'qsx_rk4_block_matrix_real_tc_supported': (_c_int, [_c_int, _c_int, _c_int]),
    'qsx_rk4_block_matrix_real_tc': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_vp, _c_int,
                                              _c_vp, _c_vp, _c_vp]),
    'qsx_rk4_real_block_workspace_bytes': (ctypes.c_size_t, [_c_int, _c_i64, _c_int, _c_int,
                                                             _c_int, _c_int]),
    'qsx_rk4_real_block_mean': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_int, _c_vp, _c_i64,
                                         _c_vp, _c_int, _c_int, _c_vp, _c_vp, ctypes.c_size_t,
                                         _c_vp, _c_vp]),
    'qsx_rk4_propagator_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_dbl,
                                            _c_int, _c_vp, _c_vp]),
    'qsx_rk4_args_bytes': (ctypes.c_size_t, []),
    'qsx_rk4_workspace_bytes': (_c_int, [ctypes.POINTER(Rk4Args),
                                         ctypes.POINTER(ctypes.c_size_t)]),
    'qsx_rk4_batched': (_c_int, [ctypes.POINTER(Rk4Args), _c_vp]),
    'qsx_rk4_block_mean_noalloc': (_c_int, [ctypes.POINTER(Rk4Args), _c_vp]),
    'qsx_heom_args_bytes': (ctypes.c_size_t, []),
    'qsx_zofe_args_bytes': (ctypes.c_size_t, []),
    'qsx_zofe_rk4': (_c_int, [ctypes.POINTER(ZofeArgs), _c_vp]),
    'qsx_heom_workspace_bytes': (_c_int, [ctypes.POINTER(HeomArgs),
                                          ctypes.POINTER(ctypes.c_size_t)]),
    'qsx_heom_rhs': (_c_int, [ctypes.POINTER(HeomArgs), _c_vp, _c_vp, _c_vp]),
    'qsx_heom_rk4': (_c_int, [ctypes.POINTER(HeomArgs), _c_vp]),
    'qsx_redfield_build_w64': (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_i64, _c_vp, _c_dbl,
                                        _c_dbl, _c_dbl, _c_int, _c_int, _c_vp, _c_int, _c_dbl,
                                        _c_dbl, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    'qsx_redfield_operators_w32': (_c_int, [_c_vp, _c_vp, _c_int, _c_int, _c_int, _c_i64,
                                            _c_dbl, _c_dbl, _c_dbl, _c_int, _c_int, _c_dbl,
                                            _c_vp, _c_vp, _c_vp]),
    'qsx_debye_matsubara_table': (_c_int, [_c_dbl, _c_dbl, _c_int, _c_int, _c_dbl, _c_vp]),
    'qsx_debye_matsubara_table_degree': (_c_int, []),
    'qsx_disordered_hamiltonians': (_c_int, [_c_vp, _c_int, _c_vp, _c_i64, _c_int, _c_int,
                                             _c_vp, _c_vp]),
    'qsx_gemm_batched': (_c_int, [_c_int, _c_int, _c_i64, _c_int, _c_int, _c_int, _c_vp,
                                  _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64,
                                  _c_dbl, _c_vp, _c_i64, _c_i64, _c_dbl, _c_vp, _c_vp]),
    'qsx_dft_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_dbl, _c_dbl, _c_vp,
                                 _c_int, _c_dbl, _c_dbl, _c_int, _c_vp, _c_vp]),
    'qsx_dft_batched_f32': (_c_int, [_c_vp, _c_int, _c_i64, _c_dbl, _c_dbl, _c_vp,
                                     _c_int, _c_dbl, _c_dbl, _c_int, _c_vp, _c_vp]),
    'qsx_dft2_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_i64, _c_i64, _c_i64,
                                  _c_dbl, _c_dbl, _c_vp, _c_int, _c_int, _c_dbl, _c_dbl, _c_vp,
                                  _c_int, _c_int, _c_dbl, _c_dbl, _c_vp, _c_vp]),
    'qsx_fblock_tensor': (_c_int, [_c_vp, _c_vp, _c_int, _c_int, _c_vp, _c_i64, _c_dbl,
                                   _c_dbl, _c_dbl, _c_int, _c_int, _c_dbl, _c_int,
                                   _c_vp, _c_vp]),
    'qsx_fe_generator': (_c_int, [_c_vp, _c_vp, _c_int, _c_int, _c_i64, _c_vp, _c_dbl,
                                  _c_int, _c_vp, _c_vp]),
    'qsx_fe_heisenberg_workspace_bytes': (ctypes.c_size_t, [_c_int, _c_int, _c_i64,
                                                            _c_int]),
    'qsx_fe_heisenberg_rk4': (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_i64,
                                       _c_int, _c_vp, _c_i64, _c_int, _c_dbl, _c_vp,
                                       _c_vp, ctypes.c_size_t, _c_vp, _c_vp]),
    'qsx_csr_map_batched': (_c_int, [_c_vp, _c_i64, _c_i64, _c_vp, _c_vp, _c_vp, _c_int,
                                     _c_vp, _c_vp]),
    'qsx_rk4_field_batched': (_c_int, [_c_vp, _c_i64, _c_vp, _c_i64, _c_int, _c_vp, _c_int,
                                       _c_i64,
                                       _c_int, _c_dbl, _c_vp, _c_i64, _c_int, _c_int, _c_vp,
                                       _c_vp, _c_vp]),
    'qsx_eigh_large_workspace_bytes': (ctypes.c_size_t, [_c_int, _c_i64]),
    'qsx_eigh_large_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_vp, _c_vp, _c_vp,
                                        ctypes.c_size_t, _c_vp, _c_vp]),
    'qsx_rk4_adjoint_batched': (_c_int, [_c_vp, _c_int, _c_i64, _c_int, _c_vp, _c_int,
                                         _c_int, _c_vp, _c_vp, _c_dbl, _c_vp, _c_vp, _c_vp]),
}

_LIB = None


def exported_symbols():
    """Names the header declares (for the ABI test)."""
    return sorted(_PROTOS)


def load(path=LIB_PATH):
    """Load libqsx.so and attach prototypes (no GPU needed)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise QsxError(
                'qsx CUDA library not found at {}; build it with '
                '`python -m qspectra_gb300.build`'.format(path))
        lib = ctypes.CDLL(path)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def _check(status, what):
    if status != 0:
        msg = load().qsx_last_error_string().decode(errors='replace')
        raise QsxError('{} failed (status {}): {}'.format(what, status, msg))


def _stream():
    return _c_vp(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return None if t is None else _c_vp(t.data_ptr())


def _need(t, dtype, name, ndim=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError('{} must be a CUDA tensor'.format(name))
    if t.dtype != dtype:
        raise ValueError('{} must be {} (got {})'.format(name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError('{} must be contiguous'.format(name))
    if ndim is not None and t.dim() != ndim:
        raise ValueError('{} must have {} dims'.format(name, ndim))
    return t


def require_gpu():
    if not torch.cuda.is_available():
        raise QsxError('qspectra_gb300 needs a CUDA GPU; none is visible')
    load()


# --------------------------------------------------------------- wrappers
def debye_corr(x, temperature, reorg_energy, cutoff_freq, matsubara_cutoff=1000,
               real_only=False):
    require_gpu()
    x = _need(x.contiguous(), torch.float64, 'x')
    out = torch.empty(x.shape, dtype=torch.complex128, device=x.device)
    _check(load().qsx_debye_corr(_p(x), x.numel(), temperature, reorg_energy,
                                 cutoff_freq, matsubara_cutoff, int(real_only),
                                 _p(out), _stream()), 'qsx_debye_corr')
    return out


def eigh(H, block_starts, precision=QSX_FP64):
    """Batched Jacobi eigensolver; H (B, n, n) float64 CUDA.  precision
    QSX_FP32 runs blocks of up to 8 states in FP32."""
    require_gpu()
    _need(H, torch.float64, 'H', 3)
    B, n, _ = H.shape
    E = torch.empty((B, n), dtype=torch.float64, device=H.device)
    U = torch.empty((B, n, n), dtype=torch.float64, device=H.device)
    blk = (ctypes.c_int * len(block_starts))(*[int(v) for v in block_starts])
    _check(load().qsx_eigh_batched_prec(_p(H), n, B, len(block_starts) - 1, blk,
                                        int(precision), _p(E), _p(U), _stream()),
           'qsx_eigh_batched')
    return E, U


def redfield_operators(E, U, occ, bath, unit_convert, discard_imag_corr=False,
                       site_basis=True, matsubara_cutoff=1000, precision=QSX_FP64):
    require_gpu()
    _need(E, torch.float64, 'E', 2)
    _need(U, torch.float64, 'U', 3)
    _need(occ, torch.float64, 'occ', 2)
    B, n = E.shape
    N = occ.shape[0]
    dev = E.device
    G = torch.empty((B, n, n), dtype=torch.complex128, device=dev)
    M = torch.empty((B, N, n, n), dtype=torch.complex128, device=dev)
    K = None if site_basis else torch.empty((B, N, n, n), dtype=torch.float64,
                                            device=dev)
    _check(load().qsx_redfield_operators_batched(
        _p(E), _p(U), n, B, _p(occ), N, bath.temperature, bath.reorg_energy,
        bath.cutoff_freq, matsubara_cutoff, int(discard_imag_corr), unit_convert,
        int(site_basis), int(precision), _p(G), _p(M), _p(K), _stream()),
        'qsx_redfield_operators_batched')
    return G, M, K


def redfield_operators_w32(E, U, n_sites, off, bath, unit_convert, discard_imag_corr=False,
                           matsubara_cutoff=1000):
    """FP32 site-basis operators G, M of a one-exciton Hilbert space, one
    warp per sample (qsx_redfield_operators_w32); E (B, n), U (B, n, n)
    float64 from the FP32 eigensolve; the coupled block is [off, off +
    n_sites)."""
    require_gpu()
    _need(E, torch.float64, 'E', 2)
    _need(U, torch.float64, 'U', 3)
    B, n = E.shape
    dev = E.device
    G = torch.empty((B, n, n), dtype=torch.complex128, device=dev)
    M = torch.empty((B, n_sites, n, n), dtype=torch.complex128, device=dev)
    _check(load().qsx_redfield_operators_w32(
        _p(E), _p(U), n, off, n_sites, B, bath.temperature, bath.reorg_energy,
        bath.cutoff_freq, matsubara_cutoff, int(discard_imag_corr), unit_convert, _p(G),
        _p(M), _stream()), 'qsx_redfield_operators_w32')
    return G, M


def disordered_hamiltonians(base, offsets, off):
    """(S, n, n) float64: base (n, n) plus diag(offsets[s]) on rows/columns
    off .. off + n_sites - 1 (qsx_disordered_hamiltonians)."""
    require_gpu()
    _need(base, torch.float64, 'base', 2)
    _need(offsets, torch.float64, 'offsets', 2)
    n = base.shape[0]
    S, N = offsets.shape
    H = torch.empty((S, n, n), dtype=torch.float64, device=base.device)
    _check(load().qsx_disordered_hamiltonians(_p(base), n, _p(offsets), S, N, off, _p(H),
                                              _stream()), 'qsx_disordered_hamiltonians')
    return H


def gemm(A, B, out=None, Cin=None, alpha=1.0, beta=1.0, status=None):
    """Batched out = alpha A B (+ beta Cin) on the GPU (qsx_gemm_batched): FP32
    operands on the tensor cores (3xTF32), FP64 on the CUDA cores.

    A (S, M, K) and B (S, K, N), either of them 2-D to share it across the
    batch; real or complex of one precision (float32/complex64 or
    float64/complex128); the result is complex when either operand is.  The
    last dimension of every operand must be contiguous.  ``out`` must not
    overlap A or B; Cin may be ``out`` itself."""
    require_gpu()
    if A.dim() not in (2, 3) or B.dim() not in (2, 3):
        raise ValueError('gemm operands must be 2-D or 3-D')
    single = A.dtype in (torch.float32, torch.complex64)
    if single != (B.dtype in (torch.float32, torch.complex64)):
        raise TypeError('gemm operands must share one precision')
    ca, cb = A.is_complex(), B.is_complex()
    mode = {(False, False): 0, (True, True): 1, (True, False): 2, (False, True): 3}[(ca, cb)]
    for t in (A, B):
        if t.shape[-1] > 1 and t.stride(-1) != 1:
            raise ValueError('gemm operands need a contiguous last dimension')
    S = max(A.shape[0] if A.dim() == 3 else 1, B.shape[0] if B.dim() == 3 else 1)
    M, K = A.shape[-2], A.shape[-1]
    if B.shape[-2] != K:
        raise ValueError('gemm: inner sizes differ ({} vs {})'.format(K, B.shape[-2]))
    N = B.shape[-1]
    cdt = (torch.complex64 if single else torch.complex128) if (ca or cb) else A.dtype
    if out is None:
        out = torch.empty((S, M, N), dtype=cdt, device=A.device)
    if out.dtype != cdt or out.shape[-2:] != (M, N) or (N > 1 and out.stride(-1) != 1):
        raise ValueError('gemm: bad output tensor')
    sa = A.stride(0) if A.dim() == 3 else 0
    sb = B.stride(0) if B.dim() == 3 else 0
    so = out.stride(0) if out.dim() == 3 else 0
    if Cin is not None:
        if Cin.dtype != cdt or Cin.shape[-2:] != (M, N) or (N > 1 and Cin.stride(-1) != 1):
            raise ValueError('gemm: bad Cin tensor')
        sc, ldc_in = (Cin.stride(0) if Cin.dim() == 3 else 0), Cin.stride(-2)
    else:
        sc, ldc_in, beta = 0, 0, 0.0
    _check(load().qsx_gemm_batched(
        QSX_FP32 if single else QSX_FP64, mode, S, M, N, K,
        _p(A), A.stride(-2), sa, _p(B), B.stride(-2), sb,
        _p(Cin) if Cin is not None else None, ldc_in, sc, float(beta),
        _p(out), out.stride(-2), so, float(alpha),
        _p(status) if status is not None else None, _stream()), 'qsx_gemm_batched')
    return out


_MATSUBARA_TABLES = {}


def matsubara_table(bath, matsubara_cutoff, xmax=4096.0, device=None):
    """(table, pieces, width): the piecewise Chebyshev table of the Debye
    Matsubara sum (qsx_debye_matsubara_table) on [0, xmax], on the GPU,
    computed once per bath.  Pieces are at most 64 cm^-1 wide and at most a
    fifth of the first Matsubara frequency, so every piece's series
    converges to FP64 rounding."""
    T, g = float(bath.temperature), float(bath.cutoff_freq)
    key = (T, g, int(matsubara_cutoff), float(xmax))
    if key not in _MATSUBARA_TABLES:
        width = min(64.0, 0.4 * np.pi * T)   # half-width <= nu_1 / 10
        pieces = int(np.ceil(xmax / width))
        deg = load().qsx_debye_matsubara_table_degree()
        coef = np.zeros((pieces, deg, 2), dtype=np.float64)
        _check(load().qsx_debye_matsubara_table(T, g, int(matsubara_cutoff), pieces, width,
                                                coef.ctypes.data_as(_c_vp)),
               'qsx_debye_matsubara_table')
        dev = device or torch.device('cuda', torch.cuda.current_device())
        _MATSUBARA_TABLES[key] = (torch.as_tensor(coef).to(dev), pieces, width)
    return _MATSUBARA_TABLES[key]


def redfield_build_w64(H, U_approx, n_sites, off, bath, unit_convert, discard_imag_corr=False,
                       matsubara_cutoff=1000):
    """FP64 eigenpairs and site-basis Redfield operators of one-exciton
    Hilbert spaces (qsx_redfield_build_w64): FP64 refinement of the
    approximate eigenvectors U_approx (e.g. the FP32 Jacobi's), then the
    operator build in FP64 with the tabulated correlation function.  H,
    U_approx (B, n, n) float64 CUDA; the coupled block is [off, off +
    n_sites).  Returns E, U, G, M."""
    require_gpu()
    _need(H, torch.float64, 'H', 3)
    _need(U_approx, torch.float64, 'U_approx', 3)
    B, n, _ = H.shape
    dev = H.device
    E = torch.empty((B, n), dtype=torch.float64, device=dev)
    U = torch.empty((B, n, n), dtype=torch.float64, device=dev)
    G = torch.empty((B, n, n), dtype=torch.complex128, device=dev)
    M = torch.empty((B, n_sites, n, n), dtype=torch.complex128, device=dev)
    table, pieces, width = matsubara_table(bath, matsubara_cutoff, device=dev)
    _check(load().qsx_redfield_build_w64(
        _p(H), n, off, n_sites, B, _p(U_approx), bath.temperature, bath.reorg_energy,
        bath.cutoff_freq, matsubara_cutoff, int(discard_imag_corr), _p(table), pieces, width,
        unit_convert, _p(E), _p(U), _p(G), _p(M), _stream()), 'qsx_redfield_build_w64')
    return E, U, G, M


def redfield_liouvillian(H, G, M, idx, unit_convert, K=None, occ=None,
                         secular=False, transpose=False):
    """Dense L[idx, idx] per sample (complex128)."""
    require_gpu()
    _need(G, torch.complex128, 'G', 3)
    _need(M, torch.complex128, 'M', 4)
    B, n, _ = G.shape
    N = M.shape[1]
    H = _need(H, torch.float64, 'H')
    h_stride = 0 if H.dim() == 2 else n * n
    if K is not None:
        _need(K, torch.float64, 'K')
        k_stride = 0 if K.dim() == 3 else N * n * n
    else:
        _need(occ, torch.float64, 'occ', 2)
        k_stride = 0
    idx = _need(idx, torch.int32, 'idx', 1)
    m = idx.numel()
    L = torch.empty((B, m, m), dtype=torch.complex128, device=G.device)
    _check(load().qsx_redfield_liouvillian_batched(
        _p(H), h_stride, _p(G), _p(M), _p(K), k_stride, _p(occ), n, N, B,
        unit_convert, _p(idx), m, int(secular), int(transpose), _p(L),
        _stream()), 'qsx_redfield_liouvillian_batched')
    return L


def redfield_propagator(H, G, M, occ, idx, unit_convert, h, precision=QSX_FP64,
                        transpose=False):
    """Fused site-basis generator block + RK4 propagator; None if it does not fit."""
    require_gpu()
    _need(G, torch.complex128, 'G', 3)
    _need(M, torch.complex128, 'M', 4)
    _need(occ, torch.float64, 'occ', 2)
    B, n, _ = G.shape
    N = M.shape[1]
    H = _need(H, torch.float64, 'H')
    h_stride = 0 if H.dim() == 2 else n * n
    idx = _need(idx, torch.int32, 'idx', 1)
    m = idx.numel()
    dt = torch.complex64 if precision == QSX_FP32 else torch.complex128
    D = torch.empty((B, m, m), dtype=dt, device=G.device)
    st = load().qsx_redfield_propagator_batched(
        _p(H), h_stride, _p(G), _p(M), _p(occ), n, N, B, unit_convert, _p(idx), m,
        int(transpose), h, precision, _p(D), _stream())
    if st == 3:  # QSX_ERR_UNSUPPORTED: too large for shared memory
        return None
    _check(st, 'qsx_redfield_propagator_batched')
    return D


def hermitian_rows(x, n, merge=False):
    """Rows of column-stacked n x n matrices to / from the Hermitian
    coordinates of their Hermitian and anti-Hermitian parts
    (qsx_hermitian_rows): complex (B, R, n^2) -> real (B, 2R, n^2), or back
    with ``merge``."""
    require_gpu()
    x = x.contiguous()
    B, rows, m = x.shape
    if m != n * n:
        raise ValueError('row length must be n^2')
    if merge:
        prec = QSX_FP32 if x.dtype == torch.float32 else QSX_FP64
        if rows % 2:
            raise ValueError('merge needs the split layout (2R rows)')
        rows //= 2
        out = torch.empty((B, rows, m), dtype=torch.complex64 if prec == QSX_FP32
                          else torch.complex128, device=x.device)
    else:
        prec = QSX_FP32 if x.dtype == torch.complex64 else QSX_FP64
        out = torch.empty((B, 2 * rows, m), dtype=torch.float32 if prec == QSX_FP32
                          else torch.float64, device=x.device)
    _check(load().qsx_hermitian_rows(_p(x), n, rows, B, prec, 1 if merge else 0, _p(out),
                                     _stream()), 'qsx_hermitian_rows')
    return out


def hermitian_real_form(A, n):
    """Real form (B, m, m) of complex (B, m, m) Hermiticity-preserving maps on
    n x n matrices (qsx_hermitian_real_form; float32 from complex64)."""
    require_gpu()
    prec = QSX_FP32 if A.dtype == torch.complex64 else QSX_FP64
    A = _need(A.contiguous(), A.dtype, 'A', 3)
    B, m, _ = A.shape
    if m != n * n:
        raise ValueError('matrix size must be n^2')
    R = torch.empty((B, m, m), dtype=torch.float32 if prec == QSX_FP32 else torch.float64,
                    device=A.device)
    _check(load().qsx_hermitian_real_form(_p(A), n, B, prec, _p(R), _stream()),
           'qsx_hermitian_real_form')
    return R


_CONSTS = {}


def const_tensor(values, dtype, device):
    """A small host array as a device tensor, uploaded once and cached by
    content.  Index tables and selections are the same on every call of a
    workload; uploading a pageable host array blocks the host until the
    stream reaches the copy, so repeated uploads would serialise the host's
    launches with the GPU's work."""
    arr = np.ascontiguousarray(values)
    key = (arr.tobytes(), arr.shape, arr.dtype.str, str(dtype), str(device))
    t = _CONSTS.get(key)
    if t is None:
        if len(_CONSTS) > 512:
            _CONSTS.clear()
        t = torch.as_tensor(arr).to(dtype=dtype, device=device).contiguous()
        _CONSTS[key] = t
    return t


_RECIPES = {}


def hermitian_recipe(nb, device):
    """Packed (m^2, 4) int32 map from the sources [Re B, Im B (nb, nb, nb),
    uc H (nb, nb)] to the real form of the Redfield generator block
    L[(a,b),(c,d)] = d_bd (-B[b]_ac - i uc H_ac) + d_ac (-conj(B[a]_bd) + i uc H_db)
    on a diagonal block of nb states (row-major over the m^2 entries)."""
    key = (nb, str(device))
    if key in _RECIPES:
        return _RECIPES[key]
    m = nb * nb
    nsrc = 2 * nb ** 3 + m
    S = np.eye(nsrc)
    Bs = (S[:, :nb ** 3] + 1j * S[:, nb ** 3:2 * nb ** 3]).reshape(nsrc, nb, nb, nb)
    uH = S[:, 2 * nb ** 3:].reshape(nsrc, nb, nb)
    I = np.eye(nb)
    L4 = (np.einsum('bd,nbac->nabcd', I, -Bs) + np.einsum('bd,nac->nabcd', I, -1j * uH)
          + np.einsum('ac,nabd->nabcd', I, -Bs.conj()) + np.einsum('ac,ndb->nabcd', I, 1j * uH))
    L = L4.transpose(0, 2, 1, 4, 3).reshape(nsrc, m, m)      # k = a + nb b, l = c + nb d
    # real form: R[k, l] = coordinate k of L applied to Hermitian basis matrix l
    k = np.arange(m)
    a, b = k % nb, k // nb
    row = np.where(a <= b, a + nb * b, b + nb * a)
    c, d = a, b
    cols_re = np.where(c <= d, c + nb * d, d + nb * c)
    cols_tr = np.where(c <= d, d + nb * c, c + nb * d)
    Lr = L[:, row, :]                                         # (nsrc, m rows k, m)
    V = np.where(c == d, Lr[:, :, k],
                 np.where(c < d, Lr[:, :, cols_re] + Lr[:, :, cols_tr],
                          1j * (Lr[:, :, d + nb * c] - Lr[:, :, c + nb * d])))
    R = np.where((a <= b)[None, :, None], V.real, V.imag)     # (nsrc, m, m)
    J = R.reshape(nsrc, m * m).T                              # (m^2, nsrc)
    rows, cols = np.nonzero(J)
    rowptr = np.zeros(m * m + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    coefs = J[rows, cols]
    if np.diff(rowptr).max(initial=0) > 4 or nsrc > 65535 or np.any(
            np.abs(coefs - np.round(coefs)) > 0) or np.abs(coefs).max(initial=0) > 127:
        raise ValueError('generator recipe does not fit the packed 4-term form')
    # packed per entry: sources (16 bits) in words 0-1, int8 coefficients in word 2
    src = np.zeros((m * m, 4), dtype=np.int64)
    cf = np.zeros((m * m, 4), dtype=np.int64)
    for e in range(m * m):
        k = rowptr[e + 1] - rowptr[e]
        src[e, :k] = cols[rowptr[e]:rowptr[e + 1]]
        cf[e, :k] = np.round(coefs[rowptr[e]:rowptr[e + 1]])
    packed = np.zeros((m * m, 4), dtype=np.int64)
    packed[:, 0] = src[:, 0] | (src[:, 1] << 16)
    packed[:, 1] = src[:, 2] | (src[:, 3] << 16)
    packed[:, 2] = ((cf[:, 0] & 0xff) | ((cf[:, 1] & 0xff) << 8) | ((cf[:, 2] & 0xff) << 16)
                    | ((cf[:, 3] & 0xff) << 24))
    packed = packed.astype(np.uint32).view(np.int32)
    out = torch.as_tensor(np.ascontiguousarray(packed), device=device)
    _RECIPES[key] = out
    return out


def redfield_propagator_hermitian(H, G, M, occ, states, unit_convert, h, precision=QSX_FP32):
    """Real one-step propagator D_r = P_r - I (B, nb^2, nb^2) of the diagonal
    block of Hilbert states ``states`` (qsx_redfield_propagator_hermitian_batched)."""
    require_gpu()
    _need(G, torch.complex128, 'G', 3)
    _need(M, torch.complex128, 'M', 4)
    _need(occ, torch.float64, 'occ', 2)
    B, n, _ = G.shape
    N = M.shape[1]
    H = _need(H, torch.float64, 'H')
    h_stride = 0 if H.dim() == 2 else n * n
    st = const_tensor(np.asarray(states, dtype=np.int32), torch.int32, G.device)
    nb = st.numel()
    recipe = hermitian_recipe(nb, G.device)
    m = nb * nb
    dt = torch.float32 if precision == QSX_FP32 else torch.float64
    D = torch.empty((B, m, m), dtype=dt, device=G.device)
    _check(load().qsx_redfield_propagator_hermitian_batched(
        _p(H), h_stride, _p(G), _p(M), _p(occ), n, N, B, unit_convert, _p(st), nb,
        _p(recipe), h, precision, _p(D), _stream()),
        'qsx_redfield_propagator_hermitian_batched')
    return D


def rk4_block_matrix_real(D, K, select):
    """(B, m + len(select) (K-1), m) real K-step blocked matrix from a real D."""
    require_gpu()
    prec = QSX_FP32 if D.dtype == torch.float32 else QSX_FP64
    _need(D, D.dtype, 'D', 3)
    B, m, _ = D.shape
    sel_np = np.asarray(select, dtype=np.int64).reshape(-1)
    if sel_np.size == 0 or sel_np.min() < 0 or sel_np.max() >= m:
        raise ValueError('select indices must lie in [0, {})'.format(m))
    sel = const_tensor(sel_np.astype(np.int32), torch.int32, D.device)
    rows = m + sel.numel() * (K - 1)
    stride = (rows * m + 3) // 4 * 4   # samples start on 16-byte boundaries
    flat = torch.empty((B, stride), dtype=D.dtype, device=D.device)
    _check(load().qsx_rk4_block_matrix_real_batched(_p(D), m, B, prec, K, _p(sel), sel.numel(),
                                                    _p(flat), _stream()),
           'qsx_rk4_block_matrix_real_batched')
    return flat[:, :rows * m].view(B, rows, m)


def rk4_block_matrix_real_tc_supported(m, K, nselect):
    """Whether the tcgen05 block build takes this shape
    (qsx_rk4_block_matrix_real_tc_supported)."""
    return bool(load().qsx_rk4_block_matrix_real_tc_supported(int(m), int(K), int(nselect)))


def rk4_block_matrix_real_tc(D, K, select):
    """As rk4_block_matrix_real for FP32, on the tensor cores (3xTF32
    tcgen05 products; qsx_rk4_block_matrix_real_tc).  Returns None when the
    shape is not supported."""
    require_gpu()
    _need(D, torch.float32, 'D', 3)
    B, m, _ = D.shape
    sel_np = np.asarray(select, dtype=np.int64).reshape(-1)
    lib = load()
    if not lib.qsx_rk4_block_matrix_real_tc_supported(m, int(K), sel_np.size):
        return None
    sel = const_tensor(sel_np.astype(np.int32), torch.int32, D.device)
    rows = m + sel.numel() * (K - 1)
    stride = (rows * m + 3) // 4 * 4
    flat = torch.empty((B, stride), dtype=torch.float32, device=D.device)
    status = torch.zeros(1, dtype=torch.int32, device=D.device)
    _check(lib.qsx_rk4_block_matrix_real_tc(_p(D), m, B, int(K), _p(sel), sel.numel(), _p(flat),
                                            _p(status), _stream()),
           'qsx_rk4_block_matrix_real_tc')
    return flat[:, :rows * m].view(B, rows, m), status


def rk4_real_block_mean(mat, y0, nsteps, select, K, check_finite=True, group=0):
    """Ensemble mean (nsteps + 1, len(select)) float64 of the selected real
    coordinates (qsx_rk4_real_block_mean).  mat (B, m + nsel (K-1), m)
    float32; y0 (m,) or (B, m) float64."""
    require_gpu()
    if mat.dtype != torch.float32 or mat.dim() != 3 or not mat.is_cuda:
        raise TypeError('mat must be a (B, rows, m) float32 CUDA tensor')
    B, rows, m = mat.shape
    # (a batch of one may report any stride for its size-1 sample dimension)
    if mat.stride(2) != 1 or mat.stride(1) != m or (
            B > 1 and mat.stride(0) != (rows * m + 3) // 4 * 4):
        raise ValueError('mat must use the padded sample layout of rk4_block_matrix_real')
    y0 = y0.to(device=mat.device, dtype=torch.float64).contiguous()
    sel = const_tensor(np.asarray(select, dtype=np.int32), torch.int32, mat.device)
    nsel = sel.numel()
    if rows != m + nsel * (K - 1):
        raise ValueError('matrix rows do not match K and select')
    lib = load()
    ws_bytes = lib.qsx_rk4_real_block_workspace_bytes(m, B, K, int(nsteps), nsel, int(group))
    ws = torch.empty(max(int(ws_bytes), 8), dtype=torch.uint8, device=mat.device)
    out = torch.empty((nsteps + 1, nsel), dtype=torch.float64, device=mat.device)
    status = torch.zeros(1, dtype=torch.int32, device=mat.device)
    _check(lib.qsx_rk4_real_block_mean(_p(mat), m, B, K, int(nsteps), _p(y0),
                                       m if y0.dim() == 2 else 0, _p(sel), nsel, int(group),
                                       _p(out), _p(ws), ws.numel(), _p(status), _stream()),
           'qsx_rk4_real_block_mean')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state in the blocked real loop')
    return out, status


def proj_block_k(nsteps, m, nproj, max_k=64):
    """Largest K <= max_k dividing nsteps with m + nproj K <= 256 (1: none)."""
    for K in range(min(max_k, (256 - m) // nproj), 1, -1):
        if nsteps % K == 0:
            return K
    return 1


def rk4_proj_block_mean(D, y0, proj, nsteps, K, check_finite=True):
    """Ensemble mean (nsteps + 1, nproj) complex128 of proj . y_n for
    y_{n+1} = (I + D) y_n (qsx_rk4_proj_block_build + qsx_rk4_proj_block_mean).
    D (B, m, m) complex64; y0 (m,) or (B, m); proj (nproj, m) shared."""
    require_gpu()
    _need(D, torch.complex64, 'D', 3)
    B, m, _ = D.shape
    proj = proj.to(device=D.device, dtype=torch.complex128).contiguous()
    P = proj.shape[0]
    y0 = y0.to(device=D.device, dtype=torch.complex128).contiguous()
    lib = load()
    mat = torch.empty((B, m + P * K, m), dtype=torch.complex64, device=D.device)
    _check(lib.qsx_rk4_proj_block_build(_p(D), m, B, K, _p(proj), P, _p(mat), _stream()),
           'qsx_rk4_proj_block_build')
    ws_bytes = lib.qsx_rk4_proj_block_workspace_bytes(m, B, K, int(nsteps), P)
    ws = torch.empty(max(int(ws_bytes), 16), dtype=torch.uint8, device=D.device)
    out = torch.empty((nsteps + 1, P), dtype=torch.complex128, device=D.device)
    status = torch.zeros(1, dtype=torch.int32, device=D.device)
    _check(lib.qsx_rk4_proj_block_mean(_p(mat), m, B, K, int(nsteps), _p(y0),
                                       m if y0.dim() == 2 else 0, P, _p(out), _p(ws),
                                       ws.numel(), _p(status), _stream()),
           'qsx_rk4_proj_block_mean')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state in the projected blocked loop')
    return out, status


def rk4_propagator(L, h, precision=QSX_FP64):
    require_gpu()
    _need(L, torch.complex128, 'L', 3)
    B, m, _ = L.shape
    dt = torch.complex64 if precision == QSX_FP32 else torch.complex128
    D = torch.empty((B, m, m), dtype=dt, device=L.device)
    _check(load().qsx_rk4_propagator_batched(_p(L), m, B, h, precision, _p(D),
                                             _stream()),
           'qsx_rk4_propagator_batched')
    return D


def rk4_block_matrix(D, K, select):
    """(B, m + len(select) (K-1), m) K-step blocked matrix from D = P - I."""
    require_gpu()
    prec = QSX_FP32 if D.dtype == torch.complex64 else QSX_FP64
    _need(D, D.dtype, 'D', 3)
    B, m, _ = D.shape
    sel_np = np.asarray(select, dtype=np.int64).reshape(-1)
    if sel_np.size == 0 or sel_np.min() < 0 or sel_np.max() >= m:
        raise ValueError('select indices must lie in [0, {})'.format(m))
    sel = const_tensor(sel_np.astype(np.int32), torch.int32, D.device)
    out = torch.empty((B, m + sel.numel() * (K - 1), m), dtype=D.dtype, device=D.device)
    _check(load().qsx_rk4_block_matrix_batched(_p(D), m, B, prec, K, _p(sel), sel.numel(),
                                               _p(out), _stream()),
           'qsx_rk4_block_matrix_batched')
    return out


def rk4(matrix, y0, nsteps, save_every=1, form=0, h=0.0, precision=None,
        state=False, proj=None, select=None, per_sample=True, mean=False,
        check_finite=True, workspace=None, block_k=0, variant=0):
    """Batched RK4 time loop (see qsx_rk4_args in include/qsx.h).

    matrix: (B, m, m) complex64 (FP32) / complex128 (FP64), or (m, m) shared.
    y0: (B, m) or (m,) complex128.  proj: (P, m) or (B, P, m) complex128.
    select: sequence of state indices.  Returns a dict with 'state'
    (B, nsave, m), 'proj' (B, nsave, P) and/or 'mean' (nsave, P).
    """
    require_gpu()
    if precision is None:
        precision = QSX_FP32 if matrix.dtype == torch.complex64 else QSX_FP64
    want = torch.complex64 if precision == QSX_FP32 else torch.complex128
    _need(matrix, want, 'matrix')
    m = matrix.shape[-1]
    rows = matrix.shape[-2]
    dev = matrix.device
    y0 = _need(y0.to(torch.complex128).contiguous(), torch.complex128, 'y0')
    B = matrix.shape[0] if matrix.dim() == 3 else (y0.shape[0] if y0.dim() == 2 else 1)
    if matrix.dim() == 3 and matrix.shape[0] != B:
        raise ValueError('matrix batch does not match')
    if y0.dim() == 2 and y0.shape[0] != B:
        raise ValueError('y0 batch does not match')
    if nsteps % save_every:
        raise ValueError('nsteps must be a multiple of save_every')
    nsave = nsteps // save_every + 1
    a = Rk4Args()
    a.precision = precision
    a.form = form
    a.m = m
    a.nsteps = nsteps
    a.batch = B
    a.matrix = matrix.data_ptr()
    a.matrix_stride = rows * m if matrix.dim() == 3 else 0
    a.block_k = block_k
    a.variant = int(variant)
    a.h = h
    a.y0 = y0.data_ptr()
    a.y0_stride = m if y0.dim() == 2 else 0
    a.save_every = save_every
    keep = []
    nout = 0
    if proj is not None:
        proj = _need(proj.to(torch.complex128).contiguous(), torch.complex128, 'proj')
        a.nproj = proj.shape[-2]
        a.proj = proj.data_ptr()
        a.proj_stride = a.nproj * m if proj.dim() == 3 else 0
        nout = a.nproj
        keep.append(proj)
    if select is not None:
        sel_np = np.asarray(select, dtype=np.int64).reshape(-1)
        if sel_np.size == 0 or sel_np.min() < 0 or sel_np.max() >= m:
            raise ValueError('select indices must lie in [0, {})'.format(m))
        if len(np.unique(sel_np)) != sel_np.size:
            raise ValueError('select indices must be distinct')
        sel = const_tensor(sel_np.astype(np.int32), torch.int32, dev)
        a.nselect = sel.numel()
        a.select = sel.data_ptr()
        nout = a.nselect
        keep.append(sel)
    out = {}
    if state:
        out['state'] = torch.empty((B, nsave, m), dtype=torch.complex128, device=dev)
        a.out_state = out['state'].data_ptr()
    if nout and per_sample:
        out['proj'] = torch.empty((B, nsave, nout), dtype=torch.complex128, device=dev)
        a.out_proj = out['proj'].data_ptr()
    if nout and mean:
        out['mean'] = torch.empty((nsave, nout), dtype=torch.complex128, device=dev)
        a.out_mean = out['mean'].data_ptr()
        a.mean_scale = 1.0 / B
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    a.status = status.data_ptr()
    lib = load()
    if mean and nout:
        nbytes = ctypes.c_size_t(0)
        _check(lib.qsx_rk4_workspace_bytes(ctypes.byref(a), ctypes.byref(nbytes)),
               'qsx_rk4_workspace_bytes')
        if workspace is None or workspace.numel() < nbytes.value:
            workspace = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=dev)
        a.workspace = workspace.data_ptr()
        a.workspace_bytes = workspace.numel()
    _check(lib.qsx_rk4_batched(ctypes.byref(a), _stream()), 'qsx_rk4_batched')
    if check_finite:
        st = int(status.item())
        if st & QSX_ERR_NONFINITE:
            raise IntegratorError('non-finite state during RK4 integration')
        if st & QSX_ERR_INVALID_ARG:
            raise QsxError('qsx_rk4_batched: index table out of range')
    out['status'] = status
    return out


def dft(x, t0, dt, freqs, rw_freq=0.0, unit_convert=1.0, sign=1, precision=QSX_FP64):
    """X[b, k] = dt Σ_n x[b, n] exp(i sign (f_k - rw) uc (t0 + n dt));
    precision QSX_FP32 rotates and sums in FP32 between FP64 phase anchors
    (qsx_dft_batched_f32), for signals from FP32 propagation."""
    require_gpu()
    x = _need(x.to(torch.complex128).contiguous(), torch.complex128, 'x')
    squeeze = x.dim() == 1
    if squeeze:
        x = x[None]
    freqs = _need(torch.as_tensor(freqs, dtype=torch.float64, device=x.device).contiguous(),
                  torch.float64, 'freqs', 1)
    B, nt = x.shape
    X = torch.empty((B, freqs.numel()), dtype=torch.complex128, device=x.device)
    fn = load().qsx_dft_batched_f32 if (precision == QSX_FP32 and nt <= 24576) \
        else load().qsx_dft_batched
    _check(fn(_p(x), nt, B, t0, dt, _p(freqs), freqs.numel(), rw_freq, unit_convert, sign,
              _p(X), _stream()), 'qsx_dft_batched')
    return X[0] if squeeze else X


def dft2(x, t01, dt1, f1, sign1, t03, dt3, f3, sign3, rw_freq=0.0, unit_convert=1.0):
    """Both time axes of a (n1, B, n3) complex signal transformed in one
    launch (qsx_dft2_batched): X[k1, b, k3] = dt1 dt3 sum x[n1, b, n3]
    exp(i sign1 (f1 - rw) uc t1) exp(i sign3 (f3 - rw) uc t3)."""
    require_gpu()
    x = _need(x.to(torch.complex128), torch.complex128, 'x', 3)
    n1, B, n3 = x.shape
    s1, sb, s3 = x.stride()
    dev = x.device
    f1 = _need(torch.as_tensor(f1, dtype=torch.float64, device=dev).contiguous(),
               torch.float64, 'f1', 1)
    f3 = _need(torch.as_tensor(f3, dtype=torch.float64, device=dev).contiguous(),
               torch.float64, 'f3', 1)
    X = torch.empty((f1.numel(), B, f3.numel()), dtype=torch.complex128, device=dev)
    _check(load().qsx_dft2_batched(_p(x), n1, B, n3, s1, sb, s3, t01, dt1, _p(f1), f1.numel(),
                                   int(sign1), t03, dt3, _p(f3), f3.numel(), int(sign3),
                                   rw_freq, unit_convert, _p(X), _stream()),
           'qsx_dft2_batched')
    return X


def _heom_args(tables, Hx, Hy, unit_convert, batch, precision=QSX_FP64):
    """Fill HeomArgs from HEOMTables (device copies kept alive by the caller)."""
    d = tables.device()
    _need(Hx, torch.float64, 'Hx')
    _need(Hy, torch.float64, 'Hy')
    a = HeomArgs()
    a.precision = precision
    a.nx, a.ny, a.nnodes = tables.nx, tables.ny, tables.nnodes
    a.nterms, a.n_sites = tables.nterms, tables.n_sites
    a.save_every, a.save_nodes = 1, 1
    a.batch = batch
    a.H_stride = 1 if Hx.dim() == 3 else 0
    a.Hx, a.Hy = Hx.data_ptr(), Hy.data_ptr()
    a.occx, a.occy = d['occx'].data_ptr(), d['occy'].data_ptr()
    a.W = d['W'].data_ptr() if d['W'] is not None else None
    a.shift, a.nbr, a.site = d['shift'].data_ptr(), d['nbr'].data_ptr(), d['site'].data_ptr()
    a.alpha, a.beta = d['alpha'].data_ptr(), d['beta'].data_ptr()
    a.gamma = d['gamma'].data_ptr() if d['gamma'] is not None else None
    a.Wraw = d['Wraw'].data_ptr() if d['Wraw'] is not None else None
    a.unit_convert = unit_convert
    return a


def heom_rhs(tables, Hx, Hy, x, unit_convert):
    """Generator applied to x (B, nnodes * nx * ny) complex128 on the GPU."""
    require_gpu()
    x = _need(x.to(torch.complex128).contiguous(), torch.complex128, 'x', 2)
    B = x.shape[0]
    if Hx.dim() == 3 and Hx.shape[0] != B:
        raise ValueError('per-sample H does not match the batch')
    a = _heom_args(tables, Hx, Hy, unit_convert, B)
    out = torch.empty_like(x)
    _check(load().qsx_heom_rhs(ctypes.byref(a), _p(x), _p(out), _stream()), 'qsx_heom_rhs')
    return out


def heom_rk4(tables, Hx, Hy, y0, nsteps, h, unit_convert, batch=None, save_every=1,
             save_nodes=1, precision=QSX_FP64, per_sample=True, mean=False,
             check_finite=True, variant=0):
    """RK4 loop over the HEOM generator for all samples (qsx_heom_rk4).
    variant 0: the library's choice (one persistent cluster launch per call
    when it fits in one wave, else per-stage launches); 1: one launch per RK4
    stage; 2: the cluster launch whenever its shared memory fits; 3: one
    launch per RK4 stage with the node commutators on the tensor cores (a
    tcgen05 3xTF32 product per tile of 64 node blocks; FP32 blocks up to
    8 x 8, other cases as 1); 4: as 1 with every coupling term of a node
    visited by every element (blocks up to 8 x 8 otherwise visit only the
    terms of their own sites)."""
    require_gpu()
    y0 = _need(y0.to(torch.complex128).contiguous(), torch.complex128, 'y0')
    if batch is None:
        batch = Hx.shape[0] if Hx.dim() == 3 else (y0.shape[0] if y0.dim() == 2 else 1)
    a = _heom_args(tables, Hx, Hy, unit_convert, batch, precision)
    a.nsteps, a.save_every, a.save_nodes = nsteps, save_every, save_nodes
    a.variant = int(variant)
    a.h = h
    a.y0, a.y0_stride = y0.data_ptr(), (1 if y0.dim() == 2 else 0)
    nsave = nsteps // save_every + 1
    E = tables.nx * tables.ny
    dev = y0.device
    out = {}
    if per_sample:
        out['state'] = torch.empty((batch, nsave, save_nodes * E), dtype=torch.complex128,
                                   device=dev)
        a.out_state = out['state'].data_ptr()
    if mean:
        out['mean'] = torch.empty((nsave, save_nodes * E), dtype=torch.complex128, device=dev)
        a.out_mean = out['mean'].data_ptr()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    a.status = status.data_ptr()
    nbytes = ctypes.c_size_t(0)
    lib = load()
    _check(lib.qsx_heom_workspace_bytes(ctypes.byref(a), ctypes.byref(nbytes)),
           'qsx_heom_workspace_bytes')
    ws = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=dev)
    a.workspace, a.workspace_bytes = ws.data_ptr(), ws.numel()
    _check(lib.qsx_heom_rk4(ctypes.byref(a), _stream()), 'qsx_heom_rk4')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state during HEOM integration')
    out['status'] = status
    return out


# ------------------------------------------------- two-exciton (f) manifold
def _real_dtype(precision):
    return torch.float32 if precision == QSX_FP32 else torch.float64


def _cplx_dtype(precision):
    return torch.complex64 if precision == QSX_FP32 else torch.complex128


def fblock_tensor(E, U, n_sites, site_pairs, bath, unit_convert, precision=QSX_FP64,
                  discard_imag_corr=False, matsubara_cutoff=1000):
    """Eigenbasis f-manifold tensor planes Y (B, P, 2N, P) in the working precision."""
    require_gpu()
    _need(E, torch.float64, 'E', 2)
    _need(U, torch.float64, 'U', 3)
    _need(site_pairs, torch.int32, 'site_pairs', 2)
    B, P = E.shape
    Y = torch.empty((B, P, 2 * n_sites, P), dtype=_real_dtype(precision), device=E.device)
    _check(load().qsx_fblock_tensor(
        _p(E), _p(U), P, n_sites, _p(site_pairs), B, bath.temperature, bath.reorg_energy,
        bath.cutoff_freq, matsubara_cutoff, int(discard_imag_corr), unit_convert,
        precision, _p(Y), _stream()), 'qsx_fblock_tensor')
    return Y


def fe_generator(M, H, pair_sites, unit_convert, precision=QSX_FP64):
    """Column operators Q (B, P, N, P) of the 'fe' block from the site-basis planes M."""
    require_gpu()
    _need(M, _real_dtype(precision), 'M', 4)
    _need(H, torch.float64, 'H', 3)
    _need(pair_sites, torch.int32, 'pair_sites', 2)
    B, P, twoN, _ = M.shape
    N = twoN // 2
    Q = torch.empty((B, P, N, P), dtype=_cplx_dtype(precision), device=M.device)
    _check(load().qsx_fe_generator(_p(M), _p(H), P, N, B, _p(pair_sites), unit_convert,
                                   precision, _p(Q), _stream()), 'qsx_fe_generator')
    return Q


def fe_heisenberg_rk4(Q, Ae, Me, pair_sites, y0, nsteps, h, precision=QSX_FP64,
                      check_finite=True):
    """States (B, nsteps+1, P*N) complex128 of the Heisenberg 'fe' RK4 loop."""
    require_gpu()
    cd = _cplx_dtype(precision)
    _need(Q, cd, 'Q', 4)
    _need(Ae, cd, 'Ae', 3)
    _need(Me, cd, 'Me', 4)
    _need(pair_sites, torch.int32, 'pair_sites', 2)
    B, P, N, _ = Q.shape
    y0 = y0.to(torch.complex128).contiguous()
    if y0.shape[-1] != P * N:
        raise ValueError('y0 must have P*N = {} components'.format(P * N))
    stride = 0 if y0.dim() == 1 else P * N
    lib = load()
    ws_bytes = lib.qsx_fe_heisenberg_workspace_bytes(P, N, B, precision)
    ws = torch.empty(max(int(ws_bytes), 1), dtype=torch.uint8, device=Q.device)
    out = torch.empty((B, nsteps + 1, P * N), dtype=torch.complex128, device=Q.device)
    status = torch.zeros(1, dtype=torch.int32, device=Q.device)
    _check(lib.qsx_fe_heisenberg_rk4(_p(Q), _p(Ae), _p(Me), _p(pair_sites), P, N, B,
                                     precision, _p(y0), stride, int(nsteps), float(h),
                                     _p(out), _p(ws), ws.numel(), _p(status), _stream()),
           'qsx_fe_heisenberg_rk4')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state in the fe propagation')
    return out


class CsrMap:
    """A sparse Liouville-space map (rows = outputs) resident on the GPU."""

    def __init__(self, dense, device='cuda'):
        dense = np.asarray(dense, dtype=complex)
        self.shape = dense.shape
        rows, cols = np.nonzero(dense)
        order = np.lexsort((cols, rows))
        rows, cols = rows[order], cols[order]
        rowptr = np.zeros(dense.shape[0] + 1, dtype=np.int32)
        np.add.at(rowptr, rows + 1, 1)
        rowptr = np.cumsum(rowptr).astype(np.int32)
        vals = dense[rows, cols]
        if len(vals) == 0:  # keep valid pointers for an all-zero map
            cols = np.zeros(1, dtype=np.int64)
            vals = np.zeros(1, dtype=complex)
        self.rowptr = torch.as_tensor(rowptr, device=device)
        self.cols = torch.as_tensor(cols.astype(np.int32), device=device)
        self.vals = torch.as_tensor(vals, dtype=torch.complex128, device=device)

    def __call__(self, x):
        """x (..., n_in) complex128 CUDA -> (..., n_out)."""
        require_gpu()
        n_out, n_in = self.shape
        if x.shape[-1] != n_in:
            raise ValueError('map takes {} components (got {})'.format(n_in, x.shape[-1]))
        lead = x.shape[:-1]
        xb = x.to(torch.complex128).reshape(-1, n_in).contiguous()
        out = torch.empty((xb.shape[0], n_out), dtype=torch.complex128, device=x.device)
        _check(load().qsx_csr_map_batched(_p(xb), n_in, xb.shape[0], _p(self.rowptr),
                                          _p(self.cols), _p(self.vals), n_out, _p(out),
                                          _stream()), 'qsx_csr_map_batched')
        return out.reshape(tuple(lead) + (n_out,))


def rk4_adjoint(D, checkpoints, ck_every, nsteps, c, g, scale, want_y0=False):
    """grad of sum_n Re(conj(g_n) x_n) w.r.t. D (and y0) for the mean projected
    RK4 loop (qsx_rk4_adjoint_batched).  D (B, m, m) complex128; checkpoints
    (B, nck, m) complex128; c (m,), g (nsteps+1,) complex128."""
    require_gpu()
    _need(D, torch.complex128, 'D', 3)
    _need(checkpoints, torch.complex128, 'checkpoints', 3)
    c = _need(c.to(torch.complex128).contiguous(), torch.complex128, 'c', 1)
    g = _need(g.to(torch.complex128).contiguous(), torch.complex128, 'g', 1)
    B, m, _ = D.shape
    if g.numel() != nsteps + 1 or c.numel() != m:
        raise ValueError('g needs nsteps+1 entries and c m entries')
    gradD = torch.empty_like(D)
    gy = torch.empty((B, m), dtype=torch.complex128, device=D.device) if want_y0 else None
    _check(load().qsx_rk4_adjoint_batched(_p(D), m, B, int(nsteps), _p(checkpoints),
                                          int(ck_every), checkpoints.shape[1], _p(c), _p(g),
                                          float(scale), _p(gradD), _p(gy), _stream()),
           'qsx_rk4_adjoint_batched')
    return (gradD, gy) if want_y0 else gradD


def eigh_large(H):
    """Batched FP64 eigensolver (Householder + implicit QL) for any n <= 2048.
    H (B, n, n) float64 CUDA, symmetric.  Returns E ascending and U."""
    require_gpu()
    _need(H, torch.float64, 'H', 3)
    B, n, _ = H.shape
    lib = load()
    ws = torch.empty(max(int(lib.qsx_eigh_large_workspace_bytes(n, B)), 1), dtype=torch.uint8,
                     device=H.device)
    E = torch.empty((B, n), dtype=torch.float64, device=H.device)
    U = torch.empty((B, n, n), dtype=torch.float64, device=H.device)
    status = torch.zeros(1, dtype=torch.int32, device=H.device)
    _check(lib.qsx_eigh_large_batched(_p(H), n, B, _p(E), _p(U), _p(ws), ws.numel(),
                                      _p(status), _stream()), 'qsx_eigh_large_batched')
    if int(status.item()):
        raise QsxError('qsx_eigh_large_batched: non-finite eigenvalue (non-finite input?)')
    return E, U


def rk4_field(L, C, coef, y0, nsteps, h, save_every=1, precision=QSX_FP64,
              check_finite=True):
    """States (B, nsteps/save_every + 1, m) complex128 of the field-driven RK4
    loop (qsx_rk4_field_batched).  L (B, m, m) or (m, m) complex128, C
    (npulses, m, m) or per sample (B, npulses, m, m) complex128, coef
    (nsteps, 3, npulses) complex128."""
    require_gpu()
    cd = torch.complex64 if precision == QSX_FP32 else torch.complex128
    Lm = L if L.dim() == 3 else L[None]
    m = Lm.shape[-1]
    y0 = y0.to(torch.complex128).contiguous()
    per_C = C is not None and C.dim() == 4
    if L.dim() == 3:
        B = Lm.shape[0]
    elif per_C:
        B = C.shape[0]
    else:
        B = y0.shape[0] if y0.dim() == 2 else 1
    for name, n in (('C', C.shape[0] if per_C else B), ('y0', y0.shape[0] if y0.dim() == 2 else B)):
        if n != B:
            raise ValueError('{} batch does not match'.format(name))
    Lw = Lm.to(cd).contiguous()
    np_ = int(C.shape[-3]) if C is not None else 0
    Cw = C.to(cd).contiguous() if np_ else None
    cw = coef.to(cd).contiguous() if np_ else None
    out = torch.empty((B, nsteps // save_every + 1, m), dtype=torch.complex128,
                      device=Lw.device)
    status = torch.zeros(1, dtype=torch.int32, device=Lw.device)
    _check(load().qsx_rk4_field_batched(
        _p(Lw), m * m if L.dim() == 3 else 0, _p(Cw), np_ * m * m if per_C else 0, np_,
        _p(cw), m, B, int(nsteps), float(h), _p(y0), m if y0.dim() == 2 else 0,
        int(save_every), precision, _p(out), _p(status), _stream()),
        'qsx_rk4_field_batched')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state in the field-driven propagation')
    return out


def zofe_rk4(H, Ld, Gamma, w, y0, nsteps, h, unit_convert, save_every=1,
             precision=QSX_FP64, V=None, coef=None, proj=None, state=True, mode=0,
             cluster=0, check_finite=True, hermit=0):
    """ZOFE time loop (qsx_zofe_rk4).

    H (n, n) or (B, n, n) float64; Ld (n_sites, n) float64; Gamma, w
    (npm, n_sites) complex128; y0 (M,) or (B, M) complex128 in the reference's
    state layout; V (np, n, n) or (B, np, n, n) and coef (nsteps, 3, np)
    complex128 for pulses; proj (P, n*n) complex128 rows over rho.  Returns a
    dict with 'state' (B, nsave, M) and/or 'proj' (B, nsave, P); with
    state='rho' the states hold rho only, (B, nsave, n*n) column-major; mode
    1 returns the right-hand side at y0 as 'rhs' (B, M).  ``hermit`` selects
    the rho_hermit forms: 0, QSX_ZOFE_RHO_HERMIT or QSX_ZOFE_RHO_HERMIT |
    QSX_ZOFE_HAM_HERMIT.
    """
    require_gpu()
    dev = y0.device
    H = H.to(device=dev, dtype=torch.float64).contiguous()
    Ld = Ld.to(device=dev, dtype=torch.float64).contiguous()
    Gamma = Gamma.to(device=dev, dtype=torch.complex128).contiguous()
    w = w.to(device=dev, dtype=torch.complex128).contiguous()
    y0 = y0.to(torch.complex128).contiguous()
    n = H.shape[-1]
    npm, N = Gamma.shape
    M = n * n + npm * N * n * n
    if y0.shape[-1] != M:
        raise ValueError('y0 must have {} components (n^2 + npm n_sites n^2)'.format(M))
    if tuple(Ld.shape) != (N, n) or tuple(w.shape) != (npm, N):
        raise ValueError('Ld must be (n_sites, n) and w (npm, n_sites)')
    batches = [t.shape[0] for t, d in ((H, 3), (y0, 2)) if t.dim() == d]
    if V is not None and V.dim() == 4:
        batches.append(V.shape[0])
    B = batches[0] if batches else 1
    if any(b != B for b in batches):
        raise ValueError('batch sizes do not match')
    if nsteps % save_every:
        raise ValueError('nsteps must be a multiple of save_every')
    nsave = 1 if mode == 1 else nsteps // save_every + 1
    keep = [H, Ld, Gamma, w, y0]
    a = ZofeArgs()
    a.precision, a.n, a.n_sites, a.npm = precision, n, N, npm
    a.nsteps, a.save_every, a.mode, a.cluster = int(nsteps), int(save_every), int(mode), int(cluster)
    a.hermit = int(hermit)
    a.batch = B
    a.H, a.H_stride = H.data_ptr(), (n * n if H.dim() == 3 else 0)
    a.Ld, a.Gamma, a.w = Ld.data_ptr(), Gamma.data_ptr(), w.data_ptr()
    if V is not None:
        V = V.to(device=dev, dtype=torch.complex128).contiguous()
        coef = coef.to(device=dev, dtype=torch.complex128).contiguous()
        a.npulses = V.shape[-3]
        a.V, a.coef = V.data_ptr(), coef.data_ptr()
        a.V_stride = a.npulses * n * n if V.dim() == 4 else 0
        keep += [V, coef]
    a.unit_convert, a.h = float(unit_convert), float(h)
    a.y0, a.y0_stride = y0.data_ptr(), (M if y0.dim() == 2 else 0)
    out = {}
    if mode == 1:
        out['rhs'] = torch.empty((B, M), dtype=torch.complex128, device=dev)
        a.out_state = out['rhs'].data_ptr()
    else:
        if state:
            width = n * n if state == 'rho' else M
            a.save_rho_only = 1 if state == 'rho' else 0
            out['state'] = torch.empty((B, nsave, width), dtype=torch.complex128, device=dev)
            a.out_state = out['state'].data_ptr()
        if proj is not None:
            proj = proj.to(device=dev, dtype=torch.complex128).contiguous()
            a.nproj = proj.shape[0]
            a.proj = proj.data_ptr()
            keep.append(proj)
            out['proj'] = torch.empty((B, nsave, a.nproj), dtype=torch.complex128, device=dev)
            a.out_proj = out['proj'].data_ptr()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    a.status = status.data_ptr()
    _check(load().qsx_zofe_rk4(ctypes.byref(a), _stream()), 'qsx_zofe_rk4')
    if check_finite and int(status.item()) & QSX_ERR_NONFINITE:
        raise IntegratorError('non-finite state in the ZOFE propagation')
    return out

