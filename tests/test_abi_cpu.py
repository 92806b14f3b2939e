"""The C-ABI library loads and exports every symbol include/qsx.h declares (no GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT
from qspectra_gb300 import _native

HEADER = os.path.join(ROOT, 'include', 'qsx.h')


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(qsx_[a-z0-9_]+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    if not os.path.exists(_native.LIB_PATH):
        from qspectra_gb300 import build
        build.build()
    return _native.load()


def test_header_and_binding_agree():
    assert header_functions() == _native.exported_symbols()


def test_every_declared_symbol_is_exported(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.qsx_version() >= 100
    assert isinstance(lib.qsx_last_error_string(), bytes)


def test_argument_validation_without_gpu(lib):
    blk = (ctypes.c_int * 2)(0, 40)
    st = lib.qsx_eigh_batched(None, 40, 1, 1, blk, None, None, None)
    assert st == 1  # QSX_ERR_INVALID_ARG, rejected before any CUDA call
    assert b'n <= 32' in lib.qsx_last_error_string()
    st = lib.qsx_rk4_propagator_batched(None, 65, 1, 1.0, 0, None, None)
    assert st == 1
    a = _native.Rk4Args()
    a.precision, a.form, a.m, a.nsteps, a.save_every = 0, 0, 7, 5, 2
    st = lib.qsx_rk4_batched(ctypes.byref(a), None)
    assert st == 1 and b'multiple of save_every' in lib.qsx_last_error_string()


def test_rk4_args_layout_matches_library(lib):
    assert ctypes.sizeof(_native.Rk4Args) == lib.qsx_rk4_args_bytes()
    assert _native.Rk4Args.batch.offset == 16


def test_zofe_args_layout_matches_library(lib):
    assert ctypes.sizeof(_native.ZofeArgs) == lib.qsx_zofe_args_bytes()
    assert _native.ZofeArgs.batch.offset == 40
    a = _native.ZofeArgs()
    a.precision, a.n, a.n_sites, a.npm, a.nsteps, a.save_every = 0, 40, 2, 2, 4, 1
    a.batch = 1
    assert lib.qsx_zofe_rk4(ctypes.byref(a), None) == 1
    assert b'bad sizes' in lib.qsx_last_error_string()



def test_tensor_core_block_shapes(lib):
    """The tcgen05 block build takes m <= 64, K = 2^J or 2^J + 1, and at most
    64 selected rows entering its last row product (host logic, no GPU)."""
    def expected(m, K, nsel):
        if m < 1 or m > 64 or K < 2 or K > 64 or nsel < 1 or nsel > m:
            return 0
        pow2 = K & (K - 1) == 0
        pow2p1 = K > 2 and (K - 1) & (K - 2) == 0
        if not (pow2 or pow2p1):
            return 0
        b = 1
        while 2 * b < K - 1:
            b *= 2
        return int(b * nsel <= 64)
    for m in (9, 16, 25, 36, 49, 64, 65):
        for K in (1, 2, 3, 4, 5, 6, 7, 8, 9, 16, 17, 27, 32, 33, 64, 65):
            for nsel in (1, 4, 7, 8, 16, 49):
                assert lib.qsx_rk4_block_matrix_real_tc_supported(m, K, nsel) == \
                    expected(m, K, nsel), (m, K, nsel)


def test_missing_library_raises_instead_of_falling_back(tmp_path, monkeypatch):
    """Without the built library the package raises; there is no CPU path."""
    monkeypatch.setattr(_native, '_LIB', None)
    with pytest.raises(_native.QsxError, match='not found'):
        _native.load(str(tmp_path / 'libqsx_missing.so'))


def test_drivers_need_a_gpu(monkeypatch):
    """With no visible GPU every numeric entry point raises QsxError."""
    import numpy as np
    import torch
    import qspectra_gb300 as qg
    monkeypatch.setattr(torch.cuda, 'is_available', lambda: False)
    with pytest.raises(_native.QsxError, match='needs a CUDA GPU'):
        _native.require_gpu()
    ham = qg.ElectronicHamiltonian(np.diag([12000.0, 12100.0]),
                                   bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 2)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS)
    with pytest.raises(_native.QsxError):
        qg.absorption_spectra(m, 100.0)
