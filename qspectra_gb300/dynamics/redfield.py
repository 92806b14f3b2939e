"""Redfield theory on the GPU (qspectra/dynamics/redfield.py).

``RedfieldModel`` keeps the reference constructor and API.  Its generator is
built per disorder sample on the GPU in FP64: Jacobi eigensolve of the
rotating-frame Hamiltonian (qsx_eigh_batched), Debye correlation function and
operator-form Redfield tensor (qsx_redfield_operators_batched), then the
requested dense Liouville block (qsx_redfield_liouvillian_batched).
``RedfieldBuild`` does the same for a whole batch of samples at once and is
what the ensemble drivers use.
"""
import numpy as np
import torch

from .. import _native
from ..operator_tools import n_excitations
from .liouville_space import LiouvilleSpaceModel

EIGH_JACOBI_MAX = 32


def manifold_bounds(n_sites, hilbert_subspace):
    """[0, end_g, end_e, ...] block boundaries of the manifolds present."""
    sizes = dict(zip('gef', n_excitations(n_sites)))
    out = [0]
    for letter in 'gef':
        if letter in hilbert_subspace and sizes[letter] > 0:
            out.append(out[-1] + int(sizes[letter]))
    return out


class RedfieldBuild:
    """Batched FP64 Redfield generator for S disorder samples.

    ``H`` is (S, n, n) float64 on the GPU: rotating-frame Hamiltonians on the
    model's Hilbert subspace.  Eigen-decomposition and the operator form are
    computed once; ``block`` then assembles any Liouville block.
    """

    def __init__(self, H, n_sites, hilbert_subspace, occ, bath, unit_convert,
                 secular=False, discard_imag_corr=False, evolve_basis='site',
                 precision=_native.QSX_FP64, build_precision=None):
        self.H = H
        self.n = H.shape[-1]
        self.n_sites = n_sites
        self.unit_convert = unit_convert
        self.secular = secular
        self.evolve_basis = evolve_basis
        self.occ = _native.const_tensor(np.asarray(occ, dtype=np.float64), torch.float64,
                                        H.device)
        bounds = manifold_bounds(n_sites, hilbert_subspace)
        if self.n > EIGH_JACOBI_MAX:
            raise _native.QsxError(
                'Hilbert space of {} states exceeds the {}-state Redfield '
                'build; use the operator-form third-order path'.format(
                    self.n, EIGH_JACOBI_MAX))
        self.site_ops = evolve_basis == 'site' and not secular
        # the eigendecomposition and operator build run in FP64 unless an FP32
        # build is asked for (it feeds only FP32 propagation)
        if build_precision is None:
            build_precision = _native.QSX_FP64
        self.build_precision = build_precision
        one_exciton = set(hilbert_subspace) <= set('ge') and 'e' in hilbert_subspace
        off = 1 if 'g' in hilbert_subspace else 0
        self.refined = (build_precision == _native.QSX_FP64 and precision == _native.QSX_FP32
                        and self.site_ops and one_exciton and 2 <= n_sites <= 8
                        and self.n == off + n_sites)
        if self.refined:
            # FP64 build for FP32 propagation: FP32 Jacobi, two FP64
            # refinement steps, FP64 operators (qsx_redfield_build_w64)
            _, U32 = _native.eigh(H, bounds, _native.QSX_FP32)
            self.E, self.U, self.G, self.M = _native.redfield_build_w64(
                H, U32, n_sites, off, bath, unit_convert, discard_imag_corr,
                matsubara_cutoff=bath.matsubara_cutoff)
            self.K = None
            return
        self.E, self.U = _native.eigh(H, bounds, build_precision)
        if (build_precision == _native.QSX_FP32 and self.site_ops and one_exciton
                and 2 <= n_sites <= 8 and self.n == off + n_sites):
            # FP32 build of a one-exciton space: the warp-per-sample operator
            # form (qsx_redfield_operators_w32)
            self.G, self.M = _native.redfield_operators_w32(
                self.E, self.U, n_sites, off, bath, unit_convert, discard_imag_corr,
                matsubara_cutoff=bath.matsubara_cutoff)
            self.K = None
            return
        self.G, self.M, self.K = _native.redfield_operators(
            self.E, self.U, self.occ, bath, unit_convert, discard_imag_corr,
            site_basis=self.site_ops, matsubara_cutoff=bath.matsubara_cutoff,
            precision=build_precision)

    def propagator(self, idx, h, precision=_native.QSX_FP64, transpose=False):
        """(S, m, m) RK4 propagator D = P - I of the block ``idx`` (m <= 64).

        Site-basis non-secular generators go through the fused kernel (the
        block is built in shared memory and never stored); other cases build
        the block first.
        """
        if self.site_ops and len(idx) <= 64:
            idx_t = _native.const_tensor(np.asarray(idx, dtype=np.int32), torch.int32,
                                         self.H.device)
            D = _native.redfield_propagator(self.H, self.G, self.M, self.occ, idx_t,
                                            self.unit_convert, h, precision, transpose)
            if D is not None:
                return D
        return _native.rk4_propagator(self.block(idx, transpose), h, precision)

    def hermitian_propagator(self, idx, nb, h, precision=_native.QSX_FP32):
        """(S, nb^2, nb^2) real one-step propagator D_r = P_r - I of the
        diagonal block of nb x nb states ``idx`` (column-stacked), in the
        Hermitian coordinates of ``hermitian_coordinates``."""
        if self.site_ops and len(idx) <= 64:
            states = np.asarray(idx)[:nb] % self.n
            return _native.redfield_propagator_hermitian(self.H, self.G, self.M, self.occ,
                                                         states, self.unit_convert, h,
                                                         precision)
        return _native.hermitian_real_form(self.propagator(idx, h, precision), nb)

    def block(self, idx, transpose=False):
        """(S, m, m) complex128 generator on the column-stacked indices ``idx``."""
        idx_np = np.asarray(idx, dtype=np.int64)
        idx_t = _native.const_tensor(idx_np.astype(np.int32), torch.int32, self.H.device)
        uc = self.unit_convert
        if self.site_ops:
            return _native.redfield_liouvillian(self.H, self.G, self.M, idx_t, uc,
                                                occ=self.occ, transpose=transpose)
        Hd = torch.diag_embed(self.E).contiguous()
        L = _native.redfield_liouvillian(Hd, self.G, self.M, idx_t, uc, K=self.K,
                                         secular=self.secular)
        if self.evolve_basis == 'site':
            # (U ⊗ U) restricted to idx: U is block-diagonal over manifolds and
            # idx is a union of Liouville blocks, so the restriction is exact.
            n = self.n
            a, b = idx_np % n, idx_np // n
            ai = torch.as_tensor(a, device=self.H.device)
            bi = torch.as_tensor(b, device=self.H.device)
            U = self.U.to(torch.complex128)
            W = U[:, ai][:, :, ai] * U[:, bi][:, :, bi]
            L = W @ L @ W.transpose(-1, -2)
        if transpose:
            L = L.transpose(-1, -2)
        return L.contiguous()


class RedfieldModel(LiouvilleSpaceModel):
    """Redfield dynamics, each site coupled to an identical independent bath
    (redfield.py:107-152)."""

    def __init__(self, hamiltonian, rw_freq=None, hilbert_subspace='gef',
                 unit_convert=1, secular=True, discard_imag_corr=False,
                 evolve_basis='site', sparse_matrix=False):
        super().__init__(hamiltonian, rw_freq, hilbert_subspace, unit_convert,
                         evolve_basis, sparse_matrix)
        self.secular = secular
        self.discard_imag_corr = discard_imag_corr

    def __repr__(self):
        return ('RedfieldModel(hilbert_subspace={!r}, unit_convert={!r}, '
                'secular={!r}, discard_imag_corr={!r}, evolve_basis={!r})').format(
            self.hilbert_subspace, self.unit_convert, self.secular,
            self.discard_imag_corr, self.evolve_basis)

    def build_batch(self, H, precision=_native.QSX_FP64, build_precision=None):
        """RedfieldBuild for a (S, n, n) batch of rotating-frame Hamiltonians.
        ``precision`` is the propagation precision; the eigendecomposition
        and operator build run in FP64 unless ``build_precision`` is
        QSX_FP32 (an FP32 build, for FP32 propagation only)."""
        ham = self.hamiltonian
        return RedfieldBuild(H, ham.n_sites, self.hilbert_subspace,
                             ham.occupation_table(self.hilbert_subspace), ham.bath,
                             self.unit_convert, self.secular, self.discard_imag_corr,
                             self.evolve_basis, precision, build_precision)

    def _build(self):
        if 'build' not in self._cache:
            _native.require_gpu()
            H = torch.as_tensor(self.hamiltonian.H(self.hilbert_subspace),
                                dtype=torch.float64).cuda()[None].contiguous()
            self._cache['build'] = self.build_batch(H)
        return self._cache['build']

    def _block(self, idx, transpose):
        return self._build().block(idx, transpose)[0]
