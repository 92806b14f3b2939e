"""Hierarchical equations of motion (qspectra/dynamics/heom.py) on the GPU.

``HEOMModel`` keeps the reference constructor and API.  Its generator is not
assembled as a sparse matrix on the hot path: the host builds small node
tables (ADO enumeration, shifts, coupling terms) once, and the GPU applies
the generator in structured form (qsx_heom_rhs) and runs the RK4 time loop
over all disorder samples at once (qsx_heom_rk4).
"""
from functools import lru_cache

import numpy as np
import scipy.sparse as sps
import torch

from .. import _native
from ..operator_tools import (SubspaceError, extract_subspace, full_liouville_subspace,
                              hilbert_subspace_index, occupation_table)
from .base import DynamicalModel, SystemOperator
from .liouville_space import (EquationOfMotion, LinearMap, LiouvilleSpaceModel,
                              LiouvilleSpaceOperator, _as_device)


@lru_cache(maxsize=None)
def multichoose(n, c):
    """Occupations of n bins summing to c, in the order of multichoose
    (heom.py:155-174): vectors with an empty first bin first (recursing on
    the other bins), then those of total c - 1 with the first bin raised."""
    if c == 0:
        return ((0,) * n,)
    if n == 0:
        return ()
    if n == 1:
        return ((c,),)
    return (tuple((0,) + v for v in multichoose(n - 1, c))
            + tuple((v[0] + 1,) + v[1:] for v in multichoose(n, c - 1)))


def ado_indices(n_sites, K, level_cutoff):
    """N x (K+1) occupation matrices with sum < level_cutoff (heom.py:92-152)."""
    out = []
    for c in range(level_cutoff):
        out.extend(multichoose(n_sites * (K + 1), c))
    return [np.array(v).reshape(n_sites, K + 1) for v in out]


def matsubara_frequencies(K, gamma, T):
    """nu_0 = gamma, nu_k = 2 pi k T (heom.py:61-67)."""
    v = 2 * np.pi * T * np.arange(K + 1)
    v[0] = gamma
    return v


def corr_func_coeffs(K, gamma, T, reorg_en, nu, aki_temp_corr=False):
    """c_0 = λγ(cot(γ/2T) - i), c_k = 4λγTν_k/(ν_k² - γ²) (heom.py:69-89)."""
    if aki_temp_corr:
        c0 = reorg_en * gamma * (1 / (gamma / (2 * T)) - 1j)
    else:
        c0 = reorg_en * gamma * (1 / np.tan(gamma / (2 * T)) - 1j)
    out = [c0]
    for k in range(1, K + 1):
        out.append(4 * reorg_en * gamma * T * nu[k] / (nu[k] ** 2 - gamma ** 2))
    return out


class HEOMTables:
    """Node tables of the HEOM generator on one Liouville block XY.

    terms[n] lists (neighbour m, site j, alpha, beta, gamma): node n receives
    (alpha occ_j(a) + beta occ_j(b) + gamma Wd[a, b] (occ_j(a) - occ_j(b)))
    rho_m[a, b] (heom.py:410-442), with Wd[a, b] = sum_i (occ_i(a) + occ_i(b)
    - 2 occ_i(a) occ_i(b)) the double commutator sum_i [K_i, [K_i, .]] for
    number operators.  gamma is nonzero only for the down couplings under
    aki_temp_corr (heom.py:438-442: -i 4 lam gamma^2 / (nu_1^2 - gamma^2)
    times that double commutator, which for number operators is diagonal, so
    the reference's product with the coupling's commutator is elementwise).
    ``transpose`` swaps sender and receiver (the Heisenberg picture).
    """

    def __init__(self, model, liouville_subspace, transpose=False):
        blocks = liouville_subspace.split(',')
        if len(blocks) != 1:
            raise NotImplementedError('the GPU HEOM path takes one Liouville block '
                                      '(e.g. "ee" or "eg"), got {!r}'.format(liouville_subspace))
        X, Y = blocks[0]
        hs = model.hilbert_subspace
        if X not in hs or Y not in hs:
            raise SubspaceError('{} not in subspace {!r}'.format(liouville_subspace, hs))
        ham = model.hamiltonian
        N = ham.n_sites
        sx = hilbert_subspace_index(X, hs, N)
        sy = hilbert_subspace_index(Y, hs, N)
        occ = occupation_table(N, hs)
        self.occx, self.occy = occ[:, sx], occ[:, sy]
        self.nx, self.ny = self.occx.shape[1], self.occy.shape[1]
        self.sx, self.sy = sx, sy
        bath = ham.bath
        T, lam, g = bath.temperature, bath.reorg_energy, bath.cutoff_freq
        K = model.K
        nu = matsubara_frequencies(K, g, T)
        c = corr_func_coeffs(K, g, T, lam, nu, model.aki_temp_corr)
        nu_inf = matsubara_frequencies(K + 5000, g, T)
        c_inf = corr_func_coeffs(K + 5000, g, T, lam, nu_inf, model.aki_temp_corr)
        kappa = 4 * lam * g ** 2 / (nu_inf[1] ** 2 - g ** 2)
        ados = model.ado_indices
        pos = {tuple(a.reshape(-1)): i for i, a in enumerate(ados)}
        self.nnodes = len(ados)
        self.shift = np.array([float(np.sum(a.dot(nu))) for a in ados])
        terms = [[] for _ in range(self.nnodes)]
        for n, ado in enumerate(ados):
            for (j, k), njk in np.ndenumerate(ado):
                up = ado.copy()
                up[j, k] += 1
                p = pos.get(tuple(up.reshape(-1)))
                if p is not None:
                    m = np.sqrt((njk + 1) * np.abs(c[k])) if model.modified_HEOM else 1.0
                    terms[n].append((p, j, -1j * m, 1j * m, 0.0))
                if njk > 0:
                    dn = ado.copy()
                    dn[j, k] -= 1
                    q = pos[tuple(dn.reshape(-1))]
                    m = np.sqrt(njk / np.abs(c[k])) if model.modified_HEOM else njk
                    a_, b_ = -1j * m * c[k], 1j * m * np.conj(c[k])
                    g_ = -1j * kappa if model.aki_temp_corr else 0.0
                    terms[n].append((q, j, a_, b_, g_))
        if transpose:
            tt = [[] for _ in range(self.nnodes)]
            for n, lst in enumerate(terms):
                for (m, j, a_, b_, g_) in lst:
                    tt[m].append((n, j, a_, b_, g_))
            terms = tt
        # grouped by site (stable): the kernel visits only the sites a
        # state occupies, through per-site ranges of this list
        terms = [sorted(lst, key=lambda term: term[1]) for lst in terms]
        self.terms = terms
        nt = max(1, max(len(t) for t in terms))
        self.nterms = nt
        self.nbr = -np.ones((self.nnodes, nt), np.int32)
        self.site = np.zeros((self.nnodes, nt), np.int32)
        self.alpha = np.zeros((self.nnodes, nt), complex)
        self.beta = np.zeros((self.nnodes, nt), complex)
        self.gamma = np.zeros((self.nnodes, nt), complex)
        for n, lst in enumerate(terms):
            for t, (m, j, a_, b_, g_) in enumerate(lst):
                self.nbr[n, t], self.site[n, t] = m, j
                self.alpha[n, t], self.beta[n, t], self.gamma[n, t] = a_, b_, g_
        ox, oy = self.occx[:, :, None], self.occy[:, None, :]
        Wab = np.sum(ox + oy - 2 * ox * oy, axis=0).reshape(-1, order='F')  # [nx ny]
        # raw double-commutator weights of the aki_temp_corr down terms
        self.Wraw = Wab.astype(float) if model.aki_temp_corr else None
        if not model.aki_temp_corr:
            self.gamma = None
        # low-temperature correction sum_j [K_j, [K_j, .]] (heom.py:386-408),
        # also applied under aki_temp_corr with the coefficient c_1 / nu_1
        self.W = None
        if model.low_temp_corr or model.aki_temp_corr:
            if model.aki_temp_corr:
                tc = (c_inf[1] / nu_inf[1]).real
            else:
                tc = np.sum((np.array(c_inf) / nu_inf)[K + 1:]).real
            self.W = tc * Wab
        self.n_sites = N
        self._dev = None

    def device(self):
        if self._dev is None:
            dev = torch.device('cuda', torch.cuda.current_device())
            t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
            self._dev = dict(
                occx=t(self.occx, torch.float64), occy=t(self.occy, torch.float64),
                W=None if self.W is None else t(self.W, torch.float64),
                shift=t(self.shift, torch.float64), nbr=t(self.nbr, torch.int32),
                site=t(self.site, torch.int32), alpha=t(self.alpha, torch.complex128),
                beta=t(self.beta, torch.complex128),
                gamma=None if self.gamma is None else t(self.gamma, torch.complex128),
                Wraw=None if self.Wraw is None else t(self.Wraw, torch.float64))
        return self._dev

    def sparse(self, Hx, Hy, unit_convert):
        """The generator as a scipy CSR matrix (API parity with HEOM_tensor)."""
        E = self.nx * self.ny
        Ix, Iy = np.eye(self.nx), np.eye(self.ny)
        comm = np.kron(Iy, Hx) - np.kron(Hy.T, Ix)
        W = np.zeros(E) if self.W is None else self.W
        rows, cols, vals = [], [], []
        for n in range(self.nnodes):
            blk = -1j * comm - np.diag(self.shift[n] + W)
            r, cidx = np.nonzero(blk)
            rows.append(r + n * E)
            cols.append(cidx + n * E)
            vals.append(blk[r, cidx])
            for t in range(self.nterms):
                m = self.nbr[n, t]
                if m < 0:
                    continue
                j = self.site[n, t]
                ox = np.kron(np.ones(self.ny), self.occx[j])
                oy = np.kron(self.occy[j], np.ones(self.nx))
                d = self.alpha[n, t] * ox + self.beta[n, t] * oy
                if self.gamma is not None:
                    d = d + self.gamma[n, t] * self.Wraw * (ox - oy)
                nz = np.nonzero(d)[0]
                rows.append(nz + n * E)
                cols.append(nz + m * E)
                vals.append(d[nz])
        L = sps.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                           shape=(self.nnodes * E,) * 2).tocsr()
        return unit_convert * L


class HEOMEquationOfMotion(EquationOfMotion):
    """GPU HEOM generator on one Liouville block; ``H`` is (S, n, n) or (n, n)."""

    def __init__(self, model, tables, Hx, Hy, liouville_subspace, heisenberg_picture):
        super().__init__(None, liouville_subspace, heisenberg_picture, model)
        self.tables = tables
        self.Hx, self.Hy = Hx, Hy

    @property
    def dim(self):
        return self.tables.nnodes * self.tables.nx * self.tables.ny

    def __call__(self, t, rho):
        x, is_tensor = _as_device(rho)
        squeeze = x.dim() == 1
        X = (x[None] if squeeze else x).contiguous()
        out = _native.heom_rhs(self.tables, self.Hx, self.Hy, X, self.model.unit_convert)
        out = out[0] if squeeze else out
        return out if is_tensor else out.cpu().numpy()


class HEOMMultiBlockEquationOfMotion(EquationOfMotion):
    """The HEOM generator on a Liouville subspace of several blocks (e.g.
    'gg,ge,eg,ee'; heom.py:298-443 builds it on the union of the blocks).
    H and the couplings are block-diagonal over the manifolds, so every block
    XY of every node evolves on its own: each block runs its structured
    generator on its share of the node vectors, gathered from and scattered
    back to the positions that block holds in the union's ascending
    column-stacked order."""

    def __init__(self, model, liouville_subspace, heisenberg_picture):
        super().__init__(None, liouville_subspace, heisenberg_picture, model)
        full = model.lspace_model.liouville_subspace_index(liouville_subspace)
        self.M = len(full)
        self.nnodes = model.ado_count
        self.parts = []
        for blk in liouville_subspace.split(','):
            eom = model.equation_of_motion(blk, heisenberg_picture)
            pos = np.searchsorted(full, model.lspace_model.liouville_subspace_index(blk))
            flat = (np.arange(self.nnodes)[:, None] * self.M + pos[None, :]).reshape(-1)
            self.parts.append((eom, flat))

    @property
    def dim(self):
        return self.nnodes * self.M

    def gather(self, x, flat):
        return x[..., _native.const_tensor(flat, torch.int64, x.device)]

    def scatter(self, out, flat, values):
        out[..., _native.const_tensor(flat, torch.int64, out.device)] = values

    def __call__(self, t, rho):
        x, is_tensor = _as_device(rho)
        out = torch.zeros_like(x)
        for eom, flat in self.parts:
            self.scatter(out, flat, eom(t, self.gather(x, flat)))
        return out if is_tensor else out.cpu().numpy()


def map_over_ados(func, state, ado_count, from_size):
    s = np.asarray(state)
    blocks = s.reshape(s.shape[:-1] + (ado_count, from_size))
    return np.asarray(func(blocks)).reshape(s.shape[:-1] + (-1,))


class HEOMSpaceOperator(SystemOperator):
    """Dipole operator acting node by node (heom.py:14-58)."""

    def __init__(self, operator, liouv_subspace_map, dynamical_model):
        self.lspace_op = LiouvilleSpaceOperator(operator, liouv_subspace_map,
                                                dynamical_model.lspace_model)
        self.ado_count = dynamical_model.ado_count
        self.from_size = self.lspace_op.from_indices.size
        self.to_size = self.lspace_op.to_indices.size

    @property
    def bra_vector(self):
        b = self.lspace_op.bra_vector
        out = np.zeros(b.size * self.ado_count, dtype=complex)
        out[:b.size] = b
        return out

    def _apply(self, fn, state):
        return map_over_ados(fn, state, self.ado_count, self.from_size)

    def left_multiply(self, state):
        return self._apply(self.lspace_op.left_multiply, state)

    def right_multiply(self, state):
        return self._apply(self.lspace_op.right_multiply, state)

    def commutator(self, state):
        return self._apply(self.lspace_op.commutator, state)

    def expectation_value(self, state):
        s = np.asarray(state)
        return self.lspace_op.expectation_value(s[..., :self.from_size])


class HEOMModel(DynamicalModel):
    """HEOM with a Drude bath per site (heom.py:177-443)."""
    system_operator = HEOMSpaceOperator

    def __init__(self, hamiltonian, rw_freq=None, hilbert_subspace='gef',
                 unit_convert=1, level_cutoff=3, K=1, low_temp_corr=True,
                 modified_HEOM=False, aki_temp_corr=False):
        super().__init__(hamiltonian, rw_freq, hilbert_subspace, unit_convert)
        self.lspace_model = LiouvilleSpaceModel(hamiltonian, rw_freq, hilbert_subspace,
                                                unit_convert, 'site')
        self.level_cutoff = level_cutoff
        self.K = K
        self.low_temp_corr = low_temp_corr
        self.modified_HEOM = modified_HEOM
        self.aki_temp_corr = aki_temp_corr
        if modified_HEOM:
            assert self.low_temp_corr
        self.ado_indices = ado_indices(self.hamiltonian.n_sites, K, level_cutoff)
        self.ado_count = len(self.ado_indices)
        self._cache = {}

    def __repr__(self):
        return 'HEOMModel(level_cutoff={!r}, K={!r}, ado_count={!r})'.format(
            self.level_cutoff, self.K, self.ado_count)

    def tables(self, liouville_subspace, transpose=False):
        key = ('tables', liouville_subspace, bool(transpose))
        if key not in self._cache:
            self._cache[key] = HEOMTables(self, liouville_subspace, transpose)
        return self._cache[key]

    def block_hamiltonians(self, liouville_subspace, H=None):
        """Hx, Hy (rotating frame) for the block, shared or per sample."""
        tb = self.tables(liouville_subspace)
        if H is None:
            H = torch.as_tensor(self.hamiltonian.H(self.hilbert_subspace),
                                dtype=torch.float64).cuda()
        Hx = H[..., tb.sx, tb.sx].contiguous()
        Hy = H[..., tb.sy, tb.sy].contiguous()
        return Hx, Hy

    def equation_of_motion(self, liouville_subspace, heisenberg_picture=False):
        """heom.py:228-244 as a GPU-resident callable; a subspace of several
        Liouville blocks composes the blocks' generators."""
        key = ('eom', liouville_subspace, bool(heisenberg_picture))
        if key not in self._cache and ',' in liouville_subspace:
            _native.require_gpu()
            self._cache[key] = HEOMMultiBlockEquationOfMotion(self, liouville_subspace,
                                                             heisenberg_picture)
        if key not in self._cache:
            _native.require_gpu()
            tb = self.tables(liouville_subspace, heisenberg_picture)
            Hx, Hy = self.block_hamiltonians(liouville_subspace)
            self._cache[key] = HEOMEquationOfMotion(self, tb, Hx, Hy, liouville_subspace,
                                                    heisenberg_picture)
        return self._cache[key]

    def HEOM_tensor(self, liouville_subspace, heisenberg_picture=False):
        """The generator as a sparse matrix, without unit_convert (heom.py:298-443);
        several Liouville blocks give the block-diagonal generator on their
        union, in the union's ascending column-stacked order per node."""
        H = self.hamiltonian.H(self.hilbert_subspace)
        if ',' not in liouville_subspace:
            tb = self.tables(liouville_subspace, heisenberg_picture)
            return tb.sparse(H[tb.sx, tb.sx], H[tb.sy, tb.sy], 1.0)
        full = self.lspace_model.liouville_subspace_index(liouville_subspace)
        M = len(full)
        rows, cols, vals = [], [], []
        for blk in liouville_subspace.split(','):
            tb = self.tables(blk, heisenberg_picture)
            L = tb.sparse(H[tb.sx, tb.sx], H[tb.sy, tb.sy], 1.0).tocoo()
            pos = np.searchsorted(full, self.lspace_model.liouville_subspace_index(blk))
            Mb = len(pos)
            rows.append((L.row // Mb) * M + pos[L.row % Mb])
            cols.append((L.col // Mb) * M + pos[L.col % Mb])
            vals.append(L.data)
        n = self.ado_count * M
        return sps.coo_matrix((np.concatenate(vals), (np.concatenate(rows),
                                                      np.concatenate(cols))),
                              shape=(n, n)).tocsr()

    def thermal_state(self, liouville_subspace):
        rho0 = self.lspace_model.thermal_state(liouville_subspace)
        rho = np.zeros(rho0.size * self.ado_count, dtype=complex)
        rho[:rho0.size] = rho0
        return rho

    def dipole_operator(self, liouv_subspace_map, polarization, transitions='-+'):
        op = self.hamiltonian.dipole_operator(self.hilbert_subspace, polarization,
                                              transitions)
        return HEOMSpaceOperator(op, liouv_subspace_map, self)

    def map_between_subspaces(self, state, from_subspace, to_subspace):
        from_size = self.lspace_model.liouville_subspace_index(from_subspace).size
        return map_over_ados(
            lambda blocks: np.array([self.lspace_model.map_between_subspaces(
                b, from_subspace, to_subspace) for b in blocks.reshape(-1, from_size)]
            ).reshape(blocks.shape[:-1] + (-1,)),
            state, self.ado_count, from_size)

    def density_matrix_to_state_vector(self, rho0, liouville_subspace):
        s0 = self.lspace_model.density_matrix_to_state_vector(rho0, liouville_subspace)
        out = np.zeros(s0.size * self.ado_count, dtype=complex)
        out[:s0.size] = s0
        return out

    def state_vector_to_density_matrix(self, rhos):
        """Node-0 blocks as density matrices (heom.py:288-296, integer sizes)."""
        nsq = rhos.shape[-1] // self.ado_count
        return self.lspace_model.state_vector_to_density_matrix(rhos[..., :nsq])
