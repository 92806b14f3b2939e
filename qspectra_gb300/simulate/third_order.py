"""Batched third-order response with a two-exciton manifold (GPU).

The reference evaluates ``third_order_response`` (qspectra/simulate/
response.py:267-337) per disorder sample and per Liouville pathway, each
integrate() call a zvode run over a dense block of the full 'gef'
Liouvillian.  For Redfield models in the site basis the generator is
block-diagonal over the g/e/f manifolds, so this engine never forms the
'gef' tensor:

* g and e blocks come from a 'ge' Redfield build (batched FP64 Jacobi
  eigensolve and operator-form tensor, one CTA per sample);
* the f manifold is diagonalised per sample (FP64 Householder + QL kernel),
  its eigenbasis tensor
  Kt_i o C is built in FP64 by ``qsx_fblock_tensor``, and two batched GEMMs
  bring M_i^f to the site basis in the working precision;
* t1 and the 'eg' t3 leg run in the batched RK4 kernels; the t2 leg applies
  P^k - I (P the RK4 step propagator of the 576-dimensional 'ee' block at 24
  sites), built by binary powering, to all t1 states at once;
* the 'fe' t3 leg (excited-state absorption) runs in the operator-form
  Heisenberg RK4 kernel;
* dipole super-operators are sample independent and applied as CSR maps;
  the t3 bra states are pulled back through V2 so that every pathway ends
  in one batched contraction against the 'ee' (and 'gg') t2 states.

Rephasing ('-++') and non-rephasing ('+-+') geometries share the t3 leg and
are evaluated together.
"""
import numpy as np
import torch

from .. import _native
from ..dynamics.redfield import RedfieldBuild, RedfieldModel
from ..operator_tools import occupation_table
from ..dynamics.liouville_space import liouville_subspace_index
from .ensemble import SampleBatch
from .utils import PRECISIONS, step_plan

ENGINE_GEOMETRIES = ('-++', '+-+')
PATHWAYS = {
    '-++': {'ESE': 'gg->ge->ee->eg->gg',
            'GSB': 'gg->ge->gg->eg->gg',
            'ESA': 'gg->ge->ee->fe->ee'},
    '+-+': {'ESE': 'gg->eg->ee->eg->gg',
            'GSB': 'gg->eg->gg->eg->gg',
            'ESA': 'gg->eg->ee->fe->ee'},
}


def supports(model, geometry):
    """Whether ``model`` and ``geometry`` run on the batched engine."""
    return (isinstance(model, RedfieldModel) and model.hilbert_subspace == 'gef'
            and not model.secular and model.evolve_basis == 'site'
            and geometry in ENGINE_GEOMETRIES
            and model.hamiltonian.n_vibrational_states == 1
            and 2 <= model.hamiltonian.n_sites <= 31)


def pair_tables(n_sites):
    """pair_sites (P, 2): the sites (k < l) of each two-exciton state in the
    all_states order (operator_tools.py:122-152); site_pairs (N, N-1): the pair
    states containing each site."""
    pairs = [(k, l) for k in range(n_sites) for l in range(k + 1, n_sites)]
    pair_sites = np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
    site_pairs = np.zeros((n_sites, n_sites - 1), dtype=np.int32)
    fill = np.zeros(n_sites, dtype=np.int64)
    for p, (k, l) in enumerate(pairs):
        site_pairs[k, fill[k]] = p
        fill[k] += 1
        site_pairs[l, fill[l]] = p
        fill[l] += 1
    return pair_sites, site_pairs


def powers_minus_identity(D, gaps):
    """{k: P^k - I} for P = I + D (batched), sharing one squaring chain.

    (I + X)(I + Y) - I = X + Y + X Y keeps the small part of each factor, so
    the powers lose no accuracy to cancellation against the identity.
    """
    out = {}
    todo = sorted({int(k) for k in gaps})
    acc = {k: None for k in todo}
    X = D
    bit = 1
    top = max(todo) if todo else 0
    while bit <= top:
        for k in todo:
            if k & bit:
                acc[k] = X if acc[k] is None else acc[k] + X + acc[k] @ X
        bit <<= 1
        if bit <= top:
            X = 2 * X + X @ X
    for k in todo:
        out[k] = acc[k] if acc[k] is not None else torch.zeros_like(D)
    return out


class ThirdOrderEngine:
    """Third-order response functions of a Redfield 'gef' model for a batch
    of disorder samples, both engine geometries at once.

    ``run(offsets)`` returns {geometry: (T1, T2, T3) complex128 tensor}, the
    sum over samples of each sample's response (response.py:297-336 summed
    over the selected pathways); divide by the sample count for the mean.
    """

    def __init__(self, model, coherence_time_max, population_times,
                 polarization='xxxx', include_signal=None, precision='fp32',
                 geometries=ENGINE_GEOMETRIES):
        for g in geometries:
            if not supports(model, g):
                raise NotImplementedError(
                    'the batched third-order engine needs a non-secular site-basis '
                    "RedfieldModel on 'gef' and geometry in {}".format(ENGINE_GEOMETRIES))
        self.model = model
        self.prec = PRECISIONS[precision]
        self.geometries = tuple(geometries)
        self.dt = model.time_step
        self.t1 = np.arange(0, coherence_time_max, self.dt)
        self.t3 = np.arange(0, coherence_time_max, self.dt)
        self.t2 = np.asarray(population_times, float)
        steps2 = step_plan(self.t2, 0.0, self.dt)
        self.gaps = np.diff(np.concatenate([[0], steps2])).astype(np.int64)
        self.polarization = polarization
        if include_signal is None:
            include_signal = ('GSB', 'ESE', 'ESA')
        elif isinstance(include_signal, str):
            include_signal = tuple(s.strip() for s in include_signal.split(','))
        self.signals = [s for s in ('GSB', 'ESE', 'ESA') if s in include_signal]
        if not self.signals:
            raise ValueError('at least one Liouville space pathway must be selected, '
                             "i.e., include_signal must include at least one of "
                             "['ESE', 'GSB', 'ESA']")
        ham = model.hamiltonian
        self.N = ham.n_sites
        self.P = self.N * (self.N - 1) // 2
        self._maps = {}

    # ----------------------------------------------------------- host setup
    def _idx(self, sub):
        return liouville_subspace_index(sub, 'ge', self.N)

    def _op(self, spec, pol, tr):
        key = (spec, pol, tr)
        if key not in self._maps:
            self._maps[key] = self.model.dipole_operator(spec, pol, tr)
        return self._maps[key]

    def _csr(self, spec, pol, tr, transpose=False):
        key = ('csr', spec, pol, tr, transpose)
        if key not in self._maps:
            m = self._op(spec, pol, tr).commutator_matrix
            self._maps[key] = _native.CsrMap(m.T if transpose else m)
        return self._maps[key]

    def _bra(self, spec, pol, tr):
        v = self._op(spec, pol, tr).bra_vector
        return torch.as_tensor(np.asarray(v, dtype=complex), dtype=torch.complex128).cuda()

    # -------------------------------------------------------------- builds
    def _f_operators(self, batch, build_e, cdt):
        """Q (S, P, N, P) column operators of the 'fe' block in precision."""
        model, N, P = self.model, self.N, self.P
        ham = model.hamiltonian
        pair_sites, site_pairs = pair_tables(N)
        self._pair_sites = torch.as_tensor(pair_sites).cuda()
        sp = torch.as_tensor(site_pairs).cuda()
        Hf = batch.H('f')
        Ef, Uf = _native.eigh_large(Hf)
        Y = _native.fblock_tensor(Ef, Uf, N, sp, ham.bath, model.unit_convert, self.prec,
                                  model.discard_imag_corr,
                                  ham.bath.matsubara_cutoff)
        S = Y.shape[0]
        U = Uf.to(Y.dtype)
        T = torch.bmm(U, Y.view(S, P, 2 * N * P))
        del Y
        Mf = torch.bmm(T.view(S, P * 2 * N, P), U.transpose(1, 2))
        del T
        Q = _native.fe_generator(Mf.view(S, P, 2 * N, P).contiguous(), Hf.contiguous(),
                                 self._pair_sites, model.unit_convert, self.prec)
        return Q

    # ----------------------------------------------------------------- run
    def run(self, offsets, events=None):
        """Summed response over the samples with the given site-energy offsets
        ((S, N) float64, CUDA or host)."""
        _native.require_gpu()
        model, N = self.model, self.N
        prec = self.prec
        cdt = torch.complex64 if prec == _native.QSX_FP32 else torch.complex128
        uc, dt = model.unit_convert, self.dt
        pol = self.polarization
        S = len(offsets)
        batch = SampleBatch(model, S, offsets=offsets)
        ham = model.hamiltonian
        _tick(events, 'build')
        Hge = batch.H('ge')
        build = RedfieldBuild(Hge, N, 'ge', occupation_table(N, 'ge'), ham.bath, uc,
                              False, model.discard_imag_corr, 'site')
        need_fe = 'ESA' in self.signals
        if need_fe:
            Me = build.M[:, :, 1:, 1:].to(cdt).contiguous()
            Ae = (build.G[:, 1:, 1:] + 1j * uc * Hge[:, 1:, 1:]).to(cdt).contiguous()
            Q = self._f_operators(batch, build, cdt)
        _tick(events, 't3')
        # ---- t3 legs (Heisenberg picture), shared by the geometries
        T3 = len(self.t3)
        y_eg = self._bra('eg->gg', pol[3], '-')
        D3 = build.propagator(self._idx('eg'), dt, prec, transpose=True)
        v_eg = _native.rk4(D3, y_eg, T3 - 1, 1, h=dt, precision=prec,
                           state=True)['state']                       # (S, T3, N)
        W = None
        if 'ESE' in self.signals:
            W = self._csr('ee->eg', pol[2], '+', transpose=True)(v_eg)  # (S, T3, N^2)
        if need_fe:
            y_fe = self._bra('fe->ee', pol[3], '-')
            v_fe = _native.fe_heisenberg_rk4(Q, Ae, Me, self._pair_sites, y_fe, T3 - 1, dt,
                                             prec)                     # (S, T3, P N)
            del Q
            w = self._csr('ee->fe', pol[2], '+', transpose=True)(v_fe)
            del v_fe
            W = w if W is None else W + w
        g3 = None
        if 'GSB' in self.signals:
            g3 = self._csr('gg->eg', pol[2], '+', transpose=True)(v_eg)[..., 0]  # (S, T3)
        _tick(events, 't2')
        # ---- t2 propagator powers on the 'ee' block
        gaps = [int(k) for k in self.gaps]
        # P^g - I for g = gcd of the gaps; each gap then applies it gap/g
        # times to the (S, T1, N^2) block of t1 states (a matrix-block product
        # costs T1/N^2 of a matrix-matrix product)
        base = int(np.gcd.reduce([k for k in gaps if k] or [1]))
        Xg = None
        if W is not None and any(gaps):
            Lee = build.block(self._idx('ee'))
            A = (dt * Lee).to(cdt)
            del Lee
            A2 = A @ A
            D = A + 0.5 * A2 + A2 @ (A / 6 + A2 / 24)
            del A, A2
            Xg = powers_minus_identity(D, [base])[base].transpose(1, 2).contiguous()
            del D
        Dgg = build.propagator(self._idx('gg'), dt, prec)[:, 0, 0] if g3 is not None else None
        _tick(events, 't1')
        out = {}
        T1 = len(self.t1)
        for geo in self.geometries:
            sub1 = 'ge' if geo == '-++' else 'eg'
            rho0 = torch.ones(1, dtype=torch.complex128, device='cuda')
            v0 = self._csr('gg->' + sub1, pol[0], geo[0])(rho0)         # (N,)
            D1 = build.propagator(self._idx(sub1), dt, prec)
            rho1 = _native.rk4(D1, v0, T1 - 1, 1, h=dt, precision=prec,
                               state=True)['state']                     # (S, T1, N)
            total = torch.zeros((T1, len(gaps), T3), dtype=torch.complex128, device='cuda')
            if W is not None:
                r = self._csr(sub1 + '->ee', pol[1], geo[1])(rho1).to(cdt)  # (S, T1, N^2)
                Wt = W.to(cdt).transpose(1, 2)                           # (S, N^2, T3)
                for j, k in enumerate(gaps):
                    for _ in range(k // base):
                        r = r + torch.bmm(r, Xg)
                    total[:, j, :] += torch.bmm(r, Wt).to(torch.complex128).sum(0)
            if g3 is not None:
                rgg = self._csr(sub1 + '->gg', pol[1], geo[1])(rho1)[..., 0]  # (S, T1)
                for j, k in enumerate(gaps):
                    if k:
                        rgg = rgg * (1 + Dgg[:, None]) ** k
                    total[:, j, :] += torch.einsum('sa,sc->ac', rgg, g3)
            out[geo] = total
        _tick(events, 'end')
        return out


def _tick(events, name):
    if events is not None:
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        events.setdefault('marks', []).append((name, e))


def third_order_ensemble(model, coherence_time_max, population_times, geometry='-++',
                         polarization='xxxx', include_signal=None, ensemble_size=None,
                         precision='fp64', chunk=None):
    """(t1, t2, t3), mean response of one geometry over the disorder samples
    0 .. ensemble_size-1 (or of the model itself when ensemble_size is None)."""
    eng = ThirdOrderEngine(model, coherence_time_max, population_times, polarization,
                           include_signal, precision, geometries=(geometry,))
    ham = model.hamiltonian
    if ensemble_size is None:
        offsets = np.zeros((1, ham.n_sites))
        count = 1
    else:
        offsets = ham.disorder_offsets(ensemble_size)
        count = ensemble_size
    chunk = chunk or len(offsets)
    total = None
    for s0 in range(0, len(offsets), chunk):
        part = eng.run(offsets[s0:s0 + chunk])[geometry]
        total = part if total is None else total + part
    return (eng.t1, eng.t2, eng.t3), (total / count).cpu().numpy()
