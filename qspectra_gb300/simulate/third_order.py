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

Orientation averages reuse the legs.  The response is linear in each
pulse's polarization vector, so it is written over lab-frame channels:
R = sum T[a, b, c, d] R(e_a, e_b, e_c, e_d).  A fixed polarization is one
channel per pulse; random ensemble orientations make that channel's vector
per sample (R_s^T e); the exact isotropic average (decorators.py:67-92)
takes the three axes per pulse with T the invariant weights.  The t1 leg
then runs once per first-pulse channel, the t3 legs once per last-pulse
channel, and only the nine (a, b) t2 products meet the nine (c, d) t3
states, where the reference re-runs all pathways for each of up to 21
polarizations.
"""
import numpy as np
import torch

from .. import _native
from ..dynamics.redfield import RedfieldBuild, RedfieldModel
from ..operator_tools import occupation_table
from ..dynamics.liouville_space import liouville_subspace_index
from ..polarization import check_polarizations, isotropic_tensor_4th_order
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


def _gemm_add(A, B, C):
    return _native.gemm(A, B, Cin=C)


def powers_minus_identity(D, gaps, mul_add=_gemm_add):
    """{k: P^k - I} for P = I + D (batched), sharing one squaring chain.

    (I + X)(I + Y) - I = X + Y + X Y keeps the small part of each factor, so
    the powers lose no accuracy to cancellation against the identity.
    ``mul_add(A, B, C)`` returns A B + C; the default runs qsx_gemm_batched
    (tensor cores for FP32).
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
                # acc + X + acc X
                acc[k] = X if acc[k] is None else mul_add(acc[k], X, acc[k] + X)
        bit <<= 1
        if bit <= top:
            X = mul_add(X, X, 2 * X)   # 2 X + X X
    for k in todo:
        out[k] = acc[k] if acc[k] is not None else torch.zeros_like(D)
    return out


class ThirdOrderEngine:
    """Third-order response functions of a Redfield 'gef' model for a batch
    of disorder samples, both engine geometries at once.

    ``run(offsets)`` returns {geometry: (T1, T2, T3) complex128 tensor}, the
    sum over samples of each sample's response (response.py:297-336 summed
    over the selected pathways); divide by the sample count for the mean.
    ``isotropic`` evaluates the exact isotropic average for the given lab
    polarizations; ``run(offsets, rotations)`` rotates each sample's dipoles.
    """

    def __init__(self, model, coherence_time_max, population_times,
                 polarization='xxxx', include_signal=None, precision='fp32',
                 geometries=ENGINE_GEOMETRIES, isotropic=False):
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
        pols = check_polarizations(polarization, 4)
        if isotropic:
            self.lab = None
            self.coupling = isotropic_tensor_4th_order(polarization)
        else:
            self.lab = pols
            self.coupling = np.ones((1, 1, 1, 1))
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
            self._maps[key] = self.model.dipole_operator(spec, np.asarray(pol, float), tr)
        return self._maps[key]

    def _csr(self, spec, pol, tr, transpose=False):
        key = ('csr', spec, pol, tr, transpose)
        if key not in self._maps:
            m = self._op(spec, pol, tr).commutator_matrix
            self._maps[key] = _native.CsrMap(m.T if transpose else m)
        return self._maps[key]

    def _channels(self, S, rotations):
        """Per pulse, its channels' polarization vectors: a shared tuple, or an
        (S, 3) CUDA tensor when the dipoles are rotated per sample."""
        axes = np.eye(3) if self.lab is None else None
        out = []
        for k in range(4):
            vecs = axes if axes is not None else self.lab[k:k + 1]
            if rotations is None:
                out.append([tuple(float(x) for x in v) for v in vecs])
            else:
                q = np.einsum('sji,cj->csi', rotations, vecs)          # (C, S, 3)
                out.append([torch.as_tensor(qc).cuda() for qc in q])
        return out

    def _apply(self, spec, tr, vec, x, transpose=False):
        """Map of polarization ``vec`` applied to x (S, ..., n_in): one CSR map
        for a shared vector, a per-sample mix of the three axis maps otherwise."""
        if isinstance(vec, tuple):
            return self._csr(spec, vec, tr, transpose)(x)
        out = None
        shape = (x.shape[0],) + (1,) * (x.dim() - 1)
        for a in range(3):
            y = self._csr(spec, tuple(np.eye(3)[a]), tr, transpose)(x)
            y = y * vec[:, a].view(shape)
            out = y if out is None else out + y
        return out

    def _bra(self, spec, vec, tr, S):
        """Bra vector of the dipole operator: (n,) shared or (S, n) per sample."""
        if isinstance(vec, tuple):
            v = self._op(spec, vec, tr).bra_vector
            return torch.as_tensor(np.asarray(v, dtype=complex),
                                   dtype=torch.complex128).cuda()
        basis = torch.as_tensor(np.array(
            [np.asarray(self._op(spec, tuple(np.eye(3)[a]), tr).bra_vector, dtype=complex)
             for a in range(3)]), dtype=torch.complex128).cuda()
        return (vec.to(basis.dtype)[:, :, None] * basis[None]).sum(1).contiguous()

    def _ket0(self, spec, vec, tr):
        """Dipole commutator on the ground state: (n,) or (S, n)."""
        rho0 = torch.ones(1, dtype=torch.complex128, device='cuda')
        if isinstance(vec, tuple):
            return self._csr(spec, vec, tr)(rho0)
        basis = torch.stack([self._csr(spec, tuple(np.eye(3)[a]), tr)(rho0)
                             for a in range(3)])
        return (vec.to(basis.dtype)[:, :, None] * basis[None]).sum(1).contiguous()

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
        # M_q = U Y_q U^T for the 2N real planes q (real and imaginary parts):
        # U times all Y_q side by side, then every T_q times U^T, real
        # products in the working precision (qsx_gemm_batched)
        U = Uf.to(Y.dtype).contiguous()
        T = _native.gemm(U, Y.view(S, P, 2 * N * P))
        del Y
        Mf = _native.gemm(T.view(S, P * 2 * N, P), U.transpose(1, 2).contiguous())
        del T
        Q = _native.fe_generator(Mf.view(S, P, 2 * N, P).contiguous(), Hf.contiguous(),
                                 self._pair_sites, model.unit_convert, self.prec)
        return Q

    # ----------------------------------------------------------------- run
    def run(self, offsets, events=None, rotations=None):
        """Summed response over the samples with the given site-energy offsets
        ((S, N) float64, CUDA or host); ``rotations`` (S, 3, 3) rotates each
        sample's dipoles."""
        _native.require_gpu()
        model, N = self.model, self.N
        prec = self.prec
        cdt = torch.complex64 if prec == _native.QSX_FP32 else torch.complex128
        uc, dt = model.unit_convert, self.dt
        S = len(offsets)
        ch = self._channels(S, None if rotations is None else np.asarray(rotations, float))
        Tw = self.coupling
        # (a, b) x (c, d) channel pairs that meet with a nonzero weight
        left = [(a, b) for a in range(Tw.shape[0]) for b in range(Tw.shape[1])
                if np.any(Tw[a, b])]
        right = sorted({(c, d) for a, b in left for c in range(Tw.shape[2])
                        for d in range(Tw.shape[3]) if Tw[a, b, c, d]})
        ch0 = sorted({a for a, _ in left})
        ch3 = sorted({d for _, d in right})
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
        D3 = build.propagator(self._idx('eg'), dt, prec, transpose=True)
        v_eg, v_fe = {}, {}
        for d in ch3:
            y_eg = self._bra('eg->gg', ch[3][d], '-', S)
            v_eg[d] = _native.rk4(D3, y_eg, T3 - 1, 1, h=dt, precision=prec,
                                  state=True)['state']                    # (S, T3, N)
            if need_fe:
                y_fe = self._bra('fe->ee', ch[3][d], '-', S)
                v_fe[d] = _native.fe_heisenberg_rk4(Q, Ae, Me, self._pair_sites, y_fe,
                                                    T3 - 1, dt, prec)     # (S, T3, P N)
        if need_fe:
            del Q
        W, g3 = {}, {}
        for c, d in right:
            w = None
            if 'ESE' in self.signals:
                w = self._apply('ee->eg', '+', ch[2][c], v_eg[d], transpose=True)
            if need_fe:
                wf = self._apply('ee->fe', '+', ch[2][c], v_fe[d], transpose=True)
                w = wf if w is None else w + wf
            if w is not None:
                W[c, d] = w                                               # (S, T3, N^2)
            if 'GSB' in self.signals:
                g3[c, d] = self._apply('gg->eg', '+', ch[2][c], v_eg[d],
                                       transpose=True)[..., 0]            # (S, T3)
        del v_fe
        # t3 states of each (a, b) channel pair, weighted by the coupling
        Wc, gc = [], []
        for a, b in left:
            terms = [(Tw[a, b, c, d], cd) for cd in right for c, d in [cd] if Tw[a, b, c, d]]
            if W:
                Wc.append(sum(float(t) * W[cd] for t, cd in terms).to(cdt).transpose(1, 2))
            if g3:
                gc.append(sum(float(t) * g3[cd] for t, cd in terms))
        del W
        Wt = torch.stack(Wc, 1).contiguous() if Wc else None          # (S, L, N^2, T3)
        _tick(events, 't2')
        # ---- t2 propagator powers on the 'ee' block
        gaps = [int(k) for k in self.gaps]
        # P^g - I for g = gcd of the gaps; each gap then applies it gap/g
        # times to the (S, L T1, N^2) block of t1 states (a matrix-block
        # product costs L T1/N^2 of a matrix-matrix product)
        base = int(np.gcd.reduce([k for k in gaps if k] or [1]))
        Xg = None
        if Wt is not None and any(gaps):
            # the ee block maps Hermitian matrices to Hermitian matrices (real
            # symmetric site-basis Hamiltonian), so its powers run in the real
            # form (Hermitian coordinates): real products, a quarter of the
            # complex multiply-adds
            Lee = build.block(self._idx('ee'))
            A = _native.hermitian_real_form((dt * Lee).to(cdt), N)
            del Lee
            A2 = _native.gemm(A, A)
            # D = A + A^2 / 2 + A^2 (A / 6 + A^2 / 24), one step of RK4
            D = _native.gemm(A2, A / 6 + A2 / 24, Cin=A + 0.5 * A2)
            del A, A2
            Xg = powers_minus_identity(D, [base])[base].transpose(1, 2).contiguous()
            del D
        Dgg = build.propagator(self._idx('gg'), dt, prec)[:, 0, 0] if gc else None
        _tick(events, 't1')
        out = {}
        T1 = len(self.t1)
        nL = len(left)
        for geo in self.geometries:
            sub1 = 'ge' if geo == '-++' else 'eg'
            D1 = build.propagator(self._idx(sub1), dt, prec)
            rho1 = {}
            for a in ch0:
                v0 = self._ket0('gg->' + sub1, ch[0][a], geo[0])          # (N,) / (S, N)
                rho1[a] = _native.rk4(D1, v0, T1 - 1, 1, h=dt, precision=prec,
                                      state=True)['state']                 # (S, T1, N)
            total = torch.zeros((T1, len(gaps), T3), dtype=torch.complex128, device='cuda')
            if Wt is not None:
                r = torch.stack([self._apply(sub1 + '->ee', geo[1], ch[1][b], rho1[a])
                                 for a, b in left], 1).to(cdt)             # (S, L, T1, N^2)
                r = r.view(S, nL * T1, N * N)
                Wv = Wt.view(S * nL, N * N, T3)
                # the t1 states as coordinates of their Hermitian and
                # anti-Hermitian parts, propagated by the real powers
                x = _native.hermitian_rows(r, N)                      # (S, 2 L T1, N^2)
                for j, k in enumerate(gaps):
                    for _ in range(k // base):
                        x = _native.gemm(x, Xg, Cin=x)          # x (I + X_g)
                    rk = _native.hermitian_rows(x, N, merge=True)
                    part = _native.gemm(rk.view(S * nL, T1, N * N), Wv)
                    total[:, j, :] += part.to(torch.complex128).sum(0)
            if gc:
                for (a, b), g in zip(left, gc):
                    rgg = self._apply(sub1 + '->gg', geo[1], ch[1][b], rho1[a])[..., 0]
                    for j, k in enumerate(gaps):
                        if k:
                            rgg = rgg * (1 + Dgg[:, None]) ** k
                        # sum over samples of rgg[s, a] g[s, c]
                        total[:, j, :] += _native.gemm(rgg.t().contiguous(),
                                                       g.contiguous())[0]
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
                         precision='fp64', chunk=None, isotropic=False,
                         random_orientations=False):
    """(t1, t2, t3), mean response of one geometry over the disorder samples
    0 .. ensemble_size-1 (or of the model itself when ensemble_size is None).
    ``isotropic`` gives the exact isotropic average; ``random_orientations``
    rotates each sample's dipoles with the reference's draws."""
    eng = ThirdOrderEngine(model, coherence_time_max, population_times, polarization,
                           include_signal, precision, geometries=(geometry,),
                           isotropic=isotropic)
    ham = model.hamiltonian
    rotations = None
    if ensemble_size is None:
        offsets = np.zeros((1, ham.n_sites))
        count = 1
    else:
        offsets = ham.disorder_offsets(ensemble_size)
        count = ensemble_size
        if random_orientations:
            rotations = ham.orientation_rotations(ensemble_size)
    chunk = chunk or len(offsets)
    total = None
    for s0 in range(0, len(offsets), chunk):
        rot = None if rotations is None else rotations[s0:s0 + chunk]
        part = eng.run(offsets[s0:s0 + chunk], rotations=rot)[geometry]
        total = part if total is None else total + part
    return (eng.t1, eng.t2, eng.t3), (total / count).cpu().numpy()
