"""Batched disorder ensembles on one GPU.

The reference averages over static disorder with a serial Python loop, one
full model rebuild and zvode solve per sample (decorators.py:40-64,
hamiltonian.py:233-274).  Here every sample's rotating-frame Hamiltonian is
built on the device, the Redfield generators for all samples are produced by
one batched build, their RK4 propagators by one kernel, and the time loops of
all samples run in one persistent kernel that also reduces the ensemble mean.
"""
import numpy as np
import torch

from .. import _native
from ..dynamics.redfield import RedfieldModel
from ..operator_tools import hilbert_subspace_index


class SampleBatch:
    """Disorder samples n = start .. start + size - 1 of a model's Hamiltonian.

    ``offsets`` holds the diagonal site-energy shifts (the same RandomState
    draws as ``sample(n)``); ``H(subspace)`` returns the (S, n, n) float64
    rotating-frame Hamiltonians on the GPU.
    """

    def __init__(self, model, size, start=0, offsets=None):
        self.model = model
        self.size = int(size)
        self.start = int(start)
        ham = model.hamiltonian
        if offsets is None:
            offsets = ham.disorder_offsets(size, start)
        if isinstance(offsets, torch.Tensor):
            self.offsets = offsets.to(device='cuda', dtype=torch.float64)
        else:
            self.offsets = torch.as_tensor(np.asarray(offsets, float),
                                           dtype=torch.float64).cuda()

    def H(self, subspace):
        ham = self.model.hamiltonian
        base = torch.as_tensor(ham.H(subspace), dtype=torch.float64).cuda()
        n = base.shape[0]
        H = base.expand(self.size, n, n).clone()
        if 'e' in subspace:
            sl = hilbert_subspace_index('e', subspace, ham.n_sites)
            idx = torch.arange(sl.start, sl.stop, device=H.device)
            H[:, idx, idx] += self.offsets
        if 'f' in subspace:
            sl = hilbert_subspace_index('f', subspace, ham.n_sites)
            pairs = [(i, j) for i in range(ham.n_sites) for j in range(i + 1, ham.n_sites)]
            ii = torch.as_tensor([p[0] for p in pairs], device=H.device)
            jj = torch.as_tensor([p[1] for p in pairs], device=H.device)
            idx = torch.arange(sl.start, sl.stop, device=H.device)
            H[:, idx, idx] += self.offsets[:, ii] + self.offsets[:, jj]
        return H.contiguous()


ROWS_KERNEL_SIZES = (9, 16, 25, 36, 49, 64)


def pick_block_k(nsteps, m, nselect, max_k=9):
    """Largest K <= max_k dividing nsteps for the K-step blocked FP32 loop (1 = none)."""
    if m not in ROWS_KERNEL_SIZES:
        return 1
    for K in range(max_k, 1, -1):
        if nsteps % K == 0 and m + nselect * (K - 1) <= 256:
            return K
    return 1


# Autotuned time-loop variants (qsx_rk4_args.variant) per (m, K, selected
# components, batch-size octave): each candidate is timed once on the first
# call's own inputs and the fastest is kept for the process.
BLOCK_VARIANTS = (1, 2, 5)
_TUNED = {}
_PINNED = None


def set_block_variant(variant=None):
    """Pin the blocked time-loop variant (1..5), or None to autotune."""
    global _PINNED
    _PINNED = variant


def tuned_block_variant(mat, y0, nsteps, select, K):
    if _PINNED is not None:
        return _PINNED
    key = (int(mat.shape[-1]), int(K), len(select), int(np.log2(max(int(mat.shape[0]), 1))))
    if key not in _TUNED:
        best, best_ms = 1, None
        for v in BLOCK_VARIANTS:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            try:
                _native.rk4(mat, y0, nsteps, 1, select=select, per_sample=False, mean=True,
                            check_finite=False, block_k=K, variant=v)
            except _native.QsxError:
                continue  # a variant this shape cannot launch is never chosen
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            if best_ms is None or ms < best_ms:
                best, best_ms = v, ms
        _TUNED[key] = best
    return _TUNED[key]


def propagate_selected_mean(D, y0, nsteps, select, precision, events=None):
    """Ensemble mean of the selected components at every step (GPU).

    FP32 runs use the K-step blocked loop when the step count allows it.
    ``events`` (a dict) receives CUDA events around the time loop and the
    matrix-vector work it executed ('flops').
    """
    K = pick_block_k(nsteps, D.shape[-1], len(select)) if precision == _native.QSX_FP32 else 1
    B, m = D.shape[0], D.shape[-1]
    mat = _native.rk4_block_matrix(D, K, select) if K > 1 else D
    rows = mat.shape[-2]
    variant = tuned_block_variant(mat, y0, nsteps, select, K) if K > 1 else 0
    if events is not None:
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record()
    out = _native.rk4(mat, y0, nsteps, 1, select=select, per_sample=False, mean=True,
                      check_finite=False, block_k=K if K > 1 else 0, variant=variant)
    if events is not None:
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record()
        events.setdefault('dyn', []).append((e0, e1))
        # complex multiply-adds of the executed form, 8 real flops each
        events['dyn_flops'] = 8.0 * B * (nsteps // K) * rows * m
        events['dyn_block_k'] = K
        events['dyn_variant'] = variant
    return out


# The real (Hermitian) form of diagonal population blocks: on by default for
# FP32 ensembles; set_hermitian_form(False) keeps the complex blocked loop.
_HERMITIAN = True


def set_hermitian_form(enabled=True):
    global _HERMITIAN
    _HERMITIAN = bool(enabled)


def hermitian_coordinates(y, n):
    """Real coordinates x[a + n b] = Re rho_ab (a <= b), Im rho_ba (a > b) of
    column-stacked n x n Hermitian matrices y (..., n^2) (numpy or torch)."""
    a, b = np.divmod(np.arange(n * n), n)[::-1]
    src = np.where(a <= b, a + n * b, b + n * a)
    take_re = a <= b
    if isinstance(y, torch.Tensor):
        v = y[..., _native.const_tensor(src, torch.int64, y.device)]
        return torch.where(_native.const_tensor(take_re, torch.bool, y.device), v.real, v.imag)
    v = np.asarray(y)[..., src]
    return np.where(take_re, v.real, v.imag)


def from_hermitian_coordinates(x, n):
    """Column-stacked complex matrices from Hermitian coordinates (inverse of
    hermitian_coordinates); x (..., n^2) real, numpy or torch."""
    a, b = np.divmod(np.arange(n * n), n)[::-1]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    re_idx = lo + n * hi
    im_idx = hi + n * lo
    sign = np.where(a < b, 1.0, np.where(a > b, -1.0, 0.0))
    if isinstance(x, torch.Tensor):
        dev = x.device
        re = x[..., _native.const_tensor(re_idx, torch.int64, dev)]
        im = (x[..., _native.const_tensor(im_idx, torch.int64, dev)]
              * _native.const_tensor(sign, x.dtype, dev))
        return torch.complex(re, im)
    x = np.asarray(x)
    return x[..., re_idx] + 1j * sign * x[..., im_idx]


def padded_block_steps(nsteps, K):
    """Steps the real blocked loop runs for block size K: the smallest
    multiple of K that covers ``nsteps`` (the outputs past ``nsteps`` are
    dropped; the ones up to it are the same as for any other K)."""
    return -(-int(nsteps) // K) * K


def _block_k_real_cost(nsteps, m, nselect, K, tensor_core):
    products = bin(K).count('1') - 1 + K.bit_length() - 1
    build = nselect * m * m * max(K - 2, 0) + products * m ** 3
    if tensor_core is not None and tensor_core(K):
        build *= 0.6
    nblk = padded_block_steps(nsteps, K) // K
    return 2.0 * nblk * (m + nselect * (K - 1)) * m + build


def pick_block_k_real(nsteps, m, nselect, max_k=64, tensor_core=None):
    """K minimising the executed work of the real blocked loop: per block-step
    (m + nsel (K-1)) m multiply-adds (weighted twice: the loop is the
    latency-bound part) over ceil(nsteps / K) block-steps, plus the block
    build, nsel m^2 (K-2) for the selected rows and m^3 per product of the
    binary powering.  Where ``tensor_core(K)`` says the tcgen05 build takes
    K, the build terms weigh 0.6 (its measured time against the CUDA-core
    build at K = 9).  K need not divide nsteps: the loop runs
    padded_block_steps(nsteps, K) steps, at most K - 1 more."""
    best, best_cost = 1, None
    for K in range(2, min(max_k, max(int(nsteps), 1)) + 1):
        if m + nselect * (K - 1) > 512:
            continue
        cost = _block_k_real_cost(nsteps, m, nselect, K, tensor_core)
        if best_cost is None or cost < best_cost:
            best, best_cost = K, cost
    return best


# Measured choice of K for the real blocked loop: the candidates the cost
# model ranks best are timed once (block build plus loop, on the first call's
# own inputs) per (m, selected coordinates, steps, batch octave), and the
# fastest is kept for the process.  set_block_k_real(K) pins a value.
_TUNED_K_REAL = {}
_PINNED_K_REAL = None
K_REAL_CANDIDATES = 5


def set_block_k_real(K=None):
    """Pin the real blocked loop's K (None: tune by measurement)."""
    global _PINNED_K_REAL
    _PINNED_K_REAL = K


def block_k_real_candidates(nsteps, m, nselect, tensor_core=None, count=K_REAL_CANDIDATES):
    """The ``count`` K values the cost model of pick_block_k_real ranks best."""
    ranked = []
    for K in range(2, min(64, max(int(nsteps), 1)) + 1):
        if m + nselect * (K - 1) > 512:
            continue
        ranked.append((_block_k_real_cost(nsteps, m, nselect, K, tensor_core), K))
    return [K for _, K in sorted(ranked)[:count]]


def _real_block_pass(Dr, K, coords, x0, nsteps, use_tc):
    tc = _native.rk4_block_matrix_real_tc(Dr, K, coords) if use_tc else None
    if tc is not None:
        mat, tc_status = tc
    else:
        mat, tc_status = _native.rk4_block_matrix_real(Dr, K, coords), None
    xm, status = _native.rk4_real_block_mean(mat, x0, padded_block_steps(nsteps, K), coords, K,
                                             check_finite=False)
    return mat, tc_status, xm[:nsteps + 1], status


def tuned_block_k_real(Dr, coords, x0, nsteps, use_tc):
    """K for the real blocked loop: pinned, measured once per shape, or (while
    a CUDA graph is being captured, where nothing can be timed) the model's."""
    m = int(Dr.shape[-1])
    tcf = ((lambda k: _native.rk4_block_matrix_real_tc_supported(m, k, len(coords)))
           if use_tc else None)
    if _PINNED_K_REAL is not None:
        return _PINNED_K_REAL
    key = (m, len(coords), int(nsteps), int(np.log2(max(int(Dr.shape[0]), 1))), bool(use_tc))
    if key in _TUNED_K_REAL:
        return _TUNED_K_REAL[key][0]
    cands = block_k_real_candidates(nsteps, m, len(coords), tcf)
    if not cands:
        return 1
    if len(cands) == 1 or torch.cuda.is_current_stream_capturing():
        return cands[0]
    times = {}
    for K in cands:
        use = use_tc and bool(tcf(K))
        _real_block_pass(Dr, K, coords, x0, nsteps, use)     # warm
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _real_block_pass(Dr, K, coords, x0, nsteps, use)
        e1.record()
        e1.synchronize()
        times[K] = e0.elapsed_time(e1)
    best = min(times, key=times.get)
    _TUNED_K_REAL[key] = (best, times)
    return best


def block_k_real_timings():
    """{shape key: (chosen K, {K: ms})} of the measured choices so far."""
    return dict(_TUNED_K_REAL)


def hermitian_block_size(idx, n_total):
    """nb when the column-stacked indices ``idx`` form one diagonal block of
    nb x nb states (e.g. 'ee'), else None."""
    idx = np.asarray(idx)
    rows, cols = idx % n_total, idx // n_total
    states = np.unique(rows)
    nb = len(states)
    if nb * nb != len(idx) or not np.array_equal(np.unique(cols), states):
        return None
    expect = (states[None, :] + n_total * states[:, None]).reshape(-1)
    return nb if np.array_equal(np.sort(idx), np.sort(expect)) else None


# FP32 blocked matrices on the tensor cores (3xTF32 tcgen05 products) where
# the shape allows; the CUDA-core kernel otherwise.
_TENSOR_CORE_BLOCKS = True


def propagate_hermitian_mean(build, idx, nb, h, y0, nsteps, select, events=None, x0=None):
    """FP32 ensemble mean of the selected components of a Hermitian diagonal
    block through its real form: real propagator, real K-step blocked matrix
    (tcgen05 3xTF32 products when the shape allows) and real blocked loop.
    Returns {'mean': (nsteps + 1, len(select)) complex128, 'status'} like
    propagate_selected_mean; when every selected component is a population
    (diagonal), 'mean_real' holds the same values as float64 without the
    complex reconstruction.  ``x0`` may pass the Hermitian coordinates of
    y0 (hermitian_coordinates) when the caller keeps them."""
    m = nb * nb
    sel = np.asarray(select, dtype=np.int64)
    a, b = sel % nb, sel // nb
    partner = np.where(a == b, sel, b + nb * a)
    coords = np.unique(np.concatenate([sel, partner]))
    Dr = build.hermitian_propagator(idx, nb, h)
    use_tc = _TENSOR_CORE_BLOCKS and Dr.dtype == torch.float32
    if x0 is None:
        x0 = hermitian_coordinates(y0, nb)
    K = tuned_block_k_real(Dr, coords, x0, nsteps, use_tc)
    use_tc = use_tc and bool(_native.rk4_block_matrix_real_tc_supported(m, K, len(coords)))
    if events is not None:
        b0 = torch.cuda.Event(enable_timing=True)
        b0.record()
    tc = _native.rk4_block_matrix_real_tc(Dr, K, coords) if use_tc else None
    if tc is not None:
        mat, tc_status = tc
    else:
        mat, tc_status = _native.rk4_block_matrix_real(Dr, K, coords), None
    if events is not None:
        b1 = torch.cuda.Event(enable_timing=True)
        b1.record()
        events.setdefault('blockbuild', []).append((b0, b1))
        events['blockbuild_variant'] = 'tcgen05' if tc is not None else 'cuda_core'
        events['blockbuild_shape'] = (Dr.shape[0], m, K, len(coords))
        # real multiply-adds of the unpadded products: the squares and the
        # final composition of the binary powering (m^3 each) and the
        # selected rows R_2 .. R_{K-1} (nsel m^2 each), 2 flops apiece
        products = (K.bit_length() - 1) + (bin(K).count('1') - 1)
        events['blockbuild_flops'] = 2.0 * Dr.shape[0] * (
            products * m ** 3 + max(K - 2, 0) * len(coords) * m * m)
    del Dr
    if events is not None:
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record()
    if K > 1:
        # the loop runs whole blocks; the outputs past nsteps are dropped
        xm, status = _native.rk4_real_block_mean(mat, x0, padded_block_steps(nsteps, K), coords,
                                                 K, check_finite=False)
        xm = xm[:nsteps + 1]
    else:
        raise NotImplementedError('the real blocked loop needs a block size K > 1')
    if tc_status is not None:
        status = status | tc_status
    if events is not None:
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record()
        events.setdefault('dyn', []).append((e0, e1))
        events['dyn_flops'] = (2.0 * mat.shape[0] * (padded_block_steps(nsteps, K) // K)
                               * mat.shape[1] * m)
        events['dyn_block_k'] = K
        events['dyn_variant'] = 'real'
    if np.all(a == b) and np.array_equal(coords, sel):
        # populations: the coordinates are the values themselves
        return {'mean_real': xm, 'status': status}
    full = torch.zeros((xm.shape[0], m), dtype=torch.float64, device=xm.device)
    full[:, _native.const_tensor(coords, torch.int64, xm.device)] = xm
    y = from_hermitian_coordinates(full, nb)
    return {'mean': y[:, _native.const_tensor(sel, torch.int64, xm.device)], 'status': status}


def can_use_hermitian(precision, idx, n_total, y0, nsteps):
    """Whether the real Hermitian form applies: FP32, a diagonal block of
    3..8 states, a Hermitian initial state and at least one K > 1."""
    if not _HERMITIAN or precision != _native.QSX_FP32:
        return None
    nb = hermitian_block_size(idx, n_total)
    if nb is None or not 3 <= nb <= 8:
        return None
    y = y0.detach().cpu().numpy() if isinstance(y0, torch.Tensor) else np.asarray(y0)
    if y.ndim != 1:
        return None
    rho = y.reshape(nb, nb, order='F')
    if np.abs(rho - rho.conj().T).max() > 1e-14 * max(np.abs(rho).max(), 1e-300):
        return None
    m = nb * nb
    if pick_block_k_real(nsteps, m, m) == 1 and pick_block_k_real(nsteps, m, nb) == 1:
        return None
    return nb


def projected_mean(D, y0, proj, nsteps):
    """Ensemble mean of proj . y_n (n = 0..nsteps) for y_{n+1} = (I + D) y_n:
    the K-step blocked projection loop for FP32 blocks of up to 8 states and
    a shared projection, else the step-by-step batched loop.  Both kernels
    OR QSX_ERR_NONFINITE into the returned status word when a sample's final
    state is not finite (a NaN or an infinity never returns to a finite
    value), so ``raise_for_status`` reports a blow-up without a host sync
    inside the loop (``check_finite=False`` only skips raising here)."""
    m = D.shape[-1]
    P = proj.shape[-2]
    K = _native.proj_block_k(nsteps, m, P) if (D.dtype == torch.complex64 and m <= 8
                                               and proj.dim() == 2 and P <= 4) else 1
    if K > 1:
        mean, status = _native.rk4_proj_block_mean(D, y0, proj, nsteps, K, check_finite=False)
        return {'mean': mean, 'status': status}
    return _native.rk4(D, y0, nsteps, 1, proj=proj, per_sample=False, mean=True,
                       check_finite=False)


def redfield_batch_build(model, batch, precision=_native.QSX_FP64, build_precision=None):
    """The batch's Redfield build: eigendecomposition and operators in FP64
    (``build_precision`` QSX_FP32 asks for the FP32 build instead, valid for
    FP32 propagation only)."""
    if not isinstance(model, RedfieldModel):
        raise NotImplementedError('batched ensembles need a RedfieldModel')
    return model.build_batch(batch.H(model.hilbert_subspace), precision, build_precision)


def sample_polarizations(polarization, rotations):
    """(S, k, 3) per-sample polarization vectors R_s^T e for lab polarizations
    ``polarization`` (k of them) and dipole rotations (S, 3, 3)."""
    from ..polarization import polarization_vector
    pols = np.array([polarization_vector(p) for p in polarization], float)
    return np.einsum('sji,kj->ski', np.asarray(rotations, float), pols)


def ensemble_linear_signal(model, time_max, ensemble_size, polarization='xx',
                           precision='fp32', path='gg->eg->gg', start=0,
                           offsets=None, return_build=False, rotations=None,
                           initial_state=None):
    """Disorder-averaged Heisenberg-picture linear response (response.py:15-43).

    ``initial_state`` (a state vector on the path's first subspace, shared by
    every sample) replaces the thermal state, as in linear_response.

    ``rotations`` (S, 3, 3) rotates each sample's dipoles (random ensemble
    orientations, decorators.py:40-64): the dipole operators are linear in
    the polarization vector, so sample s uses R_s^T e in place of e, as a
    per-sample initial state and projection of the same batched time loop.

    Returns (t, mean signal) with the signal on the GPU (complex128).
    """
    from .utils import PRECISIONS, step_plan
    prec = PRECISIONS[precision]
    subs = path.split('->')
    dt = model.time_step
    t = np.arange(0, time_max, dt)
    batch = SampleBatch(model, ensemble_size, start, offsets)
    build = redfield_batch_build(model, batch, prec)
    rho0 = (model.thermal_state(subs[0]) if initial_state is None
            else np.asarray(initial_state))
    q = None if rotations is None else torch.as_tensor(
        sample_polarizations(polarization, rotations)).cuda()      # (S, 2, 3)
    total = None
    for sim in subs[1].split(','):
        sp0, sp1 = '{}->{}'.format(subs[0], sim), '{}->{}'.format(sim, subs[2])
        D = build.propagator(model.liouville_subspace_index(sim), dt, prec, transpose=True)
        if q is None:
            V0 = model.dipole_operator(sp0, polarization[0], '+')
            V1 = model.dipole_operator(sp1, polarization[1], '-')
            y0 = torch.as_tensor(-V1.bra_vector, dtype=torch.complex128).cuda()
            proj = torch.as_tensor(np.asarray(V0.commutator(rho0))[None, :],
                                   dtype=torch.complex128).cuda()
        else:
            axes = np.eye(3)
            P0 = np.array([model.dipole_operator(sp0, a, '+').commutator(rho0) for a in axes])
            Y1 = np.array([-model.dipole_operator(sp1, a, '-').bra_vector for a in axes])
            P0 = torch.as_tensor(P0, dtype=torch.complex128).cuda()
            Y1 = torch.as_tensor(Y1, dtype=torch.complex128).cuda()
            y0 = torch.einsum('sa,am->sm', q[:, 1].to(Y1.dtype), Y1).contiguous()
            proj = torch.einsum('sa,am->sm', q[:, 0].to(P0.dtype), P0)[:, None, :].contiguous()
        steps = step_plan(t, 0.0, dt)
        out = projected_mean(D, y0, proj, int(steps[-1]))
        sig = out['mean'][:, 0]
        total = sig if total is None else total + sig
        raise_for_status(int(out['status'].item()))
    if return_build:
        return t, total, build
    return t, total


def ensemble_populations(model, initial_state, duration, ensemble_size,
                         liouville_subspace='ee', precision='fp32', full_state=False,
                         start=0, offsets=None):
    """Disorder-averaged density matrices or populations (eom.py:11-26).

    Returns (t, mean) with mean (T, M) complex128 on the GPU over the
    selected components (all M when full_state, else the diagonal).
    """
    from .utils import PRECISIONS
    prec = PRECISIONS[precision]
    dt = model.time_step
    t = np.arange(0, duration, dt)
    batch = SampleBatch(model, ensemble_size, start, offsets)
    build = redfield_batch_build(model, batch, prec)
    rho0 = np.asarray(initial_state)
    if rho0.ndim == 1:
        rho0 = np.outer(rho0.conj(), rho0)
    y0 = model.density_matrix_to_state_vector(rho0, liouville_subspace)
    idx = model.liouville_subspace_index(liouville_subspace)
    M = len(idx)
    if full_state:
        select = list(range(M))
    else:
        nn = int(round(np.sqrt(M)))
        select = [i * nn + i for i in range(nn)]
    y0t = torch.as_tensor(y0, dtype=torch.complex128).cuda()
    n_total = model.hamiltonian.n_states(model.hilbert_subspace)
    nb = can_use_hermitian(prec, idx, n_total, y0, len(t) - 1)
    if nb is not None:
        out = propagate_hermitian_mean(build, idx, nb, dt, y0t, len(t) - 1, select)
        if 'mean_real' in out:
            out['mean'] = out['mean_real'].to(torch.complex128)
    else:
        out = propagate_selected_mean(build.propagator(idx, dt, prec), y0t, len(t) - 1,
                                      select, prec)
    raise_for_status(int(out['status'].item()))
    return t, out['mean']


def raise_for_status(status):
    """Raise for a status word of the ensemble kernels: IntegratorError for a
    non-finite state (integrate()'s error in the reference,
    simulate/utils.py:12-13), QsxError for a bad index table or a timed-out
    tensor-core wait."""
    if status & _native.QSX_ERR_NONFINITE:
        raise _native.IntegratorError('non-finite state in ensemble propagation')
    if status & _native.QSX_ERR_INVALID_ARG:
        raise _native.QsxError('ensemble propagation: index table out of range')
    if status & _native.QSX_ERR_CUDA:
        raise _native.QsxError('ensemble propagation: a tensor-core wait timed out')


class RedfieldEnsembleWorkload:
    """Disorder-averaged absorption spectrum plus population dynamics.

    The batched form of ``absorption_spectra(model, absorption_time,
    ensemble_size=S)`` together with ``simulate_dynamics(model,
    initial_state, dynamics_time, ensemble_size=S)`` (response.py:103-154,
    eom.py:29-74, decorators.py:40-64).  Everything that does not depend on
    the disorder draws (dipole vectors, subspace indices, frequency grid) is
    prepared once; ``run`` takes the (S, n_sites) site-energy offsets and
    does the whole pipeline on the GPU:

      H_s -> Jacobi eigensolve -> Redfield operators -> L_eg^T, L_ee
          -> RK4 propagators -> batched RK4 + ensemble means -> DFT.
    """

    def __init__(self, model, absorption_time, dynamics_time, initial_state,
                 polarization='xx', freqs=None):
        if not isinstance(model, RedfieldModel) or model.hilbert_subspace != 'ge':
            raise NotImplementedError("the workload runs a RedfieldModel on 'ge'")
        from .utils import fft_frequencies
        self.model = model
        ham = model.hamiltonian
        self.n_sites = ham.n_sites
        self.dt = model.time_step
        self.t_abs = np.arange(0, absorption_time, self.dt)
        self.t_dyn = np.arange(0, dynamics_time, self.dt)
        dev = torch.device('cuda', torch.cuda.current_device())
        self.H_base = torch.as_tensor(ham.H('ge'), dtype=torch.float64, device=dev)
        self.e_idx = torch.arange(1, 1 + self.n_sites, device=dev)
        self.idx_eg = model.liouville_subspace_index('eg')
        self.idx_ee = model.liouville_subspace_index('ee')
        rho0 = model.thermal_state('gg')
        V0 = model.dipole_operator('gg->eg', polarization[0], '+')
        V1 = model.dipole_operator('eg->gg', polarization[1], '-')
        self.proj = torch.as_tensor(np.asarray(V0.commutator(rho0))[None, :],
                                    dtype=torch.complex128, device=dev)
        # the spectrum transforms minus the signal (response.py:150-153):
        # project with -proj so the loop yields it directly
        self.proj_neg = (-self.proj).contiguous()
        self.y_abs = torch.as_tensor(-V1.bra_vector, dtype=torch.complex128, device=dev)
        rho = np.asarray(initial_state)
        if rho.ndim == 1:
            rho = np.outer(rho.conj(), rho)
        self.y_dyn_np = np.asarray(model.density_matrix_to_state_vector(rho, 'ee'), complex)
        self.y_dyn = torch.as_tensor(self.y_dyn_np, dtype=torch.complex128, device=dev)
        self.select = [i * self.n_sites + i for i in range(self.n_sites)]
        self.x_dyn = None   # Hermitian coordinates of y_dyn, made on first use
        self.freqs_np = (fft_frequencies(self.t_abs, model.rw_freq, model.unit_convert)
                         if freqs is None else np.asarray(freqs, float))
        self.freqs = torch.as_tensor(self.freqs_np, device=dev)
        from .utils import symmetric_grid
        t_sym, _ = symmetric_grid(self.t_abs)
        self.dft_t0 = self.t_abs[0] - t_sym[t_sym.size // 2]

    def run(self, offsets, precision='fp32', events=None, build_precision='fp64'):
        """(spectrum (F,) float64, populations (T, n_sites) float64, status) on
        the GPU.

        ``offsets`` is a (S, n_sites) float64 CUDA tensor.  ``precision`` is
        the propagation precision; the eigendecomposition and Redfield build
        run in ``build_precision`` ('fp64', or 'fp32' for an FP32 build
        feeding FP32 propagation).  ``events`` (a dict) collects CUDA events
        around the build and the population propagation.
        """
        from .utils import PRECISIONS
        prec = PRECISIONS[precision]
        H = _native.disordered_hamiltonians(self.H_base, offsets.contiguous(), 1)
        if events is not None:
            a0 = torch.cuda.Event(enable_timing=True)
            a0.record()
        build = self.model.build_batch(H, prec, PRECISIONS[build_precision])
        if events is not None:
            a1 = torch.cuda.Event(enable_timing=True)
            a1.record()
            events.setdefault('build', []).append((a0, a1))
        # the absorption leg (eg propagator, time loop, DFT) runs on a side
        # stream, overlapping the population leg on the caller's stream
        # (self.overlap = False runs it first on the caller's stream)
        main = torch.cuda.current_stream()
        if getattr(self, '_side', None) is None:
            self._side = torch.cuda.Stream()
        side = self._side if getattr(self, 'overlap', True) else main
        ready = torch.cuda.Event()
        ready.record(main)
        with torch.cuda.stream(side):
            side.wait_event(ready)
            if events is not None:
                l0 = torch.cuda.Event(enable_timing=True)
                l0.record()
            D_eg = build.propagator(self.idx_eg, self.dt, prec, transpose=True)
            sig = projected_mean(D_eg, self.y_abs, self.proj_neg, len(self.t_abs) - 1)
            X = _native.dft(sig['mean'][:, 0], self.dft_t0, self.dt, self.freqs,
                            self.model.rw_freq, self.model.unit_convert, 1, prec)
            if events is not None:
                l1 = torch.cuda.Event(enable_timing=True)
                l1.record()
                events.setdefault('abs_leg', []).append((l0, l1))
        if events is not None:
            p0 = torch.cuda.Event(enable_timing=True)
            p0.record()
        nb = can_use_hermitian(prec, self.idx_ee, self.n_sites + 1, self.y_dyn_np,
                               len(self.t_dyn) - 1)
        if nb is not None:
            if self.x_dyn is None:
                self.x_dyn = hermitian_coordinates(self.y_dyn, nb).contiguous()
            pop = propagate_hermitian_mean(build, self.idx_ee, nb, self.dt, self.y_dyn,
                                           len(self.t_dyn) - 1, self.select, events,
                                           x0=self.x_dyn)
        else:
            D_ee = build.propagator(self.idx_ee, self.dt, prec)
            pop = propagate_selected_mean(D_ee, self.y_dyn, len(self.t_dyn) - 1, self.select,
                                          prec, events)
        if events is not None:
            p1 = torch.cuda.Event(enable_timing=True)
            p1.record()
            events.setdefault('pop_leg', []).append((p0, p1))
        if side is not main:
            main.wait_stream(side)
            for t in (X, sig['status']):
                t.record_stream(main)
            for t in (build.G, build.M, build.E, build.U, build.occ, H):
                t.record_stream(side)
        status = sig['status'] | pop['status']
        pops = pop['mean_real'] if 'mean_real' in pop else pop['mean'].real
        return X.real, pops, status

    def capture(self, offsets, precision='fp32', build_precision='fp64'):
        """Record one step as a CUDA graph on static buffers (a copy of
        ``offsets`` in, the outputs of ``run``), so that a step is one graph
        launch instead of some forty kernel launches and their host-side
        bookkeeping.  Returns False, leaving the eager path, if the step
        cannot be captured."""
        self._graph = None
        try:
            static_in = offsets.clone()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                for _ in range(2):   # caches filled, workspaces allocated
                    self.run(static_in, precision, build_precision=build_precision)
            torch.cuda.current_stream().wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                out = self.run(static_in, precision, build_precision=build_precision)
                # the host call's result, packed on the device by the graph:
                # spectrum, populations, status word
                packed = torch.cat([out[0], out[1].reshape(-1), out[2].to(torch.float64)])
            torch.cuda.synchronize()
        except RuntimeError:
            torch.cuda.synchronize()
            return False
        host = torch.empty(packed.shape, dtype=packed.dtype, pin_memory=True)
        self._graph = (g, static_in, out, (precision, build_precision), packed, host)
        return True

    def replay(self, offsets=None):
        """One captured step; ``offsets`` (device or pinned host, the
        captured shape) replaces the input first.  Returns ``run``'s outputs,
        which the next replay overwrites."""
        g, static_in, out = self._graph[:3]
        if offsets is not None:
            static_in.copy_(offsets, non_blocking=True)
        g.replay()
        return out

    def run_host(self, offsets_host, precision='fp32', build_precision='fp64'):
        """End-to-end call with host buffers: pinned offsets in, numpy out
        (through the captured graph when one matches)."""
        dev = self.H_base.device
        graph = getattr(self, '_graph', None)
        if (graph is not None and graph[3] == (precision, build_precision)
                and tuple(graph[1].shape) == tuple(offsets_host.shape)):
            # the replay packs the result; one copy into pinned memory
            X, pops, status = self.replay(offsets_host)
            packed, out = graph[4], graph[5]
            out.copy_(packed, non_blocking=True)
            torch.cuda.current_stream().synchronize()
        else:
            off = offsets_host.to(dev, non_blocking=True)
            X, pops, status = self.run(off, precision, build_precision=build_precision)
            out = torch.cat([X, pops.reshape(-1), status.to(torch.float64)]).to('cpu')
        n = X.numel()
        raise_for_status(int(out[-1].item()))
        # copies: the pinned buffer is rewritten by the next call
        return out[:n].numpy().copy(), out[n:-1].numpy().reshape(pops.shape).copy()
