"""Time loop and Fourier transform (qspectra/simulate/utils.py).

``integrate`` runs the whole fixed-step RK4 loop on the GPU for an
``EquationOfMotion`` (the reference drives SciPy's adaptive zvode through a
Python callback; the GB300 path replaces that with classical RK4 at a fixed
step, by default the spacing of the requested times).  ``fourier_transform``
evaluates the reference's FFT-based transform by direct DFT on the GPU.
"""
import numpy as np
import torch

from .. import _native
from ..dynamics.liouville_space import EquationOfMotion, LinearMap

PRECISIONS = {'fp64': _native.QSX_FP64, 'fp32': _native.QSX_FP32}
PROPAGATOR_MAX = 64


class IntegratorError(_native.IntegratorError):
    """Integration failed (simulate/utils.py:12-13)."""


def _precision(p):
    try:
        return PRECISIONS[p]
    except KeyError:
        raise ValueError("precision must be 'fp64' or 'fp32'")


def step_plan(t, t0, h):
    """Whole numbers of RK4 steps from t0 to each output time."""
    t = np.asarray(t, float)
    rel = (t - t0) / h
    steps = np.rint(rel).astype(np.int64)
    if np.any(np.abs(rel - steps) > 1e-6) or np.any(steps < 0):
        raise ValueError('output times must lie on the RK4 step grid t0 + k*h')
    if np.any(np.diff(steps) < 0):
        raise ValueError('output times must be non-decreasing')
    return steps


def propagate(matrix, y0, steps, h, precision=_native.QSX_FP64, proj=None,
              select=None, mean=False, per_sample=True, check_finite=True):
    """RK4 outputs at the given cumulative step counts (GPU).

    matrix: (B, M, M) or (M, M) complex128 generator L on the GPU.
    y0: (B, M) or (M,) complex128.  Returns state (B, T, M) or projections.
    """
    steps = np.asarray(steps, np.int64)
    M = matrix.shape[-1]
    mat = matrix if matrix.dim() == 3 else matrix[None]
    if M <= PROPAGATOR_MAX:
        D = _native.rk4_propagator(mat.contiguous(), h, precision)
        form = 0
        Dm = D if matrix.dim() == 3 else D[0]
    else:
        form = 1
        Dm = matrix.to(torch.complex64 if precision == _native.QSX_FP32
                       else torch.complex128).contiguous()
    uniform = len(steps) > 1 and np.all(np.diff(steps) == steps[1] - steps[0]) \
        and steps[1] > steps[0]
    kw = dict(form=form, h=h, precision=precision, proj=proj, select=select,
              mean=mean, per_sample=per_sample, check_finite=check_finite)
    want_state = proj is None and select is None
    if uniform or len(steps) == 1:
        every = int(steps[1] - steps[0]) if len(steps) > 1 else 1
        first = int(steps[0])
        y = y0
        if first > 0:
            y = _native.rk4(Dm, y, first, first, state=True, **dict(kw, proj=None, select=None,
                                                                    mean=False))['state'][:, -1]
            if y0.dim() == 1 and matrix.dim() == 2:
                y = y[0]
        n = every * (len(steps) - 1)
        return _native.rk4(Dm, y, n, every if n else 1, state=want_state, **kw)
    # irregular outputs: one call per segment
    outs = []
    y = y0
    prev = 0
    for k, s in enumerate(steps):
        seg = int(s - prev)
        r = _native.rk4(Dm, y, seg, seg if seg else 1, state=True,
                        **dict(kw, proj=None, select=None, mean=False))
        st = r['state'][:, -1]
        y = st if not (y0.dim() == 1 and matrix.dim() == 2) else st[0]
        outs.append(st)
        prev = s
    state = torch.stack(outs, dim=1)
    if want_state:
        return {'state': state}
    raise ValueError('irregular output times support full-state output only')


def integrate(f, y0, t, t0=None, method_name='rk4', f_params=None,
              save_func=None, precision='fp64', step=None, **kwargs):
    """RK4 solution of dy/dt = f(t, y) at the times t (simulate/utils.py:53-109).

    ``f`` must be an equation of motion from a qspectra_gb300 model.
    ``step`` is the RK4 step (default t[1] - t[0]).  ``save_func`` may be
    None or a linear map from an operator (e.g. ``V.commutator``,
    ``V.expectation_value``).  A 2-D ``y0`` integrates every row.
    """
    from ..dynamics.heom import HEOMEquationOfMotion, HEOMMultiBlockEquationOfMotion
    if isinstance(f, HEOMMultiBlockEquationOfMotion):
        return _integrate_heom_blocks(f, y0, t, t0, save_func, precision, step,
                                      kwargs.pop('heom_nodes', None))
    from ..dynamics.zofe import ZOFEEquationOfMotion
    if isinstance(f, HEOMEquationOfMotion):
        return _integrate_heom(f, y0, t, t0, save_func, precision, step,
                               kwargs.pop('heom_nodes', None))
    if isinstance(f, ZOFEEquationOfMotion):
        return _integrate_zofe(f, y0, t, t0, save_func, precision, step)
    if not isinstance(f, EquationOfMotion):
        raise TypeError('integrate needs an equation of motion returned by a '
                        'qspectra_gb300 model (got {!r})'.format(type(f)))
    if method_name not in ('rk4', 'zvode'):
        raise ValueError('unsupported method {!r}; the GPU path integrates with '
                         'fixed-step RK4'.format(method_name))
    if f_params:
        raise ValueError('f_params are not used by linear equations of motion')
    t = np.asarray(t, float)
    if t0 is None:
        t0 = t[0]
    if step is None:
        step = (t[1] - t[0]) if len(t) > 1 else 1.0
    steps = step_plan(t, t0, step)
    as_numpy = not isinstance(y0, torch.Tensor)
    y = torch.as_tensor(np.asarray(y0, dtype=complex) if as_numpy else y0,
                        dtype=torch.complex128, device=f.matrix.device)
    squeeze = y.dim() == 1
    Y = y[None] if squeeze else y.reshape(-1, y.shape[-1])
    B = Y.shape[0]
    L = f.matrix if B == 1 else f.matrix
    res = propagate(L, Y if B > 1 else Y[0], steps, step, _precision(precision))
    state = res['state']  # (1 or B, T, M)
    if save_func is not None:
        if isinstance(save_func, LinearMap):
            state = state @ save_func.matrix.T
            if save_func.scalar:
                state = state[..., 0]
        else:
            raise TypeError('save_func must be a linear operator map')
    if squeeze:
        state = state[0]
    else:
        state = state.reshape(tuple(y.shape[:-1]) + tuple(state.shape[1:]))
    return state.cpu().numpy() if as_numpy else state


def _integrate_heom(f, y0, t, t0, save_func, precision, step, heom_nodes):
    """integrate() for the HEOM generator: uniform outputs, full state by
    default (the reference returns every ADO), node 0 only with heom_nodes=1."""
    t = np.asarray(t, float)
    if t0 is None:
        t0 = t[0]
    if step is None:
        step = (t[1] - t[0]) if len(t) > 1 else 1.0
    steps = step_plan(t, t0, step)
    if steps[0] != 0 or (len(steps) > 1 and np.any(np.diff(steps) != steps[1] - steps[0])):
        raise ValueError('HEOM integration needs uniform output times starting at t0')
    every = int(steps[1] - steps[0]) if len(steps) > 1 else 1
    nsteps = every * (len(steps) - 1)
    tb = f.tables
    nodes = tb.nnodes if heom_nodes is None else int(heom_nodes)
    as_numpy = not isinstance(y0, torch.Tensor)
    y = torch.as_tensor(np.asarray(y0, dtype=complex) if as_numpy else y0,
                        dtype=torch.complex128, device='cuda')
    squeeze = y.dim() == 1
    Y = y[None] if squeeze else y.reshape(-1, y.shape[-1])
    B = Y.shape[0] if f.Hx.dim() == 2 else f.Hx.shape[0]
    res = _native.heom_rk4(tb, f.Hx, f.Hy, Y if Y.shape[0] > 1 else Y[0], nsteps, step,
                           f.model.unit_convert, batch=B, save_every=max(every, 1),
                           save_nodes=nodes, precision=_precision(precision))
    state = res['state']
    if save_func is not None:
        if not isinstance(save_func, LinearMap):
            state_np = state.cpu().numpy()
            out = np.asarray(save_func(state_np))
            return out[0] if squeeze else out
        state = state @ save_func.matrix.T
        if save_func.scalar:
            state = state[..., 0]
    if squeeze:
        state = state[0]
    return state.cpu().numpy() if as_numpy else state


def _integrate_heom_blocks(f, y0, t, t0, save_func, precision, step, heom_nodes):
    """integrate() for a HEOM generator on several Liouville blocks: the
    blocks evolve independently, so each runs its own loop on its share of
    the node vectors and the outputs are scattered back to the union."""
    as_numpy = not isinstance(y0, torch.Tensor)
    y = torch.as_tensor(np.asarray(y0, dtype=complex) if as_numpy else y0,
                        dtype=torch.complex128, device='cuda')
    nodes = f.nnodes if heom_nodes is None else int(heom_nodes)
    out = None
    for eom, flat in f.parts:
        part = _integrate_heom(eom, f.gather(y, flat), t, t0, None, precision, step, nodes)
        if out is None:
            out = torch.zeros(part.shape[:-1] + (nodes * f.M,), dtype=part.dtype,
                              device=part.device)
        f.scatter(out, flat[:part.shape[-1]], part)
    if save_func is not None:
        if isinstance(save_func, LinearMap):
            out = out @ save_func.matrix.T
            if save_func.scalar:
                out = out[..., 0]
        else:
            res = np.asarray(save_func(out.cpu().numpy()))
            return res if as_numpy else torch.as_tensor(res, device='cuda')
    return out.cpu().numpy() if as_numpy else out


def uniform_save_plan(t, t0, step):
    """(nsteps, save_every, first) for outputs on a uniform grid of RK4 steps
    from t0: the kernel saves every save_every steps and the outputs start at
    save index first."""
    steps = step_plan(np.asarray(t, float), t0, step)
    every = int(steps[1] - steps[0]) if len(steps) > 1 else max(int(steps[0]), 1)
    every = max(every, 1)
    if steps[0] % every or (len(steps) > 1 and np.any(np.diff(steps) != every)):
        raise ValueError('output times must be evenly spaced on the RK4 step grid from t0')
    return int(steps[-1]), every, int(steps[0]) // every


def _integrate_zofe(f, y0, t, t0, save_func, precision, step):
    """integrate() for the ZOFE master equation (qsx_zofe_rk4): uniform
    outputs; an operator's expectation value is reduced on the GPU, other
    save functions are applied to the saved states."""
    from ..dynamics.zofe import ZOFESpaceOperator
    t = np.asarray(t, float)
    if t0 is None:
        t0 = t[0]
    if step is None:
        step = (t[1] - t[0]) if len(t) > 1 else 1.0
    nsteps, every, first = uniform_save_plan(t, t0, step)
    as_numpy = not isinstance(y0, torch.Tensor)
    y = torch.as_tensor(np.asarray(y0, dtype=complex) if as_numpy else y0,
                        dtype=torch.complex128, device='cuda')
    squeeze = y.dim() == 1
    Y = y[None] if squeeze else y.reshape(-1, y.shape[-1])
    Ld, G, w = f.model.zofe_tables()
    owner = getattr(save_func, '__self__', None)
    expect = (isinstance(owner, ZOFESpaceOperator)
              and getattr(save_func, '__func__', None) is ZOFESpaceOperator.expectation_value)
    proj = None
    if expect:
        proj = torch.as_tensor(owner.expectation_row[None], dtype=torch.complex128,
                               device=Y.device)
    res = _native.zofe_rk4(f.H, Ld, G, w, Y if Y.shape[0] > 1 else Y[0], nsteps, step,
                           f.model.unit_convert, save_every=every,
                           precision=_precision(precision), proj=proj, state=not expect,
                           hermit=f.model.zofe_hermit)
    if expect:
        out = res['proj'][:, first:, 0]
    else:
        out = res['state'][:, first:]
        if save_func is not None:
            if isinstance(save_func, LinearMap):
                out = out @ save_func.matrix.T
                if save_func.scalar:
                    out = out[..., 0]
            else:
                out = save_func(out)
    if squeeze:
        out = out[0]
    else:
        out = out.reshape(tuple(y.shape[:-1]) + tuple(out.shape[1:]))
    return out.cpu().numpy() if as_numpy else out


def is_constant(x, atol=1e-7, positive=None):
    x = np.asarray(x)
    return (np.max(np.abs(x - x[0])) < atol and
            (np.all((x > 0) == positive) if positive is not None else True))


def slice_along_axis(start=None, stop=None, step=None, axis=0, ndim=1):
    return tuple(slice(start, stop, step) if (n == axis) or (n == ndim + axis)
                 else slice(None) for n in range(ndim))


def symmetric_grid(t):
    """Symmetric zero-padded time grid of _symmetrize (simulate/utils.py:128-151)."""
    t = np.asarray(t, float)
    if not is_constant(np.diff(t), positive=True):
        raise ValueError('sample times must differ by a positive constant')
    T = max(t[-1], -t[0])
    dt = t[1] - t[0]
    n_plus = int((T - t[-1]) / dt) + 1
    n_minus = int((T + t[0]) / dt) + 1
    t_sym = np.concatenate([t[0] - dt * np.arange(1, n_minus)[::-1], t,
                            t[-1] + dt * np.arange(1, n_plus)])
    start = int(np.searchsorted(t_sym, t[0]))
    return t_sym, start


def _symmetrize(t, x, axis=-1):
    """Host reference of the zero padding, kept for API parity."""
    t_sym, start = symmetric_grid(t)
    x = np.asarray(x)
    shape = list(x.shape)
    shape[axis] = t_sym.size
    out = np.zeros(shape, dtype=x.dtype)
    out[slice_along_axis(start, start + len(t), axis=axis, ndim=x.ndim)] = x
    return t_sym, out


def fft_frequencies(t, rw_freq=0, unit_convert=1, sign=1, convention='angular'):
    """Frequencies fourier_transform returns for samples at times t."""
    if convention == 'angular':
        unit_convert = unit_convert / (2 * np.pi)
    elif convention != 'linear':
        raise ValueError("convention must be 'angular' or 'linear'")
    t_sym, _ = symmetric_grid(t)
    n = t_sym.size
    dt = t_sym[1] - t_sym[0]
    f = np.fft.fftshift(np.fft.fftfreq(n, dt * unit_convert))
    if sign == 1:
        f = -f[::-1]
    return f + rw_freq


def fourier_transform(t, x, axis=-1, rw_freq=0, unit_convert=1, sign=1,
                      convention='angular', freqs=None):
    """X(ω) = ∫ exp(i sign (ω - ω0) t) x(t) dt on the GPU (simulate/utils.py:154-219).

    Returns the reference's FFT grid and values; ``freqs`` evaluates any
    other frequency grid directly instead.
    """
    t = np.asarray(t, float)
    if t.ndim != 1:
        raise ValueError('t must be one dimensional')
    xs = x if isinstance(x, torch.Tensor) else np.asarray(x)
    if t.size != xs.shape[axis]:
        raise ValueError('t must have the same length as the shape of x along '
                         'the given axis')
    if sign not in (-1, 1):
        raise ValueError('sign must be +1 or -1')
    if convention not in ('angular', 'linear'):
        raise ValueError("convention must be 'angular' or 'linear'")
    t_sym, _ = symmetric_grid(t)
    origin = t_sym[t_sym.size // 2]  # sample ifftshift moves to index 0
    uc = unit_convert if convention == 'angular' else 2 * np.pi * unit_convert
    if freqs is None:
        f = fft_frequencies(t, rw_freq, unit_convert, sign, convention)
    else:
        f = np.asarray(freqs, float)
    as_numpy = not isinstance(x, torch.Tensor)
    xt = torch.as_tensor(np.asarray(x, dtype=complex) if as_numpy else x,
                         dtype=torch.complex128).cuda()
    xt = torch.movedim(xt, axis, -1)
    lead = xt.shape[:-1]
    flat = xt.reshape(-1, xt.shape[-1]).contiguous()
    dt = t[1] - t[0]
    X = _native.dft(flat, t[0] - origin, dt, torch.as_tensor(f), rw_freq, uc, sign)
    X = torch.movedim(X.reshape(tuple(lead) + (len(f),)), -1, axis)
    return f, (X.cpu().numpy() if as_numpy else X)


def bound_signal(ticks, signal, bounds, axis=0):
    """simulate/utils.py:222-250."""
    if signal.shape[axis] != len(ticks):
        raise ValueError('ticks must have same shape as signal along given axis')
    i0, i1 = sorted(np.argmin(np.abs(ticks - b)) for b in bounds)
    sl = slice_along_axis(i0, i1 + 1, axis=axis, ndim=len(signal.shape))
    return ticks[i0:(i1 + 1)], signal[sl]
