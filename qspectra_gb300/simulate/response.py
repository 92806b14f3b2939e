"""Response-function spectra (qspectra/simulate/response.py).

Same signatures as the reference plus ``precision`` ('fp64' default, 'fp32'
for the batched split-word form).  ``ensemble_size`` runs the disorder
average as one batched GPU pipeline instead of a serial loop.
"""
import numpy as np
import torch

from ..polarization import (FOURTH_ORDER_INVARIANTS, check_polarizations,
                             invariant_polarizations, invariant_weights_4th_order)
from .. import _native
from .ensemble import ensemble_linear_signal
from .utils import fft_frequencies, fourier_transform, integrate, symmetric_grid

PUMP_PROBE_PATHWAYS = {'GSB': 'gg->eg->gg',
                       'ESE': 'ee->eg->gg',
                       'ESA': 'ee->fe->ee'}

# Liouville pathways of Abramavicius et al., Chem. Rev. 109, 2350 (2009),
# Figs. 4-6 (the same table as response.py:252-264).
THIRD_ORDER_PATHWAYS = {
    '-++': {'ESE': 'gg->ge->ee->eg->gg',
            'GSB': 'gg->ge->gg->eg->gg',
            'ESA': 'gg->ge->ee->fe->ee'},
    '+-+': {'ESE': 'gg->eg->ee->eg->gg',
            'GSB': 'gg->eg->gg->eg->gg',
            'ESA': 'gg->eg->ee->fe->ee'},
    '++-': {'ESA1': 'gg->eg->fg->fe->ee',
            'ESA2': 'gg->eg->fg->eg->gg'},
}


def _parse_pathways(possible, include_signal):
    sel = [v for k, v in possible.items() if include_signal is None or k in include_signal]
    if not sel:
        raise ValueError('at least one Liouville space pathway must be selected, '
                         'i.e., include_signal must include at least one of %r'
                         % list(possible.keys()))
    return sel


def _single_linear_response(model, liouv_space_path, time_max, initial_state,
                            polarization, precision, **kw):
    """response.py:15-43 for one model (Heisenberg picture when available)."""
    subs = liouv_space_path.split('->')
    if initial_state is None:
        initial_state = model.thermal_state(subs[0])
    t = np.arange(0, time_max, model.time_step)
    signal = 0
    for sim in subs[1].split(','):
        V = [model.dipole_operator('{}->{}'.format(a, b), p, tr)
             for a, b, p, tr in zip(subs[:-1], subs[1:], polarization, '+-')]
        v_rho0 = V[0].commutator(np.asarray(initial_state))
        try:
            eom = model.equation_of_motion(sim, heisenberg_picture=True)
        except NotImplementedError:
            eom = model.equation_of_motion(sim)
            signal = signal - integrate(eom, v_rho0, t, save_func=V[1].expectation_value,
                                        precision=precision, **kw)
        else:
            v_gt = integrate(eom, -V[1].bra_vector, t, precision=precision, **kw)
            signal = signal + np.tensordot(v_rho0, v_gt, (-1, -1))
    return t, signal


def _zofe_linear(model, time_max, ensemble_size, polarization, precision, rotations):
    """Linear response of a ZOFE model (response.py:15-43; no Heisenberg
    picture, zofe.py:211-213): -tr(V1 rho(t)) from rho(0) = [V0, rho_thermal],
    every disorder sample in one launch, tr(V1 rho) reduced on the GPU."""
    from ..dynamics.zofe import ZOFESpaceOperator, ensemble_inputs
    from .ensemble import sample_polarizations
    from .utils import PRECISIONS, uniform_save_plan
    step = model.time_step
    t = np.arange(0, time_max, step)
    nsteps, every, first = uniform_save_plan(t, 0.0, step)
    dev = torch.device('cuda', torch.cuda.current_device())
    if ensemble_size is None:
        H = model.equation_of_motion().H
        y_th = torch.as_tensor(model.thermal_state(), device=dev)[None]
    else:
        H, y_th = ensemble_inputs(model, ensemble_size)
    ham, sub = model.hamiltonian, model.hilbert_subspace
    if rotations is None:
        A0 = ZOFESpaceOperator(ham.dipole_operator(sub, polarization[0], '+'), None, model)
        y0 = A0.commutator(y_th)
        proj = torch.as_tensor(ham.dipole_operator(sub, polarization[1], '-').reshape(1, -1),
                               dtype=torch.complex128, device=dev)
    else:
        q = torch.as_tensor(sample_polarizations(polarization, rotations), device=dev)
        y0 = sum(q[:, 0, a, None] * ZOFESpaceOperator(
            ham.dipole_operator(sub, np.eye(3)[a], '+'), None, model).commutator(y_th)
            for a in range(3))
        proj = torch.as_tensor(np.array([ham.dipole_operator(sub, np.eye(3)[a], '-').reshape(-1)
                                         for a in range(3)]),
                               dtype=torch.complex128, device=dev)
    Ld, G, w = model.zofe_tables()
    out = _native.zofe_rk4(H, Ld, G, w, y0.contiguous(), nsteps, step, model.unit_convert,
                           every, PRECISIONS[precision], proj=proj, state=False,
                           hermit=model.zofe_hermit)['proj']
    out = out[:, first:]
    if rotations is not None:
        out = (out * q[:, None, 1, :].to(out.dtype)).sum(-1, keepdim=True)
    return t, -out[..., 0].mean(0).cpu().numpy()


def _isotropic(fn, polarization, order=2):
    pols = check_polarizations(polarization, order)
    weight = np.dot(*pols)
    total = 0
    t = None
    for p in ['xx', 'yy', 'zz']:
        t, s = fn(p)
        total = total + s
    return t, total * weight / 3.0


def linear_response(dynamical_model, liouv_space_path, time_max,
                    initial_state=None, polarization='xx', ensemble_size=None,
                    ensemble_random_orientations=False,
                    exact_isotropic_average=False, precision='fp64',
                    **integrate_kwargs):
    """Linear response function under the RWA (response.py:46-100).

    With ``ensemble_size`` a Redfield model runs every disorder sample in one
    batched pipeline; other models integrate the samples one after another.
    ``ensemble_random_orientations`` rotates each sample's dipoles with the
    reference's draws (hamiltonian.py:552-575).
    """
    from ..dynamics.redfield import RedfieldModel
    from ..dynamics.zofe import ZOFEModel
    rotations = None
    if ensemble_size is not None and ensemble_random_orientations:
        rotations = dynamical_model.hamiltonian.orientation_rotations(ensemble_size)
    batched = (ensemble_size is not None and isinstance(dynamical_model, RedfieldModel)
               and (initial_state is None or np.ndim(initial_state) == 1)
               and not integrate_kwargs)
    zofe = (isinstance(dynamical_model, ZOFEModel) and initial_state is None
            and not integrate_kwargs and ',' not in liouv_space_path.split('->')[1])

    def one(pol):
        if zofe:
            return _zofe_linear(dynamical_model, time_max, ensemble_size, pol, precision,
                                rotations)
        if batched:
            t, sig = ensemble_linear_signal(dynamical_model, time_max, ensemble_size,
                                            pol, precision, path=liouv_space_path,
                                            rotations=rotations,
                                            initial_state=initial_state)
            return t, sig.cpu().numpy()
        if ensemble_size is not None:
            total = 0
            for m in dynamical_model.sample_ensemble(ensemble_size,
                                                     ensemble_random_orientations):
                t, sig = _single_linear_response(m, liouv_space_path, time_max,
                                                 initial_state, pol, precision,
                                                 **integrate_kwargs)
                total = total + sig
            return t, total / ensemble_size
        return _single_linear_response(dynamical_model, liouv_space_path, time_max,
                                       initial_state, pol, precision,
                                       **integrate_kwargs)

    if exact_isotropic_average:
        return _isotropic(one, polarization)
    return one(polarization)


def absorption_spectra(dynamical_model, time_max, correlation_decay_time=None,
                       polarization='xx', ensemble_size=None,
                       ensemble_random_orientations=False,
                       exact_isotropic_average=False, precision='fp64',
                       freqs=None, **integrate_kwargs):
    """Absorption spectrum (response.py:103-154); ``freqs`` picks a custom grid."""
    t, x = linear_response(dynamical_model, 'gg->eg->gg', time_max,
                           polarization=polarization, ensemble_size=ensemble_size,
                           ensemble_random_orientations=ensemble_random_orientations,
                           exact_isotropic_average=exact_isotropic_average,
                           precision=precision, **integrate_kwargs)
    if correlation_decay_time is not None:
        x = x * np.exp(-t / correlation_decay_time)
    f, X = fourier_transform(t, -x, rw_freq=dynamical_model.rw_freq,
                             unit_convert=dynamical_model.unit_convert, freqs=freqs)
    return f, X.real


def impulsive_probe(dynamical_model, state, time_max, polarization='xx',
                    initial_liouv_subspace='gg,ge,eg,ee',
                    include_signal='GSB,ESE,ESA', ensemble_size=None,
                    ensemble_random_orientations=False,
                    exact_isotropic_average=False, precision='fp64',
                    **integrate_kwargs):
    """Impulsive probe of a 2nd-order state (response.py:174-244).

    The state minus the thermal state is split over the pump-probe pathways
    (GSB, ESE, ESA) and each portion goes through ``linear_response`` with
    the same ensemble and orientation options; the summed signal is Fourier
    transformed.  With ``ensemble_size`` on a Redfield model every disorder
    sample of a pathway runs in one batched pipeline.
    """
    init = np.asarray(state) - dynamical_model.thermal_state(initial_liouv_subspace)
    total = 0
    t = None
    for path in _parse_pathways(PUMP_PROBE_PATHWAYS, include_signal):
        first = path.split('->')[0]
        portion = np.apply_along_axis(
            lambda s: dynamical_model.map_between_subspaces(s, initial_liouv_subspace, first),
            -1, init)
        t, sig = linear_response(dynamical_model, path, time_max, portion, polarization,
                                 ensemble_size=ensemble_size,
                                 ensemble_random_orientations=ensemble_random_orientations,
                                 exact_isotropic_average=exact_isotropic_average,
                                 precision=precision, **integrate_kwargs)
        total = total + sig
    return fourier_transform(t, total, rw_freq=dynamical_model.rw_freq,
                             unit_convert=dynamical_model.unit_convert)


def _single_third_order(model, coherence_time_max, population_time_max,
                        population_times, geometry, polarization, include_signal,
                        precision, **kw):
    """Sum over Liouville pathways, Heisenberg picture for t3 (response.py:267-337)."""
    dt = model.time_step
    t1 = np.arange(0, coherence_time_max, dt)
    t2 = (np.arange(0, population_time_max, dt) if population_times is None
          else np.asarray(population_times, float))
    t3 = np.arange(0, coherence_time_max, dt)
    rho0 = model.thermal_state('gg')
    total = 0
    for path in _parse_pathways(THIRD_ORDER_PATHWAYS[geometry], include_signal):
        subs = path.split('->')
        V = [model.dipole_operator('{}->{}'.format(a, b), p, tr)
             for a, b, p, tr in zip(subs[:-1], subs[1:], polarization, geometry + '-')]
        eom = [model.equation_of_motion(s) for s in subs[1:-1]]
        v_rho0 = V[0].commutator(rho0)
        v_rho1 = integrate(eom[0], v_rho0, t1, save_func=V[1].commutator,
                           precision=precision, step=dt, **kw)
        v_rho2 = integrate(eom[1], v_rho1, t2, t0=0, save_func=V[2].commutator,
                           precision=precision, step=dt, **kw)
        try:
            eom_h = model.equation_of_motion(subs[3], heisenberg_picture=True)
        except NotImplementedError:
            total = total + integrate(eom[2], v_rho2, t3, save_func=V[3].expectation_value,
                                      precision=precision, step=dt, **kw)
        else:
            v_gt3 = integrate(eom_h, V[3].bra_vector, t3, precision=precision, step=dt, **kw)
            total = total + np.einsum('ci,abi', v_gt3, v_rho2)
    return (t1, t2, t3), total


def third_order_response(dynamical_model, coherence_time_max,
                         population_time_max=None, population_times=None,
                         geometry='-++', polarization='xxxx', include_signal=None,
                         ensemble_size=None, ensemble_random_orientations=False,
                         exact_isotropic_average=False, precision='fp64',
                         **integrate_kwargs):
    """Third-order response function under the RWA (response.py:340-427).

    Non-secular site-basis Redfield models on 'gef' with geometry '-++' or
    '+-+' run on the batched engine (simulate/third_order.py): every sample
    of an ensemble in one pass, the two-exciton block in operator form.
    Other models and geometries integrate each pathway's dense blocks.

    ``exact_isotropic_average`` sums the lab polarizations of the three
    fourth-rank invariants with the reference's weights (decorators.py:67-92;
    invariants whose weight is not above 1e-8 are left out, as there);
    ``ensemble_random_orientations`` rotates each sample's dipoles.  The
    engine evaluates both from shared legs in one pass.
    """
    from .third_order import supports, third_order_ensemble
    if supports(dynamical_model, geometry) and not integrate_kwargs:
        if population_times is None:
            population_times = np.arange(0, population_time_max, dynamical_model.time_step)
        return third_order_ensemble(dynamical_model, coherence_time_max, population_times,
                                    geometry, polarization, include_signal, ensemble_size,
                                    precision, isotropic=exact_isotropic_average,
                                    random_orientations=ensemble_random_orientations)

    def one(model):
        if not exact_isotropic_average:
            return _single_third_order(model, coherence_time_max, population_time_max,
                                       population_times, geometry, polarization,
                                       include_signal, precision, **integrate_kwargs)
        weights = invariant_weights_4th_order(polarization)
        signals = {}
        total, ticks = 0, None
        for inv, w in zip(FOURTH_ORDER_INVARIANTS, weights):
            if w > 1e-8:
                for p in invariant_polarizations(inv):
                    if p not in signals:
                        ticks, signals[p] = _single_third_order(
                            model, coherence_time_max, population_time_max,
                            population_times, geometry, p, include_signal, precision,
                            **integrate_kwargs)
                    total = total + w * signals[p]
        return ticks, total

    if ensemble_size is None:
        return one(dynamical_model)
    total = 0
    ticks = None
    for m in dynamical_model.sample_ensemble(ensemble_size, ensemble_random_orientations):
        ticks, s = one(m)
        total = total + s
    return ticks, total / ensemble_size


def two_dimensional_spectra(dynamical_model, coherence_time_max,
                            population_time_max=None, population_times=None,
                            geometry='-++', polarization='xxxx', include_signal=None,
                            ensemble_size=None, ensemble_random_orientations=False,
                            exact_isotropic_average=False, precision='fp64',
                            **integrate_kwargs):
    """2D spectrum: FT over t1 (sign -1) and t3 (response.py:430-455), both
    axes of the third-order signal in one GPU launch (qsx_dft2_batched) on
    the reference's FFT frequency grids."""
    (t1, t2, t3), X = third_order_response(
        dynamical_model, coherence_time_max, population_time_max, population_times,
        geometry, polarization, include_signal, ensemble_size,
        ensemble_random_orientations, exact_isotropic_average, precision,
        **integrate_kwargs)
    rw, uc = dynamical_model.rw_freq, dynamical_model.unit_convert
    t1, t3 = np.asarray(t1, float), np.asarray(t3, float)
    f1 = fft_frequencies(t1, rw, uc, sign=-1)
    f3 = fft_frequencies(t3, rw, uc, sign=1)
    # the sample that ifftshift moves to index 0 is the time origin
    s1, _ = symmetric_grid(t1)
    s3, _ = symmetric_grid(t3)
    as_numpy = not isinstance(X, torch.Tensor)
    xt = torch.as_tensor(np.asarray(X, dtype=complex) if as_numpy else X,
                         dtype=torch.complex128).cuda().contiguous()
    X3 = _native.dft2(xt, t1[0] - s1[s1.size // 2], t1[1] - t1[0], f1, -1,
                      t3[0] - s3[s3.size // 2], t3[1] - t3[0], f3, 1, rw, uc)
    return (f1, t2, f3), (X3.cpu().numpy() if as_numpy else X3)
