"""Free time evolution (qspectra/simulate/eom.py:11-74)."""
import numpy as np
import torch

from .. import _native

from .ensemble import ensemble_populations
from .utils import integrate


def simulate_dynamics(dynamical_model, initial_state, duration=None, times=None,
                      liouville_subspace='ee', save_func=None, ensemble_size=None,
                      ensemble_random_orientations=False, precision='fp64',
                      **integrate_kwargs):
    """Density matrices ρ(t) with no applied field (eom.py:29-74).

    Returns (t, rhos) with rhos (T, N, N) like the reference.  With
    ``ensemble_size`` the disorder average of a Redfield model is one batched
    GPU run; other models integrate the samples one after another.  Random
    orientations rotate only the dipoles, which free dynamics never reads, so
    ``ensemble_random_orientations`` leaves the result unchanged (the
    reference draws the rotation after the disorder: hamiltonian.py:552-575).
    """
    from ..dynamics.redfield import RedfieldModel
    from ..dynamics.zofe import ZOFEModel
    if (isinstance(dynamical_model, ZOFEModel) and save_func is None
            and not integrate_kwargs.get('heom_nodes')):
        return _zofe_dynamics(dynamical_model, initial_state, duration, times,
                              ensemble_size, precision, integrate_kwargs.pop('step', None))
    if ensemble_size is not None:
        if (isinstance(dynamical_model, RedfieldModel) and times is None
                and save_func is None and not integrate_kwargs):
            t, mean = ensemble_populations(dynamical_model, initial_state, duration,
                                           ensemble_size, liouville_subspace, precision,
                                           full_state=True)
            rhos = dynamical_model.state_vector_to_density_matrix(mean.cpu().numpy())
            return t, rhos
        total = 0
        for m in dynamical_model.sample_ensemble(ensemble_size,
                                                 ensemble_random_orientations):
            t, rhos = simulate_dynamics(m, initial_state, duration, times,
                                        liouville_subspace, save_func,
                                        precision=precision, **integrate_kwargs)
            total = total + rhos
        return t, total / ensemble_size
    from ..dynamics.heom import HEOMModel
    eom = dynamical_model.equation_of_motion(liouville_subspace)
    rho0 = np.asarray(initial_state)
    if rho0.ndim == 1:
        rho0 = np.outer(rho0.conj(), rho0)
    y0 = dynamical_model.density_matrix_to_state_vector(rho0, liouville_subspace)
    step = integrate_kwargs.pop('step', dynamical_model.time_step)
    t = (np.arange(0, duration, step) if times is None else np.asarray(times, float))
    if isinstance(dynamical_model, HEOMModel) and save_func is None:
        # only the physical node is returned, so only node 0 is kept on the GPU
        states = integrate(eom, y0, t, precision=precision, step=step, heom_nodes=1,
                           **integrate_kwargs)
        return t, dynamical_model.lspace_model.state_vector_to_density_matrix(states)
    states = integrate(eom, y0, t, save_func=save_func, precision=precision, step=step,
                       **integrate_kwargs)
    return t, dynamical_model.state_vector_to_density_matrix(states)


def _zofe_dynamics(model, initial_state, duration, times, ensemble_size, precision, step):
    """ZOFE free dynamics: only rho is written back, averaged over the
    samples of the same launch."""
    from ..dynamics.zofe import ensemble_inputs
    from .utils import PRECISIONS, uniform_save_plan
    step = model.time_step if step is None else step
    t = np.arange(0, duration, step) if times is None else np.asarray(times, float)
    nsteps, every, first = uniform_save_plan(t, 0.0, step)
    rho0 = np.asarray(initial_state)
    if rho0.ndim == 1:
        rho0 = np.outer(rho0.conj(), rho0)
    dev = torch.device('cuda', torch.cuda.current_device())
    y0 = torch.as_tensor(model.density_matrix_to_state_vector(rho0), device=dev)
    if ensemble_size is None:
        H = model.equation_of_motion().H
    else:
        H, _ = ensemble_inputs(model, ensemble_size)
    n = model.n_states
    Ld, G, w = model.zofe_tables()
    out = _native.zofe_rk4(H, Ld, G, w, y0, nsteps, step, model.unit_convert, every,
                           PRECISIONS[precision], state='rho', hermit=model.zofe_hermit)['state']
    vec = out[:, first:].mean(0).cpu().numpy()          # (T, n*n), column-major rho
    return t, vec.reshape(len(vec), n, n).transpose(0, 2, 1)


def _field_table(pulses, geometry, rw_freq, t0, nsteps, h):
    """a_p at t_n, t_n + h/2, t_n + h: -i E_p(t), conjugated for '+'."""
    tn = t0 + h * np.arange(nsteps)
    ts = np.stack([tn, tn + h / 2, tn + h], axis=1)            # (nsteps, 3)
    cols = []
    for pulse, trans in zip(pulses, geometry):
        E = np.asarray(pulse(ts, rw_freq), dtype=complex)
        if trans == '+':
            E = np.conj(E)
        cols.append(-1j * E)
    return np.stack(cols, axis=-1)                              # (nsteps, 3, npulses)


def simulate_with_fields(dynamical_model, pulses, geometry='-+', polarization='xx',
                         time_extra=0, times=None, liouville_subspace='gg,ge,eg,ee',
                         save_func=None, ensemble_size=None,
                         ensemble_random_orientations=False, precision='fp64',
                         **integrate_kwargs):
    """Time evolution under pulses in the rotating-wave approximation
    (eom.py:77-170), fixed-step RK4 on the GPU (qsx_rk4_field_batched).

    Returns (t, states) with states (T, M) (or save_func of them), averaged
    over ``ensemble_size`` disorder samples when given.  With
    ``ensemble_random_orientations`` each sample's field maps carry its
    rotated dipoles (hamiltonian.py:552-575): the commutator maps are linear
    in the polarization vector, so sample s gets sum_a (R_s^T e)_a C(e_a).
    """
    from .ensemble import SampleBatch, sample_polarizations
    from .utils import PRECISIONS, step_plan
    from ..dynamics.zofe import ZOFEModel
    model = dynamical_model
    if (save_func is not None and not hasattr(save_func, 'matrix')
            and not isinstance(model, ZOFEModel)):
        raise TypeError('save_func must be a linear operator map')
    prec = PRECISIONS[precision]
    h = integrate_kwargs.pop('step', model.time_step)
    t0 = min(p.t_init for p in pulses)
    tf = max(p.t_final for p in pulses)
    t = (np.arange(t0, tf + time_extra, model.time_step) if times is None
         else tf + np.asarray(times, float))
    steps = step_plan(t, t0, h)
    every = int(steps[1] - steps[0]) if len(steps) > 1 else 1
    if steps[0] % max(every, 1) or np.any(np.diff(steps) != every):
        raise ValueError('output times must be evenly spaced on the RK4 step grid from '
                         'the first pulse')
    first = int(steps[0])
    nsteps = int(steps[-1])
    dev = torch.device('cuda', torch.cuda.current_device())
    coef = torch.as_tensor(_field_table(pulses, geometry, model.rw_freq, t0, nsteps, h),
                           device=dev)
    save_every = max(every, 1) if nsteps else 1
    if isinstance(model, ZOFEModel):
        states = _zofe_fields(model, polarization, geometry, coef, nsteps, h, save_every,
                              ensemble_size, ensemble_random_orientations, prec)
        states = states[:, first // save_every:]
        states = states.mean(0) if ensemble_size is not None else states[0]
        if save_func is not None:
            states = save_func(states)
        if isinstance(states, torch.Tensor):
            states = states.cpu().numpy()
        return t, states
    idx = model.liouville_subspace_index(liouville_subspace)
    if ensemble_size is not None and ensemble_random_orientations:
        rot = model.hamiltonian.orientation_rotations(ensemble_size)
        q = torch.as_tensor(sample_polarizations(polarization, rot), device=dev)
        basis = torch.as_tensor(np.array(
            [[model.dipole_operator(liouville_subspace, a, tr).commutator_matrix
              for a in np.eye(3)] for tr in geometry], dtype=complex), device=dev)
        C = torch.einsum('spa,pamn->spmn', q.to(basis.dtype), basis)
    else:
        V = [model.dipole_operator(liouville_subspace, pol, tr)
             for pol, tr in zip(polarization, geometry)]
        C = torch.as_tensor(np.array([v.commutator_matrix for v in V], dtype=complex),
                            device=dev)
    y0 = torch.as_tensor(np.asarray(model.thermal_state(liouville_subspace), dtype=complex),
                         device=dev)
    if ensemble_size is None:
        L = model.equation_of_motion(liouville_subspace).matrix
    else:
        batch = SampleBatch(model, ensemble_size)
        L = model.build_batch(batch.H(model.hilbert_subspace)).block(idx)
    states = _native.rk4_field(L, C, coef, y0, nsteps, h, save_every, prec)
    states = states[:, first // save_every:]
    if ensemble_size is not None:
        states = states.mean(0)
    else:
        states = states[0]
    if save_func is not None:
        states = states @ save_func.matrix.T
        if save_func.scalar:
            states = states[..., 0]
    return t, states.cpu().numpy()


def _zofe_fields(model, polarization, geometry, coef, nsteps, h, save_every,
                 ensemble_size, random_orientations, prec):
    """States (B, nsave, M) of a ZOFE model under pulses (qsx_zofe_rk4 with
    the dipole operators folded into its small operators)."""
    from ..dynamics.zofe import ensemble_inputs
    from .ensemble import sample_polarizations
    dev = coef.device
    if ensemble_size is None:
        H = model.equation_of_motion().H
        y0 = torch.as_tensor(model.thermal_state(), device=dev)
    else:
        H, y0 = ensemble_inputs(model, ensemble_size)
    sub = model.hilbert_subspace
    ham = model.hamiltonian
    if ensemble_size is not None and random_orientations:
        q = torch.as_tensor(sample_polarizations(
            polarization, ham.orientation_rotations(ensemble_size)), device=dev)
        basis = torch.as_tensor(np.array(
            [[ham.dipole_operator(sub, a, tr) for a in np.eye(3)] for tr in geometry],
            dtype=complex), device=dev)
        V = torch.einsum('spa,pamn->spmn', q.to(basis.dtype), basis)
    else:
        V = torch.as_tensor(np.array([ham.dipole_operator(sub, p, tr)
                                      for p, tr in zip(polarization, geometry)],
                                     dtype=complex), device=dev)
    Ld, G, w = model.zofe_tables()
    return _native.zofe_rk4(H, Ld, G, w, y0, nsteps, h, model.unit_convert, save_every,
                            prec, V=V, coef=coef, hermit=model.zofe_hermit)['state']


def simulate_pump(dynamical_model, pump, polarization='x', time_extra=0, times=None,
                  liouville_subspace='gg,ge,eg,ee', save_func=None, ensemble_size=None,
                  ensemble_random_orientations=False, exact_isotropic_average=False,
                  precision='fp64', **integrate_kwargs):
    """A pump pulse acting twice ('-+') (eom.py:173-227).

    ``exact_isotropic_average`` sums the 'xx', 'yy' and 'zz' runs with weight
    (e . e) / 3 (decorators.py:95-125).
    """
    if exact_isotropic_average:
        from ..polarization import check_polarizations
        e = check_polarizations([polarization, polarization], 2)
        weight = float(np.dot(*e))
        total, t = 0, None
        for p in 'xyz':
            t, st = simulate_with_fields(dynamical_model, [pump, pump], '-+', [p, p],
                                         time_extra, times, liouville_subspace,
                                         save_func, ensemble_size,
                                         ensemble_random_orientations, precision,
                                         **integrate_kwargs)
            total = total + st
        return t, total * (weight / 3.0)
    return simulate_with_fields(dynamical_model, [pump, pump], '-+',
                                [polarization, polarization], time_extra, times,
                                liouville_subspace, save_func, ensemble_size,
                                ensemble_random_orientations, precision, **integrate_kwargs)
