"""Free time evolution (qspectra/simulate/eom.py:11-74)."""
import numpy as np

from .ensemble import ensemble_populations
from .utils import integrate


def simulate_dynamics(dynamical_model, initial_state, duration=None, times=None,
                      liouville_subspace='ee', save_func=None, ensemble_size=None,
                      ensemble_random_orientations=False, precision='fp64',
                      **integrate_kwargs):
    """Density matrices ρ(t) with no applied field (eom.py:29-74).

    Returns (t, rhos) with rhos (T, N, N) like the reference.  With
    ``ensemble_size`` the disorder average is one batched GPU run.
    """
    if ensemble_size is not None:
        if times is not None or save_func is not None:
            raise NotImplementedError('ensemble dynamics take duration and no save_func')
        t, mean = ensemble_populations(dynamical_model, initial_state, duration,
                                       ensemble_size, liouville_subspace, precision,
                                       full_state=True)
        rhos = dynamical_model.state_vector_to_density_matrix(mean.cpu().numpy())
        return t, rhos
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
