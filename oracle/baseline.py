"""CPU baseline for the disorder-ensemble workload (test infrastructure only).

Times the oracle's restatement of the reference path exactly as the
reference runs an ensemble: one sample at a time, each with its own
Hamiltonian sample, Redfield build and RK4 loops (decorators.py:40-64).
Samples are spread over a process pool of the host's cores.
"""
import os
import time

import numpy as np

from .restatement import (CM_FS, CM_K, DebyeBathSpec, ElectronicHamiltonianSpec,
                          RedfieldSpec, rk4_integrate)


def _fmo7_model(H1, extra, disorder_fwhm, seed=1):
    bath = DebyeBathSpec(CM_K * 77, 35, 106)
    ham = ElectronicHamiltonianSpec(H1, dipoles=[[1, 0, 0]] * len(H1),
                                    disorder=disorder_fwhm, random_seed=seed,
                                    energy_spread_extra=extra, bath=bath)
    return RedfieldSpec(ham, bath, 'ge', CM_FS, secular=False)


def fmo7_chunk(args):
    """Absorption signal sum and population sum over samples ns (one worker)."""
    H1, extra, fwhm, ns, abs_time, dyn_time = args
    base = _fmo7_model(np.asarray(H1), extra, fwhm)
    dt = base.time_step
    N = len(H1)
    t_abs = np.arange(0, abs_time, dt)
    t_dyn = np.arange(0, dyn_time, dt)
    sig_sum = np.zeros(len(t_abs), complex)
    pop_sum = np.zeros((len(t_dyn), N))
    for n in ns:
        m = base.sample(n)
        V0 = m.dipole('gg->eg', 'x', '+')
        V1 = m.dipole('eg->gg', 'x', '-')
        v_rho0 = V0.commutator(m.thermal_state('gg'))
        LH = m.eom_matrix('eg', heisenberg_picture=True)
        sig_sum += rk4_integrate(LH, -V1.bra_vector, t_abs) @ v_rho0
        L = m.eom_matrix('ee')
        y0 = np.zeros(N * N, complex)
        y0[0] = 1.0
        states = rk4_integrate(L, y0, t_dyn)
        pop_sum += states[:, [i * N + i for i in range(N)]].real
    return sig_sum, pop_sum


def time_fmo7_samples(H1, extra, fwhm, n_samples, abs_time=2048.0,
                      dyn_time=1000.0, workers=None, pool=None, start=0):
    """Wall time to run ``n_samples`` samples over ``workers`` processes."""
    workers = workers or os.cpu_count() or 1
    chunks = np.array_split(np.arange(start, start + n_samples), workers)
    jobs = [(np.asarray(H1).tolist(), extra, fwhm, c.tolist(), abs_time, dyn_time)
            for c in chunks if len(c)]
    t0 = time.perf_counter()
    if pool is None:
        results = [fmo7_chunk(j) for j in jobs]
    else:
        results = pool.map(fmo7_chunk, jobs)
    wall = time.perf_counter() - t0
    sig = sum(r[0] for r in results) / n_samples
    pop = sum(r[1] for r in results) / n_samples
    return wall, sig, pop
