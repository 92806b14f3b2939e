"""Timing of the reference's own code path for the disorder ensemble
(bench.py's reference arm only; never imported by ``qspectra_gb300``).

The reference package is installed under baseline/_ref by
oracle/install_reference.sh and imported from there unmodified.  Python
3.11 removed ``inspect.getargspec``, which the reference's decorators call
(qspectra/simulate/decorators.py:30); it is given back as a view of
``getfullargspec`` before the import, the only accommodation made.

Two figures, as the reference runs an ensemble (decorators.py:40-64):
* as shipped: one process, ``absorption_spectra(model, 2048,
  ensemble_size=S)`` and ``simulate_dynamics(model, psi, 1000,
  ensemble_size=S)`` with the reference's adaptive zvode integrator
  (simulate/utils.py:16-109), one BLAS thread;
* a process pool: the same two calls per disorder sample
  (``hamiltonian.sample(n)``), one sample at a time per worker, over all
  host cores (harness-side parallelism; the reference has none).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.path.join(os.path.dirname(HERE), 'baseline', '_ref')


def available(root=REF_ROOT):
    return os.path.isdir(os.path.join(root, 'qspectra'))


def _import(root=REF_ROOT):
    import inspect
    from collections import namedtuple
    if not hasattr(inspect, 'getargspec'):
        ArgSpec = namedtuple('ArgSpec', 'args varargs keywords defaults')

        def getargspec(func):
            spec = inspect.getfullargspec(func)
            return ArgSpec(spec.args, spec.varargs, spec.varkw, spec.defaults)
        inspect.getargspec = getargspec
    if root not in sys.path:
        sys.path.insert(0, root)
    import warnings
    warnings.simplefilter('ignore')
    import qspectra
    return qspectra


def fmo7_model(qs, H1, extra, fwhm, seed=1):
    ham = qs.ElectronicHamiltonian(np.asarray(H1), bath=qs.DebyeBath(qs.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * len(H1), disorder=fwhm,
                                   random_seed=seed, energy_spread_extra=extra)
    return qs.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qs.CM_FS, secular=False)


def time_as_shipped(H1, extra, fwhm, n_samples, abs_time=2048.0, dyn_time=1000.0):
    """Wall seconds of the reference's own ensemble calls over n_samples."""
    qs = _import()
    m = fmo7_model(qs, H1, extra, fwhm)
    psi = np.zeros(len(H1))
    psi[0] = 1.0
    t0 = time.perf_counter()
    qs.absorption_spectra(m, abs_time, ensemble_size=n_samples)
    qs.simulate_dynamics(m, psi, dyn_time, ensemble_size=n_samples)
    return time.perf_counter() - t0


def _pool_chunk(args):
    H1, extra, fwhm, ns, abs_time, dyn_time = args
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'
    qs = _import()
    m = fmo7_model(qs, np.asarray(H1), extra, fwhm)
    psi = np.zeros(len(H1))
    psi[0] = 1.0
    for n in ns:
        mn = qs.RedfieldModel(m.hamiltonian.sample(n), hilbert_subspace='ge',
                              unit_convert=qs.CM_FS, secular=False)
        qs.absorption_spectra(mn, abs_time)
        qs.simulate_dynamics(mn, psi, dyn_time)
    return len(ns)


def time_pool(H1, extra, fwhm, n_samples, pool, workers, start=0, abs_time=2048.0,
              dyn_time=1000.0):
    """Wall seconds of the reference's per-sample calls over a process pool."""
    chunks = np.array_split(np.arange(start, start + n_samples), workers)
    jobs = [(np.asarray(H1).tolist(), extra, fwhm, c.tolist(), abs_time, dyn_time)
            for c in chunks if len(c)]
    t0 = time.perf_counter()
    pool.map(_pool_chunk, jobs)
    return time.perf_counter() - t0
