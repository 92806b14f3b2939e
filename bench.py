#!/usr/bin/env python3
"""Disorder-averaged spectra per second on one GB300.

Workload (the batched-disorder configuration): 7-site Frenkel exciton
Hamiltonian (E_i ~ U(12000, 12600), J_ij ~ N(0, 50^2), seed 1234), Debye bath
λ = 35 cm^-1, γ = 106 cm^-1, T = 77 K, non-secular Redfield in the 'ge'
Hilbert space, Gaussian static disorder SD 80 cm^-1, 16384 samples.  One
step = the whole ensemble: per-sample Redfield generators, the 'eg'
absorption signal over 2048 points and the 'ee' populations over 1000 points
at dt = 1 fs (RK4), ensemble means and the DFT to the absorption spectrum.
The unit is one disorder-averaged spectrum (all 16384 samples).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ('disorder-averaged spectra/sec at ≤1e-4 rel err vs FP64; '
          'adjoint/forward time')
UNIT = 'spectra/s'
N_SAMPLES = 16384
ABS_TIME, DYN_TIME = 2048.0, 1000.0
CLOCK_QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
               'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
               'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
CONFIG = {'workload': 'fmo7 Redfield ensemble: 7 sites, 16384 disorder samples '
                      '(SD 80 cm^-1), absorption 2048 x 1 fs + ee populations '
                      '1000 x 1 fs',
          'n_samples': N_SAMPLES, 'n_sites': 7, 'dt_fs': 1.0,
          'absorption_points': 2048, 'population_points': 1000,
          'hilbert_subspace': 'ge', 'secular': False,
          'l2': 'no flush needed: each step rebuilds ~1.3 GB of generators and '
                'propagators (> 129 MB L2)'}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=30)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--samples', type=int, default=N_SAMPLES)
    p.add_argument('--cpu-samples-per-core', type=int, default=4)
    p.add_argument('--shipped-samples', type=int, default=16,
                   help='disorder samples of the single-process reference timing')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--fp64-steps', type=int, default=2)
    p.add_argument('--build', choices=['fp32', 'fp64'], default='fp32',
                   help='precision of the eigendecomposition and Redfield build of the '
                        'timed FP32 step (the other one is measured beside)')
    p.add_argument('--no-heom', action='store_true')
    p.add_argument('--only-heom', action='store_true',
                   help='run only the HEOM ring workload (for profiling)')
    p.add_argument('--heom-samples', type=int, default=64)
    p.add_argument('--no-third', action='store_true')
    p.add_argument('--no-adjoint', action='store_true')
    p.add_argument('--no-zofe', action='store_true')
    p.add_argument('--block-k-real', type=int, default=0,
                   help='pin the real population loop\'s block size K (0: measured per '
                        'shape, as a user call does; a profiler distorts that measurement, '
                        'so profiling commands pin the K the plain run reports)')
    p.add_argument('--no-graph', action='store_true',
                   help='time the eager launches only (no CUDA graph capture)')
    p.add_argument('--zofe-samples', type=int, default=152)
    p.add_argument('--only', choices=['heom', 'third', 'adjoint', 'zofe', 'plain'],
                   help='run one auxiliary workload alone and print its JSON')
    p.add_argument('--third-samples', type=int, default=256)
    p.add_argument('--third-reps', type=int, default=2)
    p.add_argument('--third-fp64-samples', type=int, default=8,
                   help='samples of the FP32-vs-FP64 check (0 skips it)')
    p.add_argument('--adjoint-samples', type=int, default=1024)
    p.add_argument('--adjoint-adam-steps', type=int, default=200)
    p.add_argument('--no-adjoint-checks', action='store_true',
                   help='skip the finite-difference and autograd gradient checks')
    p.add_argument('--heom-steps', type=int, default=1999)
    return p.parse_args()


LIB_KERNELS_PER_STEP = 15


def fmo7_inputs():
    from qspectra_gb300 import workloads as wl
    from qspectra_gb300.constants import CM_FS
    H = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H, 1.0, CM_FS)
    return H, extra, wl.fwhm_for_sd(80.0)


# ----------------------------------------------------------------- clocks
def clocks_start(index=0):
    try:
        return subprocess.Popen(['nvidia-smi', '--query-gpu=' + CLOCK_QUERY,
                                 '--format=csv,noheader,nounits', '-lms', '50',
                                 '-i', str(index)],
                                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                text=True)
    except OSError:
        return None


def clocks_stop(proc):
    if proc is None:
        return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
    proc.terminate()
    try:
        out, _ = proc.communicate(timeout=10)
    except subprocess.TimeoutExpired:
        proc.kill()
        out, _ = proc.communicate()
    sm, smax, reasons, power = [], [], set(), []
    names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
    for line in out.strip().splitlines():
        f = [x.strip() for x in line.split(',')]
        if len(f) < 9:
            continue
        try:
            sm.append(float(f[1]))
            smax.append(float(f[2]))
            power.append(float(f[3]))
        except ValueError:
            continue
        for name, val in zip(names, f[5:9]):
            if val.lower().startswith('active'):
                reasons.add(name)
    if not sm:
        return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}
    return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax),
            'power_w_max': max(power) if power else None, 'samples': len(sm),
            'reasons': sorted(reasons)}


# ------------------------------------------------------------ CPU baseline
def cpu_baseline(H, extra, fwhm, per_core, n_full=N_SAMPLES, steps=1, warmup=0):
    """CPU baseline over a spawn pool of all host cores: the reference's own
    per-sample calls (absorption_spectra + simulate_dynamics, zvode) when the
    reference is installed under baseline/_ref, else the oracle port of the
    same path.  Each measurement is a bounded sample of ``per_core`` samples
    per core; spectra/s is extrapolated linearly to ``n_full`` samples."""
    import multiprocessing as mp
    from oracle import baseline as ob
    from oracle import reference_shipped as rs
    cores = os.cpu_count() or 1
    n = per_core * cores
    ctx = mp.get_context('spawn')
    # one BLAS thread per worker process (spawned children read these at import)
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'
    ref = rs.available()
    vals, walls = [], []
    with ctx.Pool(cores) as pool:
        if ref:
            rs.time_pool(H, extra, fwhm, cores, pool, cores)   # warm (imports)
        else:
            ob.time_fmo7_samples(H, extra, fwhm, cores, workers=cores, pool=pool)
        for k in range(warmup + steps):
            if ref:
                wall = rs.time_pool(H, extra, fwhm, n, pool, cores, start=k * n)
            else:
                wall, _, _ = ob.time_fmo7_samples(H, extra, fwhm, n, workers=cores, pool=pool,
                                                  start=k * n)
            if k >= warmup:
                vals.append(1.0 / (wall / n * n_full))
                walls.append(wall)
    what = ("the reference's own absorption_spectra + simulate_dynamics calls (baseline/_ref, "
            "zvode), one disorder sample at a time per process" if ref else
            'the oracle port of the same path (RK4), one disorder sample at a time per process')
    return {'value': float(np.mean(vals)), 'unit': UNIT, 'cores': cores,
            'kind': 'reference' if ref else 'port',
            'ms_per_measurement': 1000.0 * float(np.mean(walls)),
            'sample': '{} disorder samples per measurement ({} per core): {}; spectra/s '
                      'extrapolated linearly to {} samples'.format(n, per_core, what, n_full)}


def reference_as_shipped(H, extra, fwhm, samples, n_full=N_SAMPLES, reps=1):
    """The reference as shipped: one process, one BLAS thread, its own
    ensemble loop (ensemble_size=samples) over absorption_spectra and
    simulate_dynamics; run in a spawned child so the thread setting holds."""
    import multiprocessing as mp
    from oracle import reference_shipped as rs
    if not rs.available():
        return {'unavailable': 'baseline/_ref not installed (oracle/install_reference.sh)'}
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'
    ctx = mp.get_context('spawn')
    with ctx.Pool(1) as pool:
        pool.apply(rs.time_as_shipped, (H, extra, fwhm, 1))   # warm (imports)
        walls = [pool.apply(rs.time_as_shipped, (H, extra, fwhm, samples))
                 for _ in range(reps)]
    wall = float(np.mean(walls))
    return {'value': 1.0 / (wall / samples * n_full), 'unit': UNIT, 'cores': 1,
            'kind': 'reference', 'ms_per_sample': 1000.0 * wall / samples,
            'sample': 'absorption_spectra(model, 2048, ensemble_size={0}) + '
                      'simulate_dynamics(model, psi, 1000, ensemble_size={0}) of the '
                      'reference (baseline/_ref, zvode), one process, one BLAS thread; '
                      'spectra/s extrapolated linearly to {1} samples'.format(samples, n_full)}


def reference_arm(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    H, extra, fwhm = fmo7_inputs()
    base = cpu_baseline(H, extra, fwhm, args.cpu_samples_per_core, args.samples,
                        steps=args.steps, warmup=args.warmup)
    val = base['value']
    line = {'metric': METRIC, 'value': val, 'unit': UNIT, 'impl': 'reference',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': base['ms_per_measurement'],
            'ms_per_step_note': ('measured wall time of one step, a bounded sample of the '
                                 'ensemble; value extrapolates it to the full {} samples'
                                 .format(args.samples)),
            'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c128',
            'data': 'synthetic (seeded)', 'config': dict(CONFIG),
            'cpu_baseline': base,
            'reference_as_shipped': reference_as_shipped(H, extra, fwhm,
                                                         args.shipped_samples, args.samples),
            'e2e': {'value': val, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------- GPU arm
def fma_peak_tflops(torch, native, precision=None):
    """Measured CUDA-core FMA peak (TFLOP/s) from the benchmark's own probe
    library (libqsx_probe.so, built beside libqsx.so)."""
    import ctypes
    from qspectra_gb300 import build as qbuild
    if precision is None:
        precision = native.QSX_FP32
    probe = ctypes.CDLL(qbuild.PROBE_LIB)
    probe.qsx_probe_fma.restype = ctypes.c_int
    probe.qsx_probe_fma.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    fp32 = precision == native.QSX_FP32
    blocks, threads, iters = sms * 8, 256, (4000 if fp32 else 250)
    out = torch.empty(blocks * threads, dtype=torch.float32 if fp32 else torch.float64,
                      device='cuda')
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        st = probe.qsx_probe_fma(precision, blocks, threads, iters, out.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
        if st != 0:
            raise RuntimeError('qsx_probe_fma failed with status {}'.format(st))
        e1.record()
        torch.cuda.synchronize()
        flops = 2.0 * blocks * threads * iters * 16 * 8
        best = max(best, flops / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def heom_ring8(torch, qg, native, samples=64, nsteps=1999):
    """HEOM workload: 8-site ring, K = 0, depth 4 (495 nodes x 64), 64 disorder
    samples (SD 50 cm^-1), 1 ps at dt = 0.5 fs; FP32 split-word and FP64."""
    from qspectra_gb300 import workloads as wl
    H = wl.ring_hamiltonian()
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 35, 106),
                                   disorder=wl.fwhm_for_sd(50.0), random_seed=7)
    m = qg.HEOMModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS, K=0, level_cutoff=5,
                     low_temp_corr=True)
    tb = m.tables('ee')
    offs = m.hamiltonian.disorder_offsets(samples)
    base = m.hamiltonian.H('e')
    Hb = torch.as_tensor(np.array([base + np.diag(o) for o in offs])).cuda()
    y0 = torch.zeros(m.ado_count * 64, dtype=torch.complex128, device='cuda')
    y0[0] = 1.0
    out = {'workload': 'HEOM 8-site ring, K=0, depth 4 (495 nodes), {} samples, '
                       '{} RK4 steps at 0.5 fs'.format(samples, nsteps), 'nodes': m.ado_count}
    res = {}
    for name, prec, steps in (('fp32', native.QSX_FP32, nsteps),
                              ('fp64', native.QSX_FP64, min(200, nsteps))):
        native.heom_rk4(tb, Hb, Hb, y0, 10, 0.5, qg.CM_FS, batch=samples, save_every=10,
                        precision=prec, per_sample=False, mean=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r = native.heom_rk4(tb, Hb, Hb, y0, steps, 0.5, qg.CM_FS, batch=samples, save_every=1,
                            precision=prec, per_sample=False, mean=True, check_finite=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        res[name] = r['mean']
        out[name + '_ms'] = ms * (nsteps / steps)
        out[name + '_steps_timed'] = steps
    # the forms forced, FP32 over 200 steps, scaled: the per-stage kernels
    # (one launch per RK4 stage, a warp per node block), the persistent
    # cluster kernel (one cluster of CTAs per sample for the whole loop) and
    # the per-stage kernels with the node commutators on the tensor cores
    for key, variant in (('fp32_per_stage_kernels_ms', 1), ('fp32_cluster_kernel_ms', 2),
                         ('fp32_tensor_core_commutators_ms', 3),
                         ('fp32_per_stage_all_terms_ms', 4)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        native.heom_rk4(tb, Hb, Hb, y0, 200, 0.5, qg.CM_FS, batch=samples, save_every=1,
                        precision=native.QSX_FP32, per_sample=False, mean=True,
                        check_finite=False, variant=variant)
        e1.record()
        torch.cuda.synchronize()
        out[key] = e0.elapsed_time(e1) * (nsteps / 200)
    out['form'] = ('library choice (fp32_ms, fp64_ms): the persistent cluster kernel when every '
                   "sample's cluster is resident at once, else per-stage kernels with a warp "
                   'per node block; both forced beside, and the per-stage kernels with '
                   'the node commutators on the tensor cores (variant 3)')
    k = res['fp64'].shape[0]
    a, b = res['fp32'][:k], res['fp64']
    out['fp32_vs_fp64_rel_err_first_{}_steps'.format(k - 1)] = float(
        (a - b).abs().max() / b.abs().max())
    # structured generator: 495 nodes x (2 x 8^3 commutator + coupling terms) per RHS
    flops = 8.0 * samples * 4 * nsteps * m.ado_count * (2 * 8 ** 3 + 64 * tb.nterms)
    out['fp32_tflops_executed_form'] = flops / (out['fp32_ms'] * 1e-3) / 1e12
    out['fp64_ms_note'] = 'FP64 timed over {} steps and scaled to {}'.format(min(200, nsteps),
                                                                             nsteps)
    return out


def plain_fmo7(torch, qg, reps=5, cpu=True):
    """The single-model workload (no disorder) through the public API, as a
    user calls it: simulate_dynamics of the 'ee' populations from site 1 over
    1 ps and absorption_spectra over 2048 steps, dt 1 fs, in FP64 (the plain
    form) and in FP32; the reference's own two calls (zvode, one process, one
    BLAS thread) beside it."""
    H, extra, _ = fmo7_inputs()
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, energy_spread_extra=extra)
    model = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    psi = np.zeros(7)
    psi[0] = 1.0
    out = {'workload': 'fmo7 single model: simulate_dynamics (ee, 1000 x 1 fs) + '
                       'absorption_spectra (2048 x 1 fs), no disorder, public API calls'}
    res = {}
    for prec in ('fp64', 'fp32'):
        def call():
            _, rho = qg.simulate_dynamics(model, psi, 1000.0, precision=prec)
            _, X = qg.absorption_spectra(model, 2048.0, precision=prec)
            return np.asarray(rho), np.asarray(X)
        call()
        times = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res[prec] = call()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        out[prec + '_ms'] = 1000.0 * statistics.median(times)
    r64, x64 = res['fp64']
    r32, x32 = res['fp32']
    out['fp32_vs_fp64_rel_err'] = {
        'populations': float(np.abs(r32 - r64).max() / np.abs(r64).max()),
        'spectrum': float(np.abs(x32 - x64).max() / np.abs(x64).max())}
    if cpu:
        import multiprocessing as mp
        from oracle import reference_shipped as rs
        if rs.available():
            for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
                os.environ[var] = '1'
            with mp.get_context('spawn').Pool(1) as pool:
                pool.apply(rs.time_as_shipped, (H, extra, 0.0, 1))   # warm (imports)
                walls = [pool.apply(rs.time_as_shipped, (H, extra, 0.0, 1)) for _ in range(3)]
            out['cpu_baseline'] = {
                'value': 1000.0 * statistics.median(walls), 'unit': 'ms', 'cores': 1,
                'kind': 'reference',
                'sample': "the reference's absorption_spectra(model, 2048) + simulate_dynamics("
                          "model, psi, 1000) on one model (baseline/_ref, zvode), one process"}
    return out


def zofe_fmo7(torch, qg, native, samples=152, reps=2):
    """ZOFE workload: 7 sites with 16 pseudomodes per site (seeded
    parameters), dt = 1 fs.  Single-model calls through the public API, timed
    end to end (wall clock, after a warm-up call): 'e' dynamics for 1000 fs
    (5537 state components), a pump pulse on 'ge' over 1000 fs after it
    (7232 components) and the 'ge' absorption spectrum from 2000 fs; then the
    disorder-averaged spectrum of ``samples`` samples in one launch."""
    from qspectra_gb300 import workloads as wl
    H = wl.fmo7_hamiltonian()
    extra = wl.energy_spread_for_dt(H, 1.0, qg.CM_FS)
    bath = qg.PseudomodeBath(16, *wl.pseudomode_parameters(7, 16))
    ham = qg.ElectronicHamiltonian(H, bath=bath, dipoles=wl.unit_dipoles(7),
                                   disorder=wl.fwhm_for_sd(80.0), random_seed=1,
                                   energy_spread_extra=extra)
    m_e = qg.ZOFEModel(ham, hilbert_subspace='e', unit_convert=qg.CM_FS)
    m_ge = qg.ZOFEModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS)
    pump = qg.GaussianPulse(12500.0, 50.0, scale=1e-3, freq_convert=qg.CM_FS)
    psi = np.zeros(7)
    psi[0] = 1.0
    calls = {
        'dynamics_e_1000fs': lambda p: qg.simulate_dynamics(m_e, psi, 1000.0, precision=p),
        'pump_ge_1000fs': lambda p: qg.simulate_pump(m_ge, pump, 'x', 1000.0, precision=p),
        'absorption_ge_2000fs': lambda p: qg.absorption_spectra(m_ge, 2000.0, precision=p),
    }
    out = {'workload': 'ZOFE 7 sites x 16 pseudomodes, dt 1 fs; single-model calls end to '
                       'end, plus a {}-sample ensemble absorption in one launch'.format(samples)}
    res = {}
    for name, fn in calls.items():
        for prec in ('fp64', 'fp32'):
            fn(prec)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                r = fn(prec)
            torch.cuda.synchronize()
            out['{}_{}_ms'.format(name, prec)] = (time.perf_counter() - t0) * 1e3 / reps
            res[name, prec] = np.asarray(r[1])
        a, b = res[name, 'fp32'], res[name, 'fp64']
        out[name + '_fp32_vs_fp64_rel_err'] = float(np.abs(a - b).max() / np.abs(b).max())
    # CPU baseline: the oracle's NumPy restatement of the same 'e' dynamics on
    # one host thread, 200 of the 1000 steps, scaled
    import oracle
    om = oracle.ZOFESpec(oracle.ElectronicHamiltonianSpec(H, dipoles=wl.unit_dipoles(7),
                                                          energy_spread_extra=extra),
                         *wl.pseudomode_parameters(7, 16), hilbert_subspace='e',
                         unit_convert=qg.CM_FS)
    t0 = time.perf_counter()
    oracle.zofe_dynamics(om, psi, 200.0)
    out['cpu_baseline'] = {'value': (time.perf_counter() - t0) * 1e3 * 5, 'unit': 'ms',
                           'cores': 1, 'kind': 'port',
                           'sample': "dynamics_e_1000fs: 200 of 1000 RK4 steps, scaled"}
    for prec in ('fp32', 'fp64'):
        qg.absorption_spectra(m_ge, 2000.0, ensemble_size=samples, precision=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        qg.absorption_spectra(m_ge, 2000.0, ensemble_size=samples, precision=prec)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        out['ensemble_absorption_{}_ms'.format(prec)] = ms
        out['ensemble_absorption_{}_spectra_per_s'.format(prec)] = samples / (ms * 1e-3)
    return out


def third_order_chain24(torch, qg, samples=256, fp64_samples=8, reps=2, warm=True):
    """Third-order response: 24-site chain (E ~ N(12300, 100^2), -80 / +15
    cm^-1 couplings, seed 2024), Debye bath lambda = 40, gamma = 100, 300 K,
    non-secular Redfield on 'gef' (276 two-exciton states), t1 = t3 = 128 x
    2 fs, t2 in {0, 200, 500} fs, rephasing and non-rephasing geometries
    (GSB + ESE + ESA each), 256 disorder samples (SD 60 cm^-1), FP32 bulk."""
    from qspectra_gb300 import workloads as wl
    from qspectra_gb300.simulate.third_order import ThirdOrderEngine
    H = wl.chain_hamiltonian(n_sites=24, seed=2024)
    extra = wl.energy_spread_for_dt(H, 2.0, qg.CM_FS)
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 300, 40, 100),
                                   dipoles=[[1, 0, 0]] * 24, disorder=wl.fwhm_for_sd(60.0),
                                   random_seed=3, energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='gef', unit_convert=qg.CM_FS, secular=False)
    offs = m.hamiltonian.disorder_offsets(samples)
    eng = ThirdOrderEngine(m, 256.0, [0.0, 200.0, 500.0], precision='fp32')
    if warm:
        eng.run(offs)
        torch.cuda.synchronize()
    best, phases = None, None
    for _ in range(reps):
        ev = {}
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = eng.run(offs, events=ev)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if best is None or ms < best:
            mk = ev['marks']
            best = ms
            phases = {mk[i][0]: mk[i][1].elapsed_time(mk[i + 1][1]) for i in range(len(mk) - 1)}
    err = None
    if fp64_samples:
        sub = offs[:fp64_samples]
        r64 = ThirdOrderEngine(m, 256.0, [0.0, 200.0, 500.0], precision='fp64').run(sub)
        r32 = ThirdOrderEngine(m, 256.0, [0.0, 200.0, 500.0], precision='fp32').run(sub)
        err = max(float((r32[g] - r64[g]).abs().max() / r64[g].abs().max()) for g in r64)
    return {'workload': '24-site chain third-order response, 276 two-exciton states, '
                        't1 = t3 = 128 x 2 fs, t2 = 0/200/500 fs, both geometries, '
                        '{} samples (SD 60 cm^-1), FP32 bulk'.format(samples),
            'ms_per_ensemble': best, 'ensembles_per_s': 1000.0 / best,
            'phases_ms': phases,
            'fp32_vs_fp64_rel_err': err, 'fp64_check_samples': fp64_samples,
            'output_shape': list(out['-++'].shape)}


def adjoint_fmo7(torch, qg, samples=1024, adam_steps=200, checks=True):
    """Gradient of the absorption misfit (1024 frequencies, 11800-13000 cm^-1)
    of the 7-site model's 1024-sample ensemble (SD 80 cm^-1) w.r.t. 7 site
    energies, 21 couplings and lambda; 2048 points at 1 fs, checkpoints every
    64 steps.  Adjoint time vs forward time, FD and autograd checks, Adam."""
    from qspectra_gb300 import workloads as wl
    from qspectra_gb300.simulate.adjoint import AbsorptionFit
    H7, extra, fwhm = fmo7_inputs()
    ham = qg.ElectronicHamiltonian(H7, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=fwhm, random_seed=1,
                                   energy_spread_extra=extra)
    m = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS, secular=False)
    freqs = np.linspace(11800.0, 13000.0, 1024)
    fit = AbsorptionFit(7, ham.disorder_offsets(samples), freqs, rw_freq=m.rw_freq, dt=1.0,
                        nsteps=2047, ck_every=64)
    theta_true = fit.pack(H7, 35.0)
    target = fit.spectrum(theta_true).detach()
    rng = np.random.RandomState(11)
    theta0 = theta_true.clone()
    theta0[:7] += torch.as_tensor(rng.randn(7) * 8.0).cuda()
    theta0[7:-1] += torch.as_tensor(rng.randn(21) * 4.0).cuda()
    theta0[-1] += 5.0

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) * 1000.0
            best = dt if best is None else min(best, dt)
        return best

    def forward():
        with torch.no_grad():
            return fit.misfit(theta0, target)

    holder = {}

    def fwd_graph():
        th = theta0.clone().requires_grad_(True)
        holder['th'] = th
        holder['loss'] = fit.misfit(th, target)

    def bwd():
        holder['loss'].backward()

    fwd_ms = timed(forward)
    fwdg_ms = timed(fwd_graph)
    bwd_samples = []
    for _ in range(5):
        fwd_graph()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bwd()
        torch.cuda.synchronize()
        bwd_samples.append((time.perf_counter() - t0) * 1000.0)
    bwd_ms = min(bwd_samples)
    g_adj = holder['th'].grad.detach().cpu().numpy()
    rel = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())  # noqa: E731
    out = {}
    if checks:
        th2 = theta0.clone().requires_grad_(True)
        fit.misfit(th2, target, impl='autograd').backward()
        g_ref = th2.grad.detach().cpu().numpy()
        h = 1e-3
        fd = np.zeros_like(g_adj)
        with torch.no_grad():
            for i in range(len(fd)):
                e = torch.zeros_like(theta0)
                e[i] = h
                fd[i] = ((fit.misfit(theta0 + e, target) - fit.misfit(theta0 - e, target))
                         / (2 * h)).item()
        out['grad_rel_err_vs_central_fd_h1e-3'] = rel(g_adj, fd)
        out['grad_rel_err_vs_fp64_autograd_rk4'] = rel(g_adj, g_ref)
    if adam_steps:
        t0 = time.perf_counter()
        theta_fit, hist = fit.fit(theta0, target, steps=adam_steps, lr=0.5)
        torch.cuda.synchronize()
        adam_s = time.perf_counter() - t0
        err0 = (theta0 - theta_true).abs()
        err1 = (theta_fit - theta_true).abs()
        out['adam'] = {'steps': adam_steps, 'lr': 0.5, 'seconds': adam_s,
                       'misfit_start': hist[0], 'misfit_end': hist[-1],
                       'max_abs_err_start_cm': float(err0.max()),
                       'max_abs_err_end_cm': float(err1.max()),
                       'site_energy_err_end_cm': float(err1[:7].max()),
                       'coupling_err_end_cm': float(err1[7:-1].max()),
                       'lambda_end': float(theta_fit[-1])}
    return dict({'workload': '7-site Redfield absorption misfit on 1024 frequencies '
                        '(11800-13000 cm^-1), {} disorder samples (SD 80 cm^-1), 2048 x '
                        '1 fs, checkpoints every 64 steps, 29 parameters'.format(samples),
            'forward_ms': fwd_ms, 'forward_with_graph_ms': fwdg_ms, 'adjoint_ms': bwd_ms,
            'adjoint_over_forward': bwd_ms / fwd_ms}, **out)


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured (MEASURED_PEAKS.json)'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback (6.8 TB/s)'


def measured_tf32_tflops():
    """Dense TF32 tensor rate: half the measured cuBLAS bf16 burst rate (the
    dense TF32 rate is half the bf16 rate on this part: 1.1 vs 2.25 PFLOP/s
    nominal)."""
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return (float(json.load(f)['bf16_tflops']) / 2.0,
                    'measured: MEASURED_PEAKS.json bf16_tflops / 2 (dense TF32 = half bf16)')
    except (OSError, KeyError, ValueError):
        return 1900.0 / 2.0, 'fallback: 1.9 PFLOP/s bf16 / 2'


def block_roofline(events, bb_flops, bb_ms, fma_peak):
    """Roofline of the FP32 K-step block build: the tcgen05 3xTF32 kernel
    against the dense TF32 tensor rate, or the CUDA-core kernel against the
    FP32 FMA rate.  `achieved` counts the algorithmic (unpadded) FLOPs;
    `executed_tensor_tflops` the MMA work actually issued (three TF32
    products of M = 128, N = NP, K = KP per chain)."""
    bb_achieved = bb_flops / (bb_ms * 1e-3) / 1e12 if bb_ms else None
    K = events['dyn_block_k']
    if events.get('blockbuild_variant') == 'tcgen05':
        B, m, K, nsel = events['blockbuild_shape']
        kp, np_ = (m + 7) // 8 * 8, (m + 15) // 16 * 16
        chains = (K.bit_length() - 1) + (0 if K & (K - 1) == 0 else 1)
        executed = float(B) * chains * 3 * 2 * 128 * np_ * kp
        traffic = ncu_traffic(os.path.join(ROOT, 'profiles', 'block_matrix_tc_fmo7.md'))
        peak, src = measured_tf32_tflops()
        ex = executed / (bb_ms * 1e-3) / 1e12 if bb_ms else None
        return {'kernel': 'block_matrix_tc_kernel<32> (ee populations, real Hermitian form: '
                          'K={} step blocked matrices, tcgen05 3xTF32 products in TMEM)'.format(K),
                'bound': 'tensor', 'achieved': bb_achieved, 'peak': peak, 'unit': 'TFLOP/s',
                'frac': bb_achieved / peak if bb_achieved else None, 'peak_source': src,
                'executed_tensor_tflops': ex, 'executed_frac': ex / peak if ex else None,
                'executed_flops_per_launch': executed,
                'fp32_fma_view': {'peak': fma_peak, 'frac': bb_achieved / fma_peak
                                  if bb_achieved else None,
                                  'peak_source': 'measured live by the FMA probe (libqsx_probe.so)'},
                'flops_per_launch': bb_flops, 'launch_ms': bb_ms,
                'traffic': traffic, 'hbm': hbm_view(traffic, bb_ms)}
    traffic = ncu_traffic(os.path.join(ROOT, 'profiles', 'block_matrix_real_fmo7.md'))
    return {'kernel': 'block_matrix_real_kernel<float> (ee populations, real Hermitian form: '
                      'K={} step blocked matrices, 4x4-tiled FP32 products)'.format(K),
            'bound': 'fp32_fma', 'achieved': bb_achieved, 'peak': fma_peak, 'unit': 'TFLOP/s',
            'frac': bb_achieved / fma_peak if bb_achieved else None,
            'peak_source': 'measured live by the FMA probe (libqsx_probe.so, FP32 FMA); '
                           'MEASURED_PEAKS.json has no CUDA-core figure',
            'flops_per_launch': bb_flops, 'launch_ms': bb_ms,
            'traffic': traffic, 'hbm': hbm_view(traffic, bb_ms)}


def hbm_view(traffic, launch_ms):
    """The same kernel against the HBM roofline: ncu DRAM bytes per launch
    over the CUDA-event launch time, as a fraction of the measured copy
    bandwidth."""
    peak, src = measured_hbm_gbs()
    if not traffic or not launch_ms:
        return {'peak_gbs': peak, 'peak_source': src, 'achieved_gbs': None, 'frac': None}
    gbs = traffic / (launch_ms * 1e-3) / 1e9
    return {'achieved_gbs': gbs, 'peak_gbs': peak, 'frac': gbs / peak, 'peak_source': src}


def ncu_traffic(path=os.path.join(ROOT, 'profiles', 'rk4_block_f32_fmo7.md')):
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r'traffic_bytes_per_full_launch:\s*([0-9.eE+]+)', txt)
    return float(m.group(1)) if m else None


def replica_sample_start(rank, samples_per_rank):
    """First disorder-sample index of a rank's replica: the ranks take
    disjoint consecutive ranges of the same seeded draws (weak scaling, no
    data-path collective)."""
    return rank * samples_per_rank


def max_over_ranks(values, world, device):
    """Element-wise MAX of a list of floats over the ranks (every rank gets
    it); the values themselves when there is one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def whole_job_rate(world, ms_per_step):
    """Ensembles per second of the whole job: every rank finishes one
    ensemble per step, and the step takes the slowest rank's time."""
    return world * 1000.0 / ms_per_step


def our_arm(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')
    import qspectra_gb300 as qg
    from qspectra_gb300 import _native
    from qspectra_gb300.simulate.ensemble import (RedfieldEnsembleWorkload, block_k_real_timings,
                                                  set_block_k_real)
    if args.block_k_real:
        set_block_k_real(args.block_k_real)

    H, extra, fwhm = fmo7_inputs()
    S = args.samples
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=fwhm, random_seed=1,
                                   energy_spread_extra=extra)
    model = qg.RedfieldModel(ham, hilbert_subspace='ge', unit_convert=qg.CM_FS,
                             secular=False)
    psi = np.zeros(7)
    psi[0] = 1.0
    work = RedfieldEnsembleWorkload(model, ABS_TIME, DYN_TIME, psi)
    off_host = torch.as_tensor(model.hamiltonian.disorder_offsets(
        S, start=replica_sample_start(rank, S))).pin_memory()
    off = off_host.cuda()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        work.run(off, 'fp32', build_precision=args.build)
    barrier()
    clk = clocks_start(local) if rank == 0 else None
    if clk is not None:
        time.sleep(0.6)  # the sampler's first reading lands inside the timed region
    events = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        X32, P32, status = work.run(off, 'fp32', events, build_precision=args.build)
    e1.record()
    barrier()
    eager_ms = e0.elapsed_time(e1) / args.steps
    # the batching form, measured: the two legs of a step (the absorption leg
    # on a side stream, the population leg on the caller's stream) and the
    # whole step with both legs on one stream
    legs = {'build_ms': statistics.mean(a.elapsed_time(b) for a, b in events['build']),
            'absorption_leg_ms': statistics.mean(a.elapsed_time(b) for a, b in events['abs_leg']),
            'population_leg_ms': statistics.mean(a.elapsed_time(b)
                                                 for a, b in events['pop_leg'])}
    work.overlap = False
    for _ in range(2):
        work.run(off, 'fp32', build_precision=args.build)
    barrier()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record()
    for _ in range(args.steps):
        work.run(off, 'fp32', build_precision=args.build)
    s1.record()
    barrier()
    work.overlap = True
    one_stream_ms = s0.elapsed_time(s1) / args.steps
    # the same step as one CUDA graph launch (the library's capture/replay of
    # a step, checked bit for bit against the eager steps): when capture
    # succeeds it is the timed form for `value`, and the end-to-end calls
    # below go through run_host, which replays it; the eager time is
    # reported beside
    graph_ok = (not args.no_graph) and work.capture(off, 'fp32', build_precision=args.build)
    ms = eager_ms
    graph_ms = None
    if graph_ok:
        for _ in range(args.warmup):
            work.replay()
        barrier()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record()
        for _ in range(args.steps):
            Xg, Pg, status = work.replay()
        g1.record()
        barrier()
        graph_ms = g0.elapsed_time(g1) / args.steps
        graph_vs_eager = max(float((Xg - X32).abs().max() / X32.abs().max()),
                             float((Pg - P32).abs().max() / P32.abs().max()))
    clocks = clocks_stop(clk) if rank == 0 else None
    if world > 1:
        ms, gmax = max_over_ranks([ms, graph_ms or 0.0], world, 'cuda')
        graph_ms = gmax if graph_ok else None
    eager_ms = ms
    if graph_ok and graph_vs_eager <= 1e-12:   # the replay must reproduce the step
        ms = graph_ms
    if int(status.item()) & _native.QSX_ERR_NONFINITE:
        raise _native.IntegratorError('non-finite state in the timed run')
    value = whole_job_rate(world, ms)
    dyn_ms = statistics.mean(a.elapsed_time(b) for a, b in events['dyn'])
    bb_ms = (statistics.mean(a.elapsed_time(b) for a, b in events['blockbuild'])
             if events.get('blockbuild') else None)

    # end to end through the library call with host buffers
    for _ in range(2):
        work.run_host(off_host, 'fp32', build_precision=args.build)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Xh, Ph = work.run_host(off_host, 'fp32', build_precision=args.build)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    e2e_ms = max_over_ranks([e2e_ms], world, 'cuda')[0]

    # plain FP64 form, side by side, and the FP32 error against it
    work.run(off, 'fp64')
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.fp64_steps):
        X64, P64, _ = work.run(off, 'fp64')
    f1.record()
    torch.cuda.synchronize()
    fp64_ms = f0.elapsed_time(f1) / args.fp64_steps
    err_spec = float((X32 - X64).abs().max() / X64.abs().max())
    err_pop = float((P32 - P64).abs().max() / P64.abs().max())
    # the other build precision beside: the FP64 build (FP64 eigenpairs and
    # Redfield operators feeding FP32 propagation) or the FP32 build
    other = 'fp64' if args.build == 'fp32' else 'fp32'
    for _ in range(2):
        work.run(off, 'fp32', build_precision=other)
    torch.cuda.synchronize()
    o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev_other = {}
    o0.record()
    for _ in range(args.fp64_steps + 3):
        Xo, Po, _ = work.run(off, 'fp32', ev_other, build_precision=other)
    o1.record()
    torch.cuda.synchronize()
    other_ms = o0.elapsed_time(o1) / (args.fp64_steps + 3)
    build_ms = {args.build: statistics.mean(a.elapsed_time(b) for a, b in events['build']),
                other: statistics.mean(a.elapsed_time(b) for a, b in ev_other['build'])}
    precision_forms = {
        'value_form': {'build': args.build, 'propagation': 'fp32 split-word',
                       'ms_per_step': ms, 'build_ms': build_ms[args.build],
                       'rel_err_vs_fp64': {'spectrum': err_spec, 'populations': err_pop}},
        'other_form': {'build': other, 'propagation': 'fp32 split-word',
                       'ms_per_step_eager': other_ms, 'spectra_per_s_eager': 1000.0 / other_ms,
                       'build_ms': build_ms[other],
                       'rel_err_vs_fp64': {
                           'spectrum': float((Xo - X64).abs().max() / X64.abs().max()),
                           'populations': float((Po - P64).abs().max() / P64.abs().max())}},
        'note': ('fp64 build = FP64 eigenpairs (FP32 Jacobi refined in FP64) and FP64 '
                 'Redfield operators (qsx_redfield_build_w64); fp32 build = the same formulas '
                 'in FP32; propagation FP32 split-word either way')}

    heom = heom_ring8(torch, qg, _native) if rank == 0 and not args.no_heom else None
    third = (third_order_chain24(torch, qg, samples=args.third_samples)
             if rank == 0 and not args.no_third else None)
    adj = (adjoint_fmo7(torch, qg, samples=args.adjoint_samples)
           if rank == 0 and not args.no_adjoint else None)
    zofe = (zofe_fmo7(torch, qg, _native, samples=args.zofe_samples)
            if rank == 0 and not args.no_zofe else None)
    plain = plain_fmo7(torch, qg, cpu=not args.no_cpu_baseline) if rank == 0 else None
    if rank != 0:
        return 0
    peak = fma_peak_tflops(torch, _native)
    # the plain FP64 form against the measured FP64 FMA rate.  Its algorithmic
    # work per step: the step-by-step complex loops in propagator form (one
    # complex GEMV per RK4 step: ee 49 x 49, eg 7 x 7; 8 flops per complex
    # multiply-add) and the two one-step propagators (two complex m^3
    # products each, Paterson-Stockmeyer)
    peak64 = fma_peak_tflops(torch, _native, _native.QSX_FP64)
    m_ee, m_eg = len(work.idx_ee), len(work.idx_eg)
    n_dyn, n_abs = len(work.t_dyn) - 1, len(work.t_abs) - 1
    fp64_flops = 8.0 * S * (n_dyn * m_ee ** 2 + n_abs * m_eg ** 2 + 2 * (m_ee ** 3 + m_eg ** 3))
    fp64_achieved = fp64_flops / (fp64_ms * 1e-3) / 1e12
    flops_dyn = events['dyn_flops']  # executed form (K-step blocked rows)
    dense_equiv = float(S) * (DYN_TIME - 1) * 49 * 49 * 8  # one 49x49 GEMV per step
    achieved = flops_dyn / (dyn_ms * 1e-3) / 1e12
    traffic = ncu_traffic(os.path.join(ROOT, 'profiles', 'rk4_real_two_pass_fmo7.md'))
    bb_flops = events.get('blockbuild_flops')
    base = None
    if world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(H, extra, fwhm, 4 * args.cpu_samples_per_core, S, steps=3)
    nf = Xh.size
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': ('f32/c64 split-word propagation (populations in the real Hermitian form) '
                  'after an {} eigendecomposition and Redfield build'.format(
                      'FP64' if args.build == 'fp64' else 'FP32')),
        'data': 'synthetic (seeded Hamiltonians and disorder draws)',
        'config': dict(CONFIG, parallelism='replicas (weak: each GPU runs its own '
                                           '16384-sample ensemble)' if world > 1 else 'single GPU'),
        'fp32_vs_fp64_rel_err': {'spectrum': err_spec, 'populations': err_pop},
        'precision_forms': precision_forms,
        'step_launch': ({'value': ('captured CUDA graph (replay)' if ms == graph_ms
                                   else 'eager launches (replay differed)'),
                         'e2e': 'captured CUDA graph (run_host)',
                         'eager_ms_per_step': eager_ms,
                         'graph_vs_eager_rel_diff': graph_vs_eager}
                        if graph_ok else {'value': 'eager launches', 'e2e': 'eager launches'}),
        'batching_form': dict(
            legs, form=('one launch sequence per step over all 16384 samples: build, then the '
                        'absorption leg on a side stream beside the population leg, '
                        'captured as one CUDA graph'),
            two_stream_eager_ms=eager_ms, one_stream_eager_ms=one_stream_ms,
            graph_ms=graph_ms,
            block_k_real=[{'K': v[0], 'ms': v[1]} for v in block_k_real_timings().values()]),
        'fp64_ms_per_step': fp64_ms, 'speedup_fp32_vs_fp64': fp64_ms / ms,
        'roofline_fp64_form': {
            'kernel': 'plain FP64 step (complex propagator-form RK4 loops, ee {0} x {0} for {1} '
                      'steps and eg {2} x {2} for {3} steps, and their one-step propagators; '
                      'the whole step timed)'.format(m_ee, n_dyn, m_eg, n_abs),
            'bound': 'fp64_fma', 'achieved': fp64_achieved, 'peak': peak64, 'unit': 'TFLOP/s',
            'frac': fp64_achieved / peak64 if peak64 else None, 'flops_per_step': fp64_flops,
            'peak_source': 'measured live by the FMA probe (libqsx_probe.so, FP64 FMA)'},
        'e2e': {'value': whole_job_rate(world, e2e_ms), 'unit': UNIT,
                'h2d_bytes_per_step': int(off_host.numel() * 8),
                'd2h_bytes_per_step': int((nf + Ph.size + 1) * 8)},
        'roofline': block_roofline(events, bb_flops, bb_ms, peak),
        'roofline_time_loop': {
            'kernel': '{} (ee populations, K={} step blocking, variant {})'.format(
                'rk4_hchain_f32<49> + rk4_hcontract_tc<49> + hblock_reduce_kernel (two-pass '
                'real loop: the state chain on the CUDA cores, the ensemble contraction as one '
                'long-K tcgen05 GEMM; times are the whole library call)'
                if events.get('dyn_variant') == 'real' else 'rk4_block_f32<49>',
                events['dyn_block_k'], events.get('dyn_variant')),
            'dense_step_equivalent_tflops': dense_equiv / (dyn_ms * 1e-3) / 1e12,
            'bound': 'fp32_fma', 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s',
            'frac': achieved / peak, 'flops_per_launch': flops_dyn, 'launch_ms': dyn_ms,
            'traffic': traffic, 'hbm': hbm_view(traffic, dyn_ms)},
        # the library's kernels per step of the timed FP32-build form: disordered
        # Hamiltonians, zero fill, two eigensolve kernels, operators, the eg
        # propagator, projection build, loop and reduction, DFT, Hermitian
        # propagator, tensor-core block build, chain, contraction, reduction
        # (the launch list of one step; torch adds five status-word kernels)
        'gpu_launches': LIB_KERNELS_PER_STEP * args.steps,
        'clocks': clocks,
    }
    if adj is not None:
        line['adjoint'] = adj
        line['adjoint_over_forward'] = adj['adjoint_over_forward']
    if third is not None:
        line['third_order_chain24'] = third
    if heom is not None:
        line['heom_ring8'] = heom
    if zofe is not None:
        line['zofe_fmo7'] = zofe
    if plain is not None:
        line['plain_fmo7'] = plain
    if base is not None:
        line['cpu_baseline'] = base
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.impl == 'reference':
        return reference_arm(args)
    if args.only_heom:
        args.only = 'heom'
    if args.only:
        import torch
        import qspectra_gb300 as qg
        from qspectra_gb300 import _native
        if args.only == 'heom':
            out = heom_ring8(torch, qg, _native, samples=args.heom_samples,
                             nsteps=args.heom_steps)
        elif args.only == 'zofe':
            out = zofe_fmo7(torch, qg, _native, samples=args.zofe_samples)
        elif args.only == 'plain':
            out = plain_fmo7(torch, qg)
        elif args.only == 'third':
            out = third_order_chain24(torch, qg, samples=args.third_samples,
                                      fp64_samples=args.third_fp64_samples,
                                      reps=args.third_reps, warm=args.third_reps > 1)
        else:
            out = adjoint_fmo7(torch, qg, samples=args.adjoint_samples,
                               adam_steps=args.adjoint_adam_steps,
                               checks=not args.no_adjoint_checks)
        print(json.dumps(out), flush=True)
        return 0
    return our_arm(args)


if __name__ == '__main__':
    sys.exit(main())
