"""Build the in-tree CUDA library ``qspectra_gb300/_lib/libqsx.so`` for sm_103a.

Plain nvcc, one object per translation unit compiled in parallel, then one
shared library with the CUDA runtime linked statically.  Usage:

    python -m qspectra_gb300.build          # or qspectra_gb300.build.build()
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT_DIR = os.path.join(HERE, '_lib')
LIB = os.path.join(OUT_DIR, 'libqsx.so')
# the FMA-throughput probe the benchmark uses for its CUDA-core roofline
# denominators: a separate library, not part of libqsx.so or include/qsx.h
PROBE_SRC = os.path.join(CSRC, 'probe', 'fma_probe.cu')
PROBE_LIB = os.path.join(OUT_DIR, 'libqsx_probe.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC',
         '--expt-relaxed-constexpr']


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None and os.path.exists('/usr/local/cuda/bin/nvcc'):
        exe = '/usr/local/cuda/bin/nvcc'
    if exe is None:
        raise RuntimeError('nvcc not found; the qsx CUDA library cannot be built')
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith('.cu'))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile every .cu under csrc/ and link libqsx.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith('.cuh')]
    headers.append(os.path.join(os.path.dirname(HERE), 'include', 'qsx.h'))
    srcs = sources()
    objs = [os.path.join(OUT_DIR, os.path.basename(s)[:-3] + '.o') for s in srcs]
    exe = nvcc()

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + headers):
            return obj
        cmd = [exe] + ARCH + FLAGS + ['-c', src, '-o', obj]
        if verbose:
            print(' '.join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on {}:\n{}'.format(src, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    if force or _stale(LIB, objs):
        cmd = [exe] + ARCH + ['-shared', '-cudart', 'static', '-o', LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n' + r.stderr)
    if force or _stale(PROBE_LIB, [PROBE_SRC]):
        cmd = [exe] + ARCH + FLAGS + ['-shared', '-cudart', 'static', PROBE_SRC,
                                      '-o', PROBE_LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on {}:\n{}'.format(PROBE_SRC, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build(verbose=True, force='--force' in sys.argv))
