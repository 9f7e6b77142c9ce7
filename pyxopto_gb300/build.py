"""In-tree build of libxopto_gb300.so for GB300 (sm_103a).

Every translation unit is compiled in parallel with nvcc (or g++ for plain
host C++) into ``pyxopto_gb300/_build/`` and linked into
``pyxopto_gb300/libxopto_gb300.so`` with the CUDA runtime linked statically.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libxopto_gb300.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_COMMON = ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                      '-Xcompiler', '-fno-strict-aliasing', '--expt-relaxed-constexpr']

# (source, extra flags); exact-math units must not contract a*b+c into FMA.
UNITS = [
    ('transport_exact_mcml_static.cu', ['-fmad=false']),
    ('transport_exact_mcml_dynamic.cu', ['-fmad=false']),
    ('transport_exact_mcvox_static.cu', ['-fmad=false']),
    ('transport_exact_mcvox_dynamic.cu', ['-fmad=false']),
    ('transport_fast_mcml_static.cu', ['-use_fast_math']),
    ('transport_fast_mcml_dynamic.cu', ['-use_fast_math']),
    ('transport_fast_mcvox_static.cu', ['-use_fast_math']),
    ('transport_fast_mcvox_dynamic.cu', ['-use_fast_math']),
    ('capi.cu', []),
    ('batched.cu', ['-use_fast_math']),
    ('batched_exact.cu', ['-fmad=false']),
    ('mlp.cu', []),
    ('noalloc.cu', []),
    ('sampling_volume.cu', ['-fmad=false']),
    ('voxel_radius.cu', []),
    ('rng_host.cpp', None),
]


def nvcc_path():
    for cand in (shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found; the CUDA 13 toolkit is required to build libxopto_gb300.so')


def _compile(nvcc, src, flags, verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + '.o')
    if flags is None:
        cmd = ['g++', '-O2', '-std=c++17', '-fPIC', '-c', path, '-o', obj]
    else:
        cmd = [nvcc] + NVCC_COMMON + flags + (['-Xptxas', '-v'] if verbose else []) + \
              ['-c', path, '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('compiling {} failed:\n{}\n{}'.format(src, ' '.join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose: bool = False, jobs: int = None) -> str:
    """Compile and link the library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    units = [(s, f) for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda u: _compile(nvcc, u[0], u[1], verbose), units))
    if verbose:
        for (src, _), (_, log) in zip(units, results):
            if log.strip():
                sys.stderr.write('--- {}\n{}\n'.format(src, log))
    objs = [o for o, _ in results]
    tmp = LIB + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lpthread']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('linking failed:\n{}\n{}'.format(' '.join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
