"""Build libphk.so (the sm_103a kernels behind the C ABI) in the source tree.

    python -m pyheadtail_gb300._build

compiles every ``csrc/*.cu`` translation unit in parallel with one
``-gencode arch=compute_103a,code=sm_103a`` and links the shared library
next to this file.  Objects go to ``_build/`` (git-ignored).  A rebuild is
skipped when the library is newer than every source and header.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libphk.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-O2', '--expt-relaxed-constexpr',
              '-I' + INCLUDE, '-I' + CSRC]


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'),
                 '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: set NVCC or put CUDA 13 on PATH')


def sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = (sources() + glob.glob(os.path.join(CSRC, '*.h')) +
            glob.glob(os.path.join(CSRC, '*.cuh')) +
            glob.glob(os.path.join(INCLUDE, '*.h')) + [__file__])
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ['-c', src, '-o', obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' %
                           (src, ' '.join(cmd), p.stderr[-4000:]))
    return obj, p.stderr


def build(force=False, verbose=False, extra=()):
    """Compile and link libphk.so; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + '.tmp'
    cmd = [nvcc()] + ARCH + ['-shared', '-o', tmp] + objs
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (' '.join(cmd), p.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True,
                extra=['-Xptxas', '-v'] if '--ptxas' in sys.argv else []))
