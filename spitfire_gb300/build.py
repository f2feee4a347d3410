"""Build the spitfire_gb300 CUDA library in-tree (spitfire_gb300/_build/libspitfire_gb300.so).

Every translation unit under csrc/ is compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``),
in parallel, then linked into one shared library that exports the C ABI of include/spitfire_gb300.h. nvcc
cross-compiles without a GPU, so this runs on the CPU build host as well as on the GPU machine (where it must run,
since binaries are architecture specific).
"""

import concurrent.futures
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, '_build')
LIB = os.path.join(OUT, 'libspitfire_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc():
    cand = os.environ.get('NVCC') or shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found (set NVCC or add CUDA to PATH)')
    return cand


def _flags(verbose_ptxas=False):
    f = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2', '--expt-relaxed-constexpr',
         '-I' + os.path.join(HERE, '..', 'include')] + ARCH
    if verbose_ptxas:
        f += ['-Xptxas', '-v']
    return f


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))


def _fingerprint():
    h = hashlib.sha256()
    for p in _sources() + sorted(glob.glob(os.path.join(CSRC, '*.h')) + glob.glob(os.path.join(CSRC, '*.cuh'))) + \
            [os.path.join(HERE, '..', 'include', 'spitfire_gb300.h')]:
        with open(p, 'rb') as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(' '.join(_flags()).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose_ptxas=False, jobs=None):
    """Compile if sources changed since the last build; return the library path."""
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, 'stamp')
    fp = _fingerprint()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    nv = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + '.o')
        cmd = [nv, '-c', src, '-o', obj] + _flags(verbose_ptxas)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed on {src}:\n{r.stdout}\n{r.stderr}')
        return obj, (r.stdout + r.stderr)

    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    logs = []
    for obj, log in results:
        objs.append(obj)
        if log.strip():
            logs.append(log)
    cmd = [nv, '-shared', '-o', LIB + '.tmp'] + objs + ARCH + ['-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'link failed:\n{r.stdout}\n{r.stderr}')
    os.replace(LIB + '.tmp', LIB)
    with open(stamp, 'w') as f:
        f.write(fp)
    if verbose_ptxas:
        sys.stdout.write('\n'.join(logs))
    return LIB


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose_ptxas='-v' in sys.argv)
    print(LIB)
