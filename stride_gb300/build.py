"""Builds libstrideacc.so (the CUDA kernels and the C ABI) for sm_103a with nvcc.

Every translation unit compiles in parallel to an object file under ``stride_gb300/_build``
and the objects link into one shared library with the CUDA runtime linked statically, so
the library needs nothing but the driver at run time.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, '_build')
LIB = os.path.join(OUT, 'libstrideacc.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']


def nvcc():
    path = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(path):
        raise RuntimeError('nvcc not found: the CUDA extension cannot be built')
    return path


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + '.o')
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    deps.append(os.path.join(HERE, '..', 'include', 'strideacc.h'))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + extra + ['-c', src, '-o', obj]
    subprocess.run(cmd, check=True)
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart_static', '-lrt', '-ldl', '-lpthread']
        subprocess.run(cmd, check=True)
    if verbose:
        print(LIB)
    return LIB


if __name__ == '__main__':
    build(verbose=True, extra=sys.argv[1:])
