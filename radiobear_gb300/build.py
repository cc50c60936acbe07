"""Build the in-tree CUDA library ``radiobear_gb300/lib/librbgpu.so``.

nvcc compiles each translation unit for sm_103a only (one ``-gencode``),
in parallel, then links a shared object exporting the C ABI declared in
``include/radiobear_gb300.h``.  No cmake, no torch extension machinery.

    python -m radiobear_gb300.build          # build if sources changed
    python -m radiobear_gb300.build --force
"""
from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIBDIR = os.path.join(PKG, 'lib')
LIB = os.path.join(LIBDIR, 'librbgpu.so')
SOURCES = ['rb_alpha.cu', 'rb_raypath.cu', 'rb_tb.cu', 'rb_probe.cu', 'rb_noalloc.cu', 'rb_adjoint.cu',
           'rb_extra.cu', 'rb_atm.cu',
           'rb_api.cu']
HEADERS = ['rb_common.cuh', 'rb_args.cuh', 'rb_f32x2.cuh', 'rb_expint.cuh', 'rb_assemble.cuh']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
              '-Xptxas', '-v'] + ARCH
# Per-file flags.  The ray set-up and walk run their float64 set-up in two
# kernels (one ray per thread, or inside the walk's warp) and their float32
# steps from it: without implicit multiply-add contraction both compile to
# the same roundings (explicit fmaf calls stay fused).
FILE_FLAGS = {'rb_raypath.cu': ['-fmad=false']}


def nvcc_path():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build radiobear_gb300')


def _digest():
    h = hashlib.sha256()
    for name in SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), 'rb') as fp:
            h.update(fp.read())
    with open(os.path.join(ROOT, 'include', 'radiobear_gb300.h'), 'rb') as fp:
        h.update(fp.read())
    h.update(' '.join(NVCC_FLAGS).encode())
    h.update(repr(sorted(FILE_FLAGS.items())).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile (if needed) and return the path of the shared library."""
    stamp = os.path.join(LIBDIR, '.stamp')
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fp:
            if fp.read().strip() == dig:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = nvcc_path()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace('.cu', '.o'))
        cmd = [nvcc, '-c', os.path.join(CSRC, src), '-o', obj] + NVCC_FLAGS + FILE_FLAGS.get(src, [])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for {}:\n{}\n{}'.format(src, r.stdout, r.stderr))
        return obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for (_, log), src in zip(results, SOURCES):
            print('==', src)
            print(log)
    tmp = LIB + '.tmp'
    cmd = [nvcc, '-shared', '-o', tmp] + objs + ARCH + ['-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n{}\n{}'.format(r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, 'w') as fp:
        fp.write(dig)
    return LIB


if __name__ == '__main__':
    path = build(force='--force' in sys.argv, verbose='-v' in sys.argv or '--force' in sys.argv)
    print(path)
