"""In-tree build of the package's native libraries.

``libbsam_dev.so``  CUDA kernels + C-ABI (nvcc, sm_103a only)
``libbsam_host.so`` host set-up helpers (gcc)

Both land in ``bsam-in-matlab_gb300/lib/`` and are rebuilt when a source is
newer than the library.
"""
from __future__ import annotations

import os
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, 'csrc')
LIBDIR = os.path.join(PKG, 'lib')
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, 'include')

HOST_LIB = os.path.join(LIBDIR, 'libbsam_host.so')
DEV_LIB = os.path.join(LIBDIR, 'libbsam_dev.so')

DEV_SOURCES = ['bsam_dev.cu', 'bsam_noalloc.cu', 'bsam_geom.cu']
NVCC_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-lineinfo', '-std=c++17',
              '--fmad=false', '-Xcompiler', '-fPIC,-ffp-contract=off']
# per-source extra flags (none at present)
SOURCE_FLAGS = {}


def _stale(lib, srcs):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_host(force=False):
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(CSRC, 'bsam_host.c')
    if force or _stale(HOST_LIB, [src]):
        subprocess.check_call(['gcc', '-O3', '-ffp-contract=off', '-fno-fast-math', '-fPIC', '-shared',
                               '-pthread', '-o', HOST_LIB, src, '-lm'])
    return HOST_LIB


def build_dev(force=False, verbose=False):
    """Compiles every CUDA source to an object (in parallel, each with its own
    flags) and links the shared library."""
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in DEV_SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if force or _stale(DEV_LIB, deps):
        objdir = os.path.join(LIBDIR, 'obj')
        os.makedirs(objdir, exist_ok=True)
        procs, objs = [], []
        for name, src in zip(DEV_SOURCES, srcs):
            obj = os.path.join(objdir, name.replace('.cu', '.o'))
            cmd = ['nvcc'] + NVCC_FLAGS + SOURCE_FLAGS.get(name, []) + ['-I', INCLUDE, '-c', '-o', obj, src]
            if verbose:
                cmd.insert(1, '-Xptxas=-v')
            procs.append((cmd, subprocess.Popen(cmd)))
            objs.append(obj)
        for cmd, p in procs:
            if p.wait() != 0:
                raise subprocess.CalledProcessError(p.returncode, cmd)
        subprocess.check_call(['nvcc', '-gencode', 'arch=compute_103a,code=sm_103a', '-shared', '-o', DEV_LIB] + objs)
    return DEV_LIB


def build_all(force=False):
    build_host(force)
    build_dev(force)
