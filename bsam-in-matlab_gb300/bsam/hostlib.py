"""ctypes access to ``libbsam_host.so`` (set-up helpers, see csrc/bsam_host.c)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import build_host

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build_host())
        P, I64 = C.c_void_p, C.c_int64
        for fn in ('exp', 'tanh', 'cosh', 'sin', 'cos', 'sqrt'):
            getattr(L, 'bsam_v' + fn).argtypes = [P, P, I64]
        L.bsam_vatan2.argtypes = [P, P, P, I64]
        L.bsam_vhypot.argtypes = [P, P, P, I64]
        L.bsam_starfish_new.restype = P
        L.bsam_starfish_new.argtypes = [C.c_int] + [C.c_double] * 5
        L.bsam_starfish_free.argtypes = [P]
        L.bsam_starfish_nvert.restype = C.c_int
        L.bsam_starfish_nvert.argtypes = [P]
        L.bsam_starfish_vertices.argtypes = [P, P]
        L.bsam_starfish_distance.argtypes = [P, P, P, P, I64]
        L.bsam_starfish_distance_mt.argtypes = [P, P, P, P, I64, C.c_int]
        L.bsam_starfish_init_sign.argtypes = [P, P, P, P, P, I64]
        _lib = L
    return _lib


def host_threads():
    """Host threads for the set-up's point searches: ``BSAM_HOST_THREADS``
    if set (processes of a builder pool set 1), else the host's cores, at
    most 16."""
    v = os.environ.get('BSAM_HOST_THREADS')
    if v:
        return max(1, int(v))
    return max(1, min(16, os.cpu_count() or 1))


def _v1(name, x):
    x = np.asarray(x, dtype=np.float64)
    xc = np.ascontiguousarray(x.ravel(order='F'))
    y = np.empty_like(xc)
    getattr(lib(), 'bsam_v' + name)(xc.ctypes.data, y.ctypes.data, xc.size)
    return y.reshape(x.shape, order='F') if x.ndim else float(y[0])


def exp(x): return _v1('exp', x)
def tanh(x): return _v1('tanh', x)
def cosh(x): return _v1('cosh', x)
def sin(x): return _v1('sin', x)
def cos(x): return _v1('cos', x)


def _v2(name, a, b):
    a, b = np.broadcast_arrays(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64))
    ac = np.ascontiguousarray(a.ravel(order='F'))
    bc = np.ascontiguousarray(b.ravel(order='F'))
    y = np.empty_like(ac)
    getattr(lib(), 'bsam_v' + name)(ac.ctypes.data, bc.ctypes.data, y.ctypes.data, ac.size)
    return y.reshape(a.shape, order='F') if a.ndim else float(y[0])


def atan2(y, x): return _v2('atan2', y, x)
def hypot(x, y): return _v2('hypot', x, y)
