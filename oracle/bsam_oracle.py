"""ctypes loader for the C oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the parity checker for the CUDA solve path: a CPU restatement
of the reference's MATLAB hot path (``bsam_oracle.c``).  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module; the product path never does.

``OracleBackend`` has the same interface as ``bsam.device.DeviceBackend``
(``run`` for set-up operations, ``solve_cycles`` for ``ebSolveCycles``) so
the reference's own driver sequence (``ebSolve``: setup, tag, add level,
solve) can be replayed on the CPU and compared with the device.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, '_build', 'liboracle.so')


def build(force=False):
    """Compile the oracle (gcc, no FMA contraction, OpenMP over patches)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    src = os.path.join(HERE, 'bsam_oracle.c')
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ['gcc', '-O2', '-ffp-contract=off', '-fno-fast-math', '-fopenmp', '-fPIC', '-shared',
           '-o', LIB, src, '-lm']
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.oracle_new.restype = P
        L.oracle_new.argtypes = [C.c_int, C.c_int, C.c_int] + [P] * 22 + [C.c_int] * 3 + [C.c_double] + \
                                [C.c_int] * 3 + [C.c_double]
        L.oracle_free.argtypes = [P]
        for name in ('oracle_fill_ghosts', 'oracle_restrict', 'oracle_ring'):
            getattr(L, name).argtypes = [P, C.c_int]
        L.oracle_correct.argtypes = [P, C.c_int, C.c_int]
        L.oracle_coarse_load.argtypes = [P, C.c_int]
        L.oracle_relax_level.argtypes = [P, C.c_int, C.c_int]
        L.oracle_vcycle.argtypes = [P, C.c_int]
        L.oracle_filldown.argtypes = [P]
        L.oracle_coarsest.argtypes = [P]
        L.oracle_residual.argtypes = [P, P]
        L.oracle_solve_cycles.restype = C.c_int
        L.oracle_solve_cycles.argtypes = [P, P, C.c_int, P, P]
        L.oracle_composite_mean.argtypes = [P, P, P]
        L.oracle_mass_check.argtypes = [P, P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


class OracleHier:
    """The flat arrays of one hierarchy, held alive for the C oracle."""

    def __init__(self, fl, opts):
        self.fl = fl
        self.keep = []
        L = lib()

        def P(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self.keep.append(a)
            return _ptr(a)

        self.Q = np.ascontiguousarray(fl.Q.copy())
        self.F = np.ascontiguousarray(fl.F.copy())
        self.FTrue = np.ascontiguousarray(fl.FTrue.copy())
        self.QC = np.ascontiguousarray(fl.QC.copy())
        self.h = L.oracle_new(
            fl.nlev, fl.rootIdx, fl.npatch, P(fl.levels, np.int32), P(fl.hs, np.float64),
            P(fl.patches, np.int32), _ptr(self.Q), _ptr(self.F), _ptr(self.FTrue), _ptr(self.QC),
            P(fl.CC, np.float64), P(fl.InvDiagS, np.float64), P(fl.DeW, np.float64), P(fl.DnS, np.float64),
            P(fl.bcg, np.float64), P(fl.cfd, np.float64), P(fl.pcoef, np.float64), P(fl.covered, np.uint8),
            P(fl.same, np.int32), P(fl.ring, np.int32), P(fl.win, np.int32), P(fl.fp, np.int32),
            P(fl.corr, np.int32), P(fl.Ainv, np.float64), P(fl.bcRhs, np.float64), int(fl.bcRhs.size),
            int(opts.NPre), int(opts.NPost), float(opts.Omega), int(opts.GhostInterp == 'qif'),
            int(bool(opts.MassCorrection)), int(opts.MaxVCycles), float(opts.RelTol))

    def __del__(self):
        try:
            lib().oracle_free(self.h)
        except Exception:
            pass

    def op(self, name, *args):
        getattr(lib(), 'oracle_' + name)(self.h, *args)

    def residual(self):
        out = np.zeros(5)
        lib().oracle_residual(self.h, _ptr(out))
        return {'linf': out[0], 'l2': out[1], 'fnorm': out[2], 'rel': out[3], 'ncell': int(out[4])}

    def solve_cycles(self, hist_cap=4096):
        hist = np.zeros(hist_cap)
        fr = np.zeros(1)
        vc = np.zeros(1, dtype=np.int64)
        it = lib().oracle_solve_cycles(self.h, _ptr(hist), hist_cap, _ptr(fr), _ptr(vc))
        return it, hist[:it + 1].copy(), float(fr[0]), int(vc[0])

    def mass_check(self):
        out = np.zeros(4)
        lib().oracle_mass_check(self.h, _ptr(out))
        return {'lhs': out[0], 'flux': out[1], 'defect': out[2], 'rel': out[3]}

    def composite_mean(self):
        m = np.zeros(1)
        a = np.zeros(1)
        lib().oracle_composite_mean(self.h, _ptr(m), _ptr(a))
        return float(m[0]), float(a[0])


class OracleBackend:
    """CPU execution of the hot path with the ``bsam.device`` backend API."""

    name = 'oracle'

    def _hier(self, H):
        from bsam.flat import flatten
        fl = flatten(H)
        return fl, OracleHier(fl, H.opts)

    def _writeback(self, H, fl, oh):
        H.dirty.clear()
        from bsam.flat import scatter_field, FIELD_Q, FIELD_QC, FIELD_F, FIELD_FTRUE
        scatter_field(H, fl, FIELD_Q, oh.Q)
        scatter_field(H, fl, FIELD_QC, oh.QC)
        scatter_field(H, fl, FIELD_F, oh.F)

    def run(self, H, ops):
        fl, oh = self._hier(H)
        for op in ops:
            if op[0] == 'fill':
                oh.op('fill_ghosts', op[1])
            elif op[0] == 'prolong':
                oh.op('correct', op[1], 0)
            elif op[0] == 'filldown':
                oh.op('filldown')
            else:
                raise ValueError(op)
        self._writeback(H, fl, oh)

    def solve_cycles(self, H):
        fl, oh = self._hier(H)
        it, hist, rel, vis = oh.solve_cycles(int(H.opts.MaxVCycles) + 2)
        self._writeback(H, fl, oh)
        return it, hist, rel, vis

    def residual(self, H):
        fl, oh = self._hier(H)
        res = oh.residual()
        self._writeback(H, fl, oh)
        return res

    def mass_check(self, H):
        fl, oh = self._hier(H)
        return oh.mass_check()

    def composite_mean(self, H):
        fl, oh = self._hier(H)
        return oh.composite_mean()
