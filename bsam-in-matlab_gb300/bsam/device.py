"""ctypes binding of ``libbsam_dev.so`` (the C-ABI of ``include/bsam_dev.h``).

``DeviceBackend`` is what the host drivers call for every numerical step of
the solve path: the ghost fills and prolongation of hierarchy set-up and
``ebSolveCycles``.  A hierarchy is uploaded once per structural change
(``H.version``) and stays resident; after each call the solution, coarse
shadows and working force are read back into ``H`` so the host keeps the
reference's value semantics (``H = ebSolveCycles(H)``).

There is no fallback: if the library cannot be built or loaded, or no
sm_103 device is present, the calls raise ``DeviceError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
import time

import numpy as np

from .build import build_dev
from .flat import flatten, scatter_field, gather_field, FIELD_Q, FIELD_F, FIELD_QC

P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double

BSAM_FIELD_Q, BSAM_FIELD_F, BSAM_FIELD_FTRUE, BSAM_FIELD_QC, BSAM_FIELD_CC, BSAM_FIELD_INVDIAG = range(6)
(BSAM_FIELD_DEW, BSAM_FIELD_DNS, BSAM_FIELD_PCOEF, BSAM_FIELD_CFD, BSAM_FIELD_BCG, BSAM_FIELD_AINV,
 BSAM_FIELD_BCRHS, BSAM_FIELD_UO, BSAM_FIELD_UOO) = range(6, 15)
# coefficient arrays of the flat tables replaced by an incremental upload
COEF_FIELDS = (('DeW', BSAM_FIELD_DEW), ('DnS', BSAM_FIELD_DNS), ('CC', BSAM_FIELD_CC),
               ('InvDiagS', BSAM_FIELD_INVDIAG), ('pcoef', BSAM_FIELD_PCOEF), ('cfd', BSAM_FIELD_CFD),
               ('bcg', BSAM_FIELD_BCG), ('Ainv', BSAM_FIELD_AINV), ('bcRhs', BSAM_FIELD_BCRHS))
NKINDS = 9
KIND_NAMES = ['relax', 'ghost', 'restrict', 'ring', 'coarse_load', 'corrections', 'prolong', 'coarsest', 'residual']
ERRNAMES = {1: 'arg', 2: 'cuda', 3: 'nomem', 4: 'state', 5: 'nodev'}


class DeviceError(RuntimeError):
    """A C-ABI call failed; ``ident`` mirrors the MEX error id bsam:device:<code>."""

    def __init__(self, code, msg):
        self.code = code
        self.ident = f'bsam:device:{ERRNAMES.get(code, code)}'
        super().__init__(f'{self.ident}: {msg}')


class HierDesc(C.Structure):
    _fields_ = [('nlev', I32), ('root_idx', I32), ('npatch', I32),
                ('levels', P), ('hs', P), ('patches', P),
                ('Q', P), ('F', P), ('FTrue', P), ('QC', P), ('CC', P), ('InvDiagS', P), ('DeW', P), ('DnS', P),
                ('bcg', P), ('cfd', P), ('pcoef', P), ('covered', P),
                ('same', P), ('ring', P), ('win', P), ('fp', P), ('corr', P),
                ('Ainv', P), ('bcRhs', P),
                ('n_q', I64), ('n_cells', I64), ('n_dew', I64), ('n_dns', I64), ('n_qc', I64), ('n_bcg', I64),
                ('n_cfd', I64), ('n_pcoef', I64), ('n_same', I64), ('n_ring', I64), ('n_win', I64), ('n_fp', I64),
                ('n_corr', I64),
                ('ncoarse', I32), ('singular', I32),
                ('ninst', I32), ('patch_inst', P), ('inst_root', P)]


class SolveOpts(C.Structure):
    _fields_ = [('npre', I32), ('npost', I32), ('omega', D), ('ghost_interp', I32), ('mass_correction', I32),
                ('max_vcycles', I32), ('rel_tol', D), ('precision', I32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_dev()
        L = C.CDLL(path)
        L.bsam_last_error.restype = C.c_char_p
        L.bsam_ctx_create.argtypes = [C.c_int, C.POINTER(P)]
        L.bsam_ctx_destroy.argtypes = [P]
        L.bsam_hier_upload.argtypes = [P, C.POINTER(HierDesc), C.POINTER(SolveOpts), C.POINTER(P)]
        L.bsam_hier_free.argtypes = [P]
        L.bsam_set_opts.argtypes = [P, C.POINTER(SolveOpts)]
        L.bsam_set_field.argtypes = [P, C.c_int, P, I64]
        L.bsam_get_field.argtypes = [P, C.c_int, P, I64]
        L.bsam_fill_ghosts.argtypes = [P, C.c_int]
        L.bsam_prolong_level.argtypes = [P, C.c_int]
        L.bsam_solve_cycles.argtypes = [P, P, C.c_int, C.POINTER(C.c_int), C.POINTER(D), C.POINTER(I64)]
        L.bsam_vcycle.argtypes = [P]
        L.bsam_filldown.argtypes = [P]
        L.bsam_comp_residual.argtypes = [P, P]
        L.bsam_composite_mean.argtypes = [P, C.POINTER(D), C.POINTER(D)]
        L.bsam_mass_check.argtypes = [P, P]
        L.bsam_stream.argtypes = [P, C.POINTER(P)]
        L.bsam_profile_vcycles.argtypes = [P, C.c_int, C.c_int, P, P, P]
        L.bsam_time_relax.argtypes = [P, C.c_int, C.c_int, C.POINTER(D)]
        L.bsam_kernels_per_vcycle.argtypes = [P, C.POINTER(I64)]
        L.bsam_save_state.argtypes = [P]
        L.bsam_restore_state.argtypes = [P]
        L.bsam_launch_count.argtypes = [P, C.POINTER(I64)]
        L.bsam_relax_tuning.argtypes = [P, C.c_int, P, C.c_int]
        L.bsam_batch_result.argtypes = [P, C.c_int, P, C.c_int, C.POINTER(C.c_int), C.POINTER(D), C.POINTER(I64)]
        L.bsam_batch_set_stop.argtypes = [P, C.c_int, C.c_int, D]
        L.bsam_polygon_dist2.argtypes = [P, P, C.c_int, P, P, P, I64]
        L.bsam_device_memory.argtypes = [C.c_int, C.POINTER(I64), C.POINTER(I64)]
        L.bsam_fp64_rate.argtypes = [P, C.POINTER(D)]
        L.bsam_setup_levels.argtypes = [P]
        L.bsam_parabolic_rhs.argtypes = [P, C.c_int, D, P, I64]
        L.bsam_history_push.argtypes = [P]
        L.bsam_history_transfer.argtypes = [P, P, P, I64, C.c_int]
        L.bsam_tag_level.argtypes = [P, C.c_int, C.c_int, D, C.c_int, C.c_int, C.c_int, P]
        _lib = L
    return _lib


_trace_path = os.environ.get('BSAM_TRACE')


def trace(event, **fields):
    """Append one JSON line per event to the file named by BSAM_TRACE (per
    solve: V-cycles, residual history, final rel, wall ms)."""
    if not _trace_path:
        return
    import json
    rec = {'event': event, 'time': time.time()}
    rec.update(fields)
    with open(_trace_path, 'a') as f:
        f.write(json.dumps(rec) + '\n')


def check(rc):
    if rc != 0:
        raise DeviceError(rc, lib().bsam_last_error().decode(errors='replace'))


def solve_opts(opts):
    return SolveOpts(int(opts['NPre']), int(opts['NPost']), float(opts['Omega']),
                     0 if str(opts['GhostInterp']).lower() == 'qif' else 1, int(bool(opts['MassCorrection'])),
                     int(opts['MaxVCycles']), float(opts['RelTol']),
                     1 if str(opts.get('Precision', 'fp64')).lower() == 'mixed' else 0)


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def make_desc(fl, keep):
    """Fill a HierDesc from a Flat (``keep`` collects arrays to hold alive)."""
    def arr(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return _ptr(a)
    d = HierDesc()
    d.nlev, d.root_idx, d.npatch = fl.nlev, fl.rootIdx, fl.npatch
    d.levels, d.hs, d.patches = arr(fl.levels, np.int32), arr(fl.hs, np.float64), arr(fl.patches, np.int32)
    for name in ('Q', 'F', 'FTrue', 'QC', 'CC', 'InvDiagS', 'DeW', 'DnS', 'bcg', 'cfd', 'pcoef'):
        setattr(d, name, arr(getattr(fl, name), np.float64))
    d.covered = arr(fl.covered, np.uint8)
    for name in ('same', 'ring', 'win', 'fp', 'corr'):
        setattr(d, name, arr(getattr(fl, name), np.int32))
    d.Ainv, d.bcRhs = arr(fl.Ainv, np.float64), arr(fl.bcRhs, np.float64)
    d.n_q, d.n_cells, d.n_dew, d.n_dns = fl.Q.size, fl.F.size, fl.DeW.size, fl.DnS.size
    d.n_qc, d.n_bcg, d.n_cfd, d.n_pcoef = fl.QC.size, fl.bcg.size, fl.cfd.size, fl.pcoef.size
    d.n_same, d.n_ring, d.n_win = fl.same.shape[0], fl.ring.shape[0], fl.win.size
    d.n_fp, d.n_corr = fl.fp.shape[0], fl.corr.size
    d.ncoarse, d.singular = int(fl.bcRhs.size), int(fl.singular)
    ninst = int(getattr(fl, 'ninst', 1))
    d.ninst = ninst
    if ninst > 1:
        d.patch_inst, d.inst_root = arr(fl.patch_inst, np.int32), arr(fl.inst_root, np.int32)
    return d


class Context:
    def __init__(self, device=0):
        self.device = device
        h = P()
        check(lib().bsam_ctx_create(int(device), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            lib().bsam_ctx_destroy(self.h)
        except Exception:
            pass

    def __copy__(self):
        raise TypeError('bsam_device:copy: a device context cannot be copied')

    __deepcopy__ = lambda self, memo: self.__copy__()


class DevHier:
    """One uploaded hierarchy (device-resident)."""

    def __init__(self, ctx, fl, opts):
        self.ctx = ctx
        self.fl = fl
        keep = []
        desc = make_desc(fl, keep)
        self.opts = solve_opts(opts)
        h = P()
        check(lib().bsam_hier_upload(ctx.h, C.byref(desc), C.byref(self.opts), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            lib().bsam_hier_free(self.h)
        except Exception:
            pass

    def __copy__(self):
        raise TypeError('bsam_device:copy: an uploaded hierarchy cannot be copied (its handle would be freed twice)')

    __deepcopy__ = lambda self, memo: self.__copy__()

    def set_opts(self, opts):
        self.opts = solve_opts(opts)
        check(lib().bsam_set_opts(self.h, C.byref(self.opts)))

    def get(self, which, n):
        out = np.empty(n)
        check(lib().bsam_get_field(self.h, which, _ptr(out), n))
        return out

    def set(self, which, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        check(lib().bsam_set_field(self.h, which, _ptr(arr), arr.size))

    def fill(self, k):
        check(lib().bsam_fill_ghosts(self.h, int(k)))

    def prolong(self, k):
        check(lib().bsam_prolong_level(self.h, int(k)))

    def solve_cycles(self, hist_cap):
        hist = np.zeros(max(hist_cap, 1))
        it = C.c_int(0)
        rel = D(0)
        vis = I64(0)
        t0 = time.perf_counter()
        check(lib().bsam_solve_cycles(self.h, _ptr(hist), hist.size, C.byref(it), C.byref(rel), C.byref(vis)))
        out = it.value, hist[:it.value + 1].copy(), rel.value, vis.value
        trace('solve_cycles', ms=1e3 * (time.perf_counter() - t0), vcycles=out[0], resHist=out[1].tolist(),
              finalRel=out[2], visibleCells=out[3], ninst=int(getattr(self.fl, 'ninst', 1)))
        return out

    def checkpoint(self):
        """Host snapshot of the solution state (Q, QC, F, FTrue and the
        parabolic history when present), for a resume on a fresh upload."""
        fl = self.fl
        cp = {'Q': self.get(BSAM_FIELD_Q, fl.Q.size), 'QC': self.get(BSAM_FIELD_QC, fl.QC.size),
              'F': self.get(BSAM_FIELD_F, fl.F.size), 'FTrue': self.get(BSAM_FIELD_FTRUE, fl.F.size)}
        for name, which in (('Uo', BSAM_FIELD_UO), ('Uoo', BSAM_FIELD_UOO)):
            cp[name] = self.get(which, fl.F.size)
        return cp

    def resume(self, cp):
        """Load a checkpoint of the same hierarchy (same flat tables)."""
        for name, which in (('Q', BSAM_FIELD_Q), ('QC', BSAM_FIELD_QC), ('F', BSAM_FIELD_F),
                            ('FTrue', BSAM_FIELD_FTRUE), ('Uo', BSAM_FIELD_UO), ('Uoo', BSAM_FIELD_UOO)):
            if name in cp:
                self.set(which, cp[name])

    def batch_result(self, inst, hist_cap):
        """(vcycles, resHist, finalRel, visibleCells) of one instance of a
        batch after solve_cycles."""
        hist = np.zeros(max(hist_cap, 1))
        it = C.c_int(0)
        rel = D(0)
        vis = I64(0)
        check(lib().bsam_batch_result(self.h, int(inst), _ptr(hist), hist.size, C.byref(it), C.byref(rel),
                                      C.byref(vis)))
        return it.value, hist[:it.value + 1].copy(), rel.value, vis.value

    def set_stop(self, inst, max_vcycles, rel_tol):
        check(lib().bsam_batch_set_stop(self.h, int(inst), int(max_vcycles), float(rel_tol)))

    def parabolic_rhs(self, scheme, dt, f=None):
        """FTrue of a BE (0) / BDF2 (1) step from the resident history."""
        if f is not None:
            f = np.ascontiguousarray(f, dtype=np.float64)
        check(lib().bsam_parabolic_rhs(self.h, int(scheme), float(dt), _ptr(f), 0 if f is None else f.size))

    def history_transfer(self, old, src_old, has_uoo):
        """BDF2 history from the hierarchy `old` (a DevHier on the same
        device) after a regrid; see bsam_history_transfer."""
        src = np.ascontiguousarray(src_old, dtype=np.int32)
        check(lib().bsam_history_transfer(self.h, old.h, src.ctypes.data, src.size, int(bool(has_uoo))))

    def history_push(self):
        check(lib().bsam_history_push(self.h))

    def tag_level(self, level, indicator, threshold, buffer, n0, n1):
        """Buffered, cover-limited tag mask of a level, shape (n0, n1)."""
        out = np.zeros(int(n0) * int(n1), dtype=np.uint8)
        check(lib().bsam_tag_level(self.h, int(level), {'ulap': 0, 'rte': 1}[indicator], float(threshold),
                                   int(buffer), int(n0), int(n1), _ptr(out)))
        return out.reshape(int(n0), int(n1)).astype(bool)

    def setup_levels(self):
        """Run the deferred set-up steps (new-level prolongations, fills)."""
        check(lib().bsam_setup_levels(self.h))

    def vcycle(self):
        check(lib().bsam_vcycle(self.h))

    def filldown(self):
        check(lib().bsam_filldown(self.h))

    def residual(self):
        out = np.zeros(5)
        check(lib().bsam_comp_residual(self.h, _ptr(out)))
        return {'linf': out[0], 'l2': out[1], 'fnorm': out[2], 'rel': out[3], 'ncell': int(out[4])}

    def mass_check(self):
        out = np.zeros(4)
        check(lib().bsam_mass_check(self.h, _ptr(out)))
        return {'lhs': out[0], 'flux': out[1], 'defect': out[2], 'rel': out[3]}

    def composite_mean(self):
        m, a = D(0), D(0)
        check(lib().bsam_composite_mean(self.h, C.byref(m), C.byref(a)))
        return m.value, a.value

    def stream(self):
        s = P()
        check(lib().bsam_stream(self.h, C.byref(s)))
        return s.value

    def profile(self, ncycles, level=0):
        ms = np.zeros(NKINDS)
        nl = np.zeros(NKINDS, dtype=np.int64)
        by = np.zeros(NKINDS)
        check(lib().bsam_profile_vcycles(self.h, int(ncycles), int(level), _ptr(ms), _ptr(nl), _ptr(by)))
        return {KIND_NAMES[i]: {'ms': ms[i], 'launches': int(nl[i]), 'bytes': by[i]} for i in range(NKINDS)}

    def time_relax(self, level, reps=20):
        """Microseconds per colour pass of `level`'s smoother, replayed as a
        graph of chained launches (bsam_time_relax)."""
        us = D(0)
        check(lib().bsam_time_relax(self.h, int(level), int(reps), C.byref(us)))
        return us.value

    def save_state(self):
        check(lib().bsam_save_state(self.h))

    def restore_state(self):
        check(lib().bsam_restore_state(self.h))

    def launch_count(self):
        n = I64(0)
        check(lib().bsam_launch_count(self.h, C.byref(n)))
        return n.value

    def relax_tuning(self, precision=0):
        """Smoother launch form per level 1..nlev as tuned: colour cells per
        thread (1, 2, 4), 3 persistent blocks, 0 the single-cluster launch, 5
        the single-cluster launch with the level's solution in distributed
        shared memory, -1 not yet run."""
        out = np.zeros(int(self.fl.nlev), np.int32)
        check(lib().bsam_relax_tuning(self.h, int(precision), out.ctypes.data, out.size))
        return out

    def kernels_per_vcycle(self):
        n = I64(0)
        check(lib().bsam_kernels_per_vcycle(self.h, C.byref(n)))
        return n.value


def memory_info(device=0):
    """(free, total) device memory in bytes."""
    f, t = I64(0), I64(0)
    check(lib().bsam_device_memory(int(device), C.byref(f), C.byref(t)))
    return f.value, t.value


def fp64_rate(ctx):
    """Measured FP64 multiply/add issue rate of the device, 1e9 ops/s."""
    g = D(0)
    check(lib().bsam_fp64_rate(ctx.h, C.byref(g)))
    return g.value


def polygon_dist2(ctx, verts, x, y, best):
    """best <- min(best, squared distance of (x, y) to the closed polygon
    verts [n, 2]), on the device (in place; float64 contiguous arrays)."""
    verts = np.ascontiguousarray(verts, dtype=np.float64)
    check(lib().bsam_polygon_dist2(ctx.h, _ptr(verts), int(verts.shape[0]), _ptr(x), _ptr(y), _ptr(best),
                                   int(best.size)))
    return best


class DeferredBackend:
    """Set-up backend of a host without a device: the set-up's device steps
    (ghost fills, new-level prolongations) are left to bsam_setup_levels on
    the uploaded hierarchy, which runs them in the same order."""

    name = 'deferred'

    def run(self, H, ops):
        for op in ops:
            if op[0] not in ('fill', 'prolong'):
                raise ValueError(f'bsam_device:deferred: set-up step {op[0]} cannot be deferred')

    def solve_cycles(self, H):
        raise RuntimeError('bsam_device:deferred: a deferred set-up has no solve; upload the hierarchy')


class DeviceBackend:
    """Backend of the host drivers: every numerical step runs on the GPU."""

    name = 'device'
    _instances = {}

    _lock = threading.RLock()

    @classmethod
    def get(cls, device=0):
        """The process-wide backend of a device (one context per device,
        created once even when several threads ask at the same time)."""
        with cls._lock:
            if device not in cls._instances:
                cls._instances[device] = cls(device)
            return cls._instances[device]

    # the parabolic driver keeps its state (solution, BDF2 history, source)
    # on the device between steps
    resident = True

    def __init__(self, device=0, ctx=None):
        self.ctx = ctx if ctx is not None else Context(device)

    @classmethod
    def on(cls, ctx):
        """A backend issuing its work on an existing context (stream)."""
        return cls(ctx.device, ctx)

    def ensure(self, H):
        """The resident copy of H: re-uploaded after a structural change,
        otherwise refreshed with the fields the host has modified ('coef':
        every coefficient array, an incremental upload with no new plan)."""
        cur = getattr(H, '_dev', None)
        if cur is not None and cur[0] == H.version and cur[1].ctx is self.ctx:
            dh = cur[1]
            dh.set_opts(H.opts)
            for name in sorted(H.dirty):
                if name == 'coef':
                    fl = flatten(H)
                    for attr, which in COEF_FIELDS:
                        dh.set(which, np.asarray(getattr(fl, attr), dtype=np.float64).ravel())
                    continue
                which = {'Q': BSAM_FIELD_Q, 'F': BSAM_FIELD_F, 'FTrue': BSAM_FIELD_FTRUE,
                         'QC': BSAM_FIELD_QC}[name]
                dh.set(which, gather_field(H, dh.fl, which))
            H.dirty.clear()
            return dh
        if getattr(H, 'host_stale', False):
            raise RuntimeError('bsam_device:stale: the host copy is older than the device state; sync_host first')
        fl = flatten(H)
        dh = DevHier(self.ctx, fl, H.opts)
        H._dev = (H.version, dh)
        H.dirty.clear()
        return dh

    def _writeback(self, H, dh):
        if H.par.get('resident') if isinstance(getattr(H, 'par', None), dict) else False:
            H.host_stale = True          # the state stays on the device
            return
        fl = dh.fl
        scatter_field(H, fl, FIELD_Q, dh.get(BSAM_FIELD_Q, fl.Q.size))
        scatter_field(H, fl, FIELD_QC, dh.get(BSAM_FIELD_QC, fl.QC.size))
        scatter_field(H, fl, FIELD_F, dh.get(BSAM_FIELD_F, fl.F.size))
        H.host_stale = False

    def sync_host(self, H):
        """Copy the device state of a resident hierarchy back to H."""
        if not getattr(H, 'host_stale', False):
            return
        dh = H._dev[1]
        fl = dh.fl
        scatter_field(H, fl, FIELD_Q, dh.get(BSAM_FIELD_Q, fl.Q.size))
        scatter_field(H, fl, FIELD_QC, dh.get(BSAM_FIELD_QC, fl.QC.size))
        scatter_field(H, fl, FIELD_F, dh.get(BSAM_FIELD_F, fl.F.size))
        scatter_field(H, fl, 2, dh.get(BSAM_FIELD_FTRUE, fl.F.size))
        H.host_stale = False

    # ---- parabolic steps on the resident hierarchy --------------------------
    def _cells(self, H, dh, arrays):
        """Flat cell array from per-patch arrays {(k, p): (mx, my)}."""
        from .flat import PD_COFF
        out = np.zeros(dh.fl.F.size)
        for (k, p), g in dh.fl.pglob.items():
            a = arrays.get((k, p))
            if a is None:
                continue
            o = int(dh.fl.patches[g][PD_COFF])
            out[o:o + a.size] = np.asarray(a, dtype=np.float64).ravel(order='F')
        return out

    def parabolic_rhs(self, H, scheme, dt, f_patches=None):
        dh = self.ensure(H)
        f = None if f_patches is None else self._cells(H, dh, f_patches)
        dh.parabolic_rhs({'be': 0, 'bdf2': 1}[scheme], dt, f)

    def history_push(self, H):
        self.ensure(H).history_push()

    def tag_mask(self, H, indicator, threshold, buffer):
        """ebTagCluster's tag mask of the finest level computed on the device."""
        dh = self.ensure(H)
        n = H.lev[H.nlev].n
        return dh.tag_level(H.nlev, indicator, threshold, buffer, n[0], n[1])

    # history downloads so far (a regrid on the device makes none)
    history_downloads = 0

    def history_get(self, H):
        """(Uo, Uoo) as per-patch arrays {(k, p): (mx, my)}."""
        from .flat import PD_COFF, PD_MX, PD_MY
        dh = self.ensure(H)
        DeviceBackend.history_downloads += 1
        out = []
        for which in (BSAM_FIELD_UO, BSAM_FIELD_UOO):
            v = dh.get(which, dh.fl.F.size)
            d = {}
            for (k, p), g in dh.fl.pglob.items():
                r = dh.fl.patches[g]
                mx, my, o = int(r[PD_MX]), int(r[PD_MY]), int(r[PD_COFF])
                d[(k, p)] = v[o:o + mx * my].reshape((mx, my), order='F').copy(order='F')
            out.append(d)
        return out[0], out[1]

    def history_transfer(self, Hn, Hold, has_uoo):
        """ebpRegrid's history transfer from Hold's resident state to Hn's,
        on the device (Hn uploaded here; Hold's copy must be current)."""
        from .parabolic import history_sources
        cur = getattr(Hold, '_dev', None)
        if cur is None or cur[0] != Hold.version:
            raise RuntimeError('bsam_device:state: the old hierarchy is not resident')
        dn = self.ensure(Hn)
        dn.history_transfer(cur[1], history_sources(Hn, dn.fl, Hold, cur[1].fl), has_uoo)

    def history_set(self, H, Uo, Uoo):
        dh = self.ensure(H)
        dh.set(BSAM_FIELD_UO, self._cells(H, dh, Uo))
        dh.set(BSAM_FIELD_UOO, self._cells(H, dh, Uoo or {}))

    def run(self, H, ops):
        dh = self.ensure(H)
        for op in ops:
            if op[0] == 'fill':
                dh.fill(op[1])
            elif op[0] == 'prolong':
                dh.prolong(op[1])
            elif op[0] == 'filldown':
                dh.filldown()
            else:
                raise ValueError(op)
        self._writeback(H, dh)

    def solve_cycles(self, H):
        dh = self.ensure(H)
        out = dh.solve_cycles(int(H.opts.MaxVCycles) + 2)
        self._writeback(H, dh)
        return out

    def residual(self, H):
        dh = self.ensure(H)
        res = dh.residual()
        self._writeback(H, dh)
        return res

    def mass_check(self, H):
        return self.ensure(H).mass_check()

    def composite_mean(self, H):
        return self.ensure(H).composite_mean()
