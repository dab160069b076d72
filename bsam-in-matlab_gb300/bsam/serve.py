"""Request serving: a continuous-batching loop over independent solves.

Requests (diffuse-domain star problems, or any elliptic problem given as a
builder spec) arrive at any time.  Each one goes through two stages:

  build  host set-up in a pool of worker processes (spawned, without a CUDA
         context: geometry, coefficients, tagging and clustering, the
         hierarchy and its flat upload tables -- the reference's ebSetup /
         ebAddLevel / ddTransmissionProblem path; the polygon distances of
         their sample points go to the server's DistanceService, which runs
         them on the GPU); the set-up's device steps
         (ghost fills, new-level prolongations) are deferred to the wave,
         which runs them on the merged upload (bsam_setup_levels) -- many
         processes issuing small synchronous GPU calls would time-slice one
         GPU between their contexts;
  solve  ebSolveCycles on the GPU, in waves: the dispatcher merges ready
         requests that share a level ladder and solve options into one batch
         (bsam.batch), admitted while their device footprint fits the memory
         budget, and runs each wave on its own stream; a request that becomes
         ready while waves run is admitted into the next wave as soon as a
         wave slot and memory are free, so its work overlaps the running
         waves on the device.

A parabolic request (a time-stepping run, ebpSolve) is not merged: it holds
one wave slot for its whole run, its hierarchy, coefficients and BDF2
history resident on that slot's stream across steps and regrids, while
other waves run beside it.

Every instance of a wave keeps its own stop test and is frozen once it has
converged, so a request's result is the same alone and in any mix.
Latency is measured from submission to the solved result on the host.
"""
from __future__ import annotations

import concurrent.futures as cf
import multiprocessing as mp
import os
import threading
import time
from collections import deque

import numpy as np

STAR_BOX = [-2.0, 2.0, -2.0, 2.0]
STAR_DATA = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'g': 4}


def star_request(seed, precision='mixed'):
    """One request of the served diffuse-domain stream: a star interface
    r(theta) = a0 (1 + b sin(k theta + theta0)) with k in {3..7}, b ~ U[0.3,
    0.8], a0 ~ U[0.8, 1.2], theta0 ~ U[0, 2 pi), eps ~ U[0.02, 0.08], base
    64^2, MaxLevels ~ U{3, 4, 5}; draws with a0 (1 + b) > 1.9 (interface
    leaving [-2, 2]^2) are redrawn.  Seeded with numpy's PCG64."""
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    while True:
        k = int(rng.integers(3, 8))
        b = float(rng.uniform(0.3, 0.8))
        a0 = float(rng.uniform(0.8, 1.2))
        th0 = float(rng.uniform(0.0, 2 * np.pi))
        eps = float(rng.uniform(0.02, 0.08))
        ml = int(rng.integers(3, 6))
        if a0 * (1 + b) <= 1.9:
            break
    return {'kind': 'dd_star', 'seed': int(seed), 'k': k, 'b': b, 'a0': a0, 'th0': th0, 'eps': eps,
            'MaxLevels': ml, 'Precision': precision}


def heat_request(seed, precision='fp64'):
    """A served parabolic request: BDF2 heat diffusion on [0,1]^2 (D = 1,
    C = 0, f = 0, homogeneous Neumann) from u0 = 1 + a cos(2 pi kx x)
    cos(2 pi ky y), a ~ U[0.1, 0.3], kx, ky in {1, 2}, Dt 0.002, TFinal
    0.02, RegridEvery 5, BaseCells 32, MaxLevels 3 -- the README heat
    example's recipe, seeded."""
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    return {'kind': 'parabolic', 'seed': int(seed), 'a': float(rng.uniform(0.1, 0.3)),
            'kx': int(rng.integers(1, 3)), 'ky': int(rng.integers(1, 3)), 'Dt': 0.002, 'TFinal': 0.02,
            'RegridEvery': 5, 'BaseCells': 32, 'MaxLevels': 3, 'Precision': precision}


def run_parabolic(spec, backend):
    """One parabolic request on a device backend (its own stream)."""
    from .parabolic import ebpProblem, ebpSolve
    a, kx, ky = spec['a'], spec['kx'], spec['ky']
    u0 = lambda x, y: 1 + a * np.cos(2 * np.pi * kx * x) * np.cos(2 * np.pi * ky * y)
    prob = ebpProblem([0, 1, 0, 1], 1, 0, 0, ('neumann', 0), u0)
    return ebpSolve(prob, 'Scheme', 'bdf2', 'Dt', spec['Dt'], 'TFinal', spec['TFinal'], 'BaseCells',
                    spec['BaseCells'], 'MaxLevels', spec['MaxLevels'], 'RegridEvery', spec['RegridEvery'],
                    'StepVerbose', 0, 'Precision', spec.get('Precision', 'fp64'), backend=backend)


class DistanceService:
    """The polygon distances of the builder processes, computed on the GPU.

    A builder has no CUDA context (many contexts would time-slice the GPU),
    but most of a diffuse-domain request's host set-up is the signed distance
    of every sample point to its 3000-point interface (the segment minimum of
    ddStarfishGeometry.m:140-177).  The builder keeps the O(n) host part
    (polar-angle segment, starting candidate, radial sign) and hands the
    segment minimum to this service: the points go through a shared-memory
    block, one thread of the server process runs ``bsam_polygon_dist2`` on a
    context and stream of its own, and writes the minima back in place.  The
    minimum over all segments is the same whichever search finds it, so a
    hierarchy built this way equals the host-built one bit for bit.
    """

    def __init__(self, mpctx, nworkers, device=0, dist2=None, threads=2):
        self.req = mpctx.Queue()
        self.resp = [mpctx.Queue() for _ in range(nworkers)]
        self.slot = mpctx.Value('i', 0)
        self.calls = 0
        self.points = 0
        self.busy_s = 0.0
        self.stat = threading.Lock()
        # several serving threads, each with its own context and stream, so
        # one builder's copies overlap another's kernel
        self.threads = []
        for i in range(max(1, int(threads))):
            fn = dist2
            if fn is None:     # the device's segment minimum on a context of its own
                from .device import Context, polygon_dist2
                ctx = Context(device)
                fn = lambda verts, x, y, best, ctx=ctx: polygon_dist2(ctx, verts, x, y, best)
            t = threading.Thread(target=self._serve, args=(fn,), name=f'bsam-distance-{i}', daemon=True)
            t.start()
            self.threads.append(t)

    def initargs(self):
        return (self.req, self.resp, self.slot)

    def _serve(self, dist2):
        from multiprocessing import shared_memory
        while True:
            msg = self.req.get()
            if msg is None:
                return
            wid, name, nv, n = msg
            err = None
            t0 = time.perf_counter()
            try:
                # the builder owns the block and unlinks it (the builders share
                # this process's resource tracker, so attaching adds nothing
                # it has to forget)
                shm = shared_memory.SharedMemory(name=name)
                buf = np.ndarray((2 * nv + 3 * n,), dtype=np.float64, buffer=shm.buf)
                verts = buf[:2 * nv].reshape(nv, 2)
                x, y, best = buf[2 * nv:2 * nv + n], buf[2 * nv + n:2 * nv + 2 * n], buf[2 * nv + 2 * n:]
                dist2(verts, x, y, best)
                del buf, verts, x, y, best
                shm.close()
                with self.stat:
                    self.calls += 1
                    self.points += n
            except Exception as e:  # noqa: BLE001 -- reported to the builder
                err = repr(e)
            with self.stat:
                self.busy_s += time.perf_counter() - t0
            self.resp[wid].put(err)

    def close(self):
        for _ in self.threads:
            self.req.put(None)
        for t in self.threads:
            t.join()


class RemoteDistance:
    """A builder's handle on the DistanceService (``StarGeometry(device=...)``)."""

    def __init__(self, req, resp, wid):
        self.req, self.resp, self.wid = req, resp, wid

    def dist2(self, verts, x, y, best):
        from multiprocessing import shared_memory
        nv, n = int(verts.shape[0]), int(x.size)
        shm = shared_memory.SharedMemory(create=True, size=8 * (2 * nv + 3 * n))
        try:
            buf = np.ndarray((2 * nv + 3 * n,), dtype=np.float64, buffer=shm.buf)
            buf[:2 * nv] = np.ascontiguousarray(verts, dtype=np.float64).ravel()
            buf[2 * nv:2 * nv + n] = x
            buf[2 * nv + n:2 * nv + 2 * n] = y
            buf[2 * nv + 2 * n:] = best
            self.req.put((self.wid, shm.name, nv, n))
            err = self.resp.get(timeout=300)
            if err is not None:
                raise RuntimeError(f'bsam_serve:distance: {err}')
            best[:] = buf[2 * nv + 2 * n:]
            del buf
        finally:
            shm.close()
            shm.unlink()
        return best


_REMOTE = None        # this builder's RemoteDistance (set by _worker_init)


def _worker_init(req=None, resp=None, slot=None):
    global _REMOTE
    os.environ['OMP_NUM_THREADS'] = '1'
    os.environ['OPENBLAS_NUM_THREADS'] = '1'
    os.environ['BSAM_HOST_THREADS'] = '1'       # the pool already uses every core
    if req is not None:
        with slot.get_lock():
            wid = slot.value
            slot.value += 1
        _REMOTE = RemoteDistance(req, resp[wid], wid)


def _warm(_):
    """Import the set-up modules in a fresh builder process."""
    from . import ddm, flat, hierarchy, solve, tagcluster  # noqa: F401
    return os.getpid()


def _solve_key(opts, fl):
    return (tuple(np.round(fl.hs[0], 15)), int(fl.patches[0][5]), int(fl.patches[0][6]),
            int(opts['NPre']), int(opts['NPost']), float(opts['Omega']), str(opts['GhostInterp']).lower(),
            bool(opts['MassCorrection']), str(opts['Precision']).lower())


def footprint_bytes(fl, mixed):
    """Device bytes a flat hierarchy holds while it is solved: FP64 fields
    and coefficients (with the state snapshot), the plan's index tables, and
    the FP32 copies of the mixed form."""
    cells, q, qc = fl.F.size, fl.Q.size, fl.QC.size
    f64 = 2 * q + 6 * cells + fl.DeW.size + fl.DnS.size + 2 * qc + fl.pcoef.size + fl.cfd.size + fl.bcg.size + \
        np.asarray(fl.Ainv).size + fl.bcRhs.size
    ints = fl.same.size + fl.ring.size + fl.win.size + fl.fp.size + fl.corr.size + 12 * cells // 8 + 10 * q // 8
    f32 = (q + 4 * cells + fl.DeW.size + fl.DnS.size + qc + fl.pcoef.size + fl.cfd.size + fl.bcg.size) if mixed else 0
    return int(8 * f64 + 4 * ints + 4 * f32 + cells + (1 << 20))


def build_spec(spec):
    """Build one request's hierarchy (runs in a builder process); returns the
    flat tables, solve options and footprint."""
    import warnings
    t0 = time.perf_counter()
    from .flat import flatten
    from .options import ebOptions
    from .solve import build_hierarchy
    from .device import DeferredBackend
    be = DeferredBackend()
    if spec['kind'] == 'dd_star':
        from .ddm import StarGeometry, ddTransmissionProblem, starfish_q, starfish_h, starfish_tag
        g = StarGeometry(3000, spec['a0'], 1.0, spec['b'], float(spec['k']), spec['th0'], device=_REMOTE)
        data = dict(STAR_DATA, q=starfish_q, h=starfish_h)
        prob, _ = ddTransmissionProblem(g, spec['eps'], STAR_BOX, data)
        opts = ebOptions('BaseCells', 64, 'MaxLevels', int(spec['MaxLevels']), 'Indicator', 'fun',
                         'TagFunction', starfish_tag(g, spec['eps'], 64), 'TagBuffer', 2, 'RelTol', 1e-10,
                         'MaxVCycles', 100, 'Verbose', 0, 'Precision', spec.get('Precision', 'mixed'))
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            H = build_hierarchy(prob, opts, be)
        fl = flatten(H)
    elif spec['kind'] == 'elliptic':
        # an elliptic problem with a geometric ('fun') tag rule:
        # spec['problem'] = (domain, D, C, f, bc), spec['options'] ebOptions pairs
        from .problem import ebProblem
        prob = ebProblem(*spec['problem'])
        opts = ebOptions(*spec['options'])
        if str(opts.Indicator).lower() != 'fun':
            raise ValueError('bsam_serve:indicator: served elliptic requests use a geometric tag function')
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            H = build_hierarchy(prob, opts, be)
        fl = flatten(H)
    else:
        raise ValueError(f"bsam_serve:kind: unknown request kind {spec['kind']}")
    mixed = str(opts['Precision']).lower() == 'mixed'
    sopts = {k: opts[k] for k in ('NPre', 'NPost', 'Omega', 'GhostInterp', 'MassCorrection', 'MaxVCycles',
                                  'RelTol', 'Precision')}
    return {'flat': fl, 'opts': sopts, 'key': _solve_key(sopts, fl), 'footprint': footprint_bytes(fl, mixed),
            'build_s': time.perf_counter() - t0}


class Result:
    def __init__(self, rid, spec, Q, flat, vcycles, hist, rel, visible, times):
        self.id, self.spec, self.Q, self.flat = rid, spec, Q, flat
        self.vcycles, self.hist, self.final_rel, self.visible_cells = vcycles, hist, rel, visible
        self.times = times

    @property
    def latency_s(self):
        return self.times['done'] - self.times['submit']


class Server:
    """The serving loop (see the module docstring).

    builders       worker processes for the host set-up
    waves          waves in flight on the GPU at once (one stream each)
    wave_size      most requests merged into one wave
    budget_bytes   device memory the in-flight waves may hold (default: half
                   of the free device memory at start)
    """

    def __init__(self, builders=None, waves=3, wave_size=64, budget_bytes=None, device=0, build_fn=None,
                 gpu_distance=True):
        from .device import Context
        self.device = device
        self.nbuild = builders or max(1, min(16, (os.cpu_count() or 2) - 1))
        self.pool = None
        self.distance = None
        if build_fn is None:
            # builder processes inherit a one-thread BLAS / OpenMP setting
            # (several of them share the host's cores)
            saved = {k: os.environ.get(k) for k in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS')}
            os.environ.update(OMP_NUM_THREADS='1', OPENBLAS_NUM_THREADS='1')
            try:
                spawn = mp.get_context('spawn')
                if gpu_distance and device is not None:
                    self.distance = DistanceService(spawn, self.nbuild, device)
                self.pool = cf.ProcessPoolExecutor(self.nbuild, mp_context=spawn, initializer=_worker_init,
                                                   initargs=self.distance.initargs() if self.distance else ())
                list(self.pool.map(_warm, range(self.nbuild)))
            finally:
                for k, v in saved.items():
                    if v is None:
                        os.environ.pop(k, None)
                    else:
                        os.environ[k] = v
            build_fn = build_spec
        self.build_fn = build_fn
        # device None: host logic only (waves run by an overriding _solve)
        self.ctxs = [Context(device) if device is not None else None for _ in range(waves)]
        if budget_bytes is None:
            from .device import memory_info
            budget_bytes = memory_info(device)[0] // 2
        self.budget = int(budget_bytes)
        self.wave_size = int(wave_size)
        self.lock = threading.Condition()
        self.ready = deque()           # (rid, spec, built, times)
        self.free_slots = list(range(waves))
        self.inflight = 0
        self.nextid = 0
        self.futures = {}
        self.closed = False
        self.waves_run = []
        self.errors = []
        # one long-lived worker thread per wave slot
        self.workers = cf.ThreadPoolExecutor(max_workers=waves, thread_name_prefix='bsam-wave')
        self.dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.dispatcher.start()

    # ---- client side ----------------------------------------------------------
    def submit(self, spec):
        with self.lock:
            rid = self.nextid
            self.nextid += 1
            fut = cf.Future()
            self.futures[rid] = fut
        times = {'submit': time.perf_counter()}
        if spec.get('kind') == 'parabolic':
            # no host set-up stage: the run sets up and steps on its slot
            base = int(spec['BaseCells'])
            built = {'flat': None, 'opts': {}, 'key': ('parabolic', rid), 'build_s': 0.0, 'solo': True,
                     'footprint': int(400 * base * base * 4 ** (int(spec['MaxLevels']) - 1)) + (1 << 22)}
            bf = cf.Future()
            bf.set_result(built)
            bf.add_done_callback(lambda f, rid=rid, spec=spec, times=times: self._built(rid, spec, f, times))
            return fut
        if self.pool is not None:
            bf = self.pool.submit(self.build_fn, spec)
        else:
            bf = cf.Future()
            try:
                bf.set_result(self.build_fn(spec))
            except Exception as e:  # noqa: BLE001 -- delivered to the caller
                bf.set_exception(e)
        bf.add_done_callback(lambda f, rid=rid, spec=spec, times=times: self._built(rid, spec, f, times))
        return fut

    def close(self):
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        self.dispatcher.join()
        self.workers.shutdown()
        if self.pool is not None:
            self.pool.shutdown()
        if self.distance is not None:
            self.distance.close()

    # ---- stages -----------------------------------------------------------------
    def _built(self, rid, spec, f, times):
        times['built'] = time.perf_counter()
        try:
            built = f.result()
        except Exception as e:  # noqa: BLE001
            self.futures.pop(rid).set_exception(e)
            return
        if built['footprint'] > self.budget:
            self.futures.pop(rid).set_exception(
                MemoryError(f"bsam_serve:footprint: request needs {built['footprint']} bytes, budget {self.budget}"))
            return
        with self.lock:
            self.ready.append((rid, spec, built, times))
            self.lock.notify_all()

    def _take_wave(self):
        """Oldest ready request's group, FIFO, while memory and size allow."""
        if not self.ready or not self.free_slots:
            return None
        key = self.ready[0][2]['key']
        take, rest, used = [], deque(), 0
        for item in self.ready:
            b = item[2]
            if (b['key'] == key and len(take) < (1 if b.get('solo') else self.wave_size) and
                    self.inflight + used + b['footprint'] <= self.budget):
                take.append(item)
                used += b['footprint']
            else:
                rest.append(item)
        if not take:
            return None
        self.ready = rest
        self.inflight += used
        return self.free_slots.pop(), take, used

    def _dispatch(self):
        while True:
            with self.lock:
                while True:
                    w = self._take_wave()
                    if w is not None or (self.closed and not self.ready and len(self.free_slots) == len(self.ctxs)):
                        break
                    self.lock.wait(0.05)
                if w is None:
                    return
            self.workers.submit(self._run_wave, *w)

    def _solve(self, slot, items):
        """One wave on the GPU: merged upload, ebSolveCycles of every
        instance, per-instance solutions and histories (a parabolic request:
        its whole run on the slot's stream)."""
        if items[0][2].get('solo'):
            from .device import DeviceBackend
            from .flat import flatten
            sol = run_parabolic(items[0][1], DeviceBackend.on(self.ctxs[slot]))
            fl = flatten(sol['H'])
            items[0][2]['flat'] = fl
            items[0][2]['solution'] = sol
            return [(fl.Q, int(np.sum(sol['cycles'])), np.asarray(sol['relres']), float(np.max(sol['relres'])),
                     int(fl.F.size))]
        from .batch import merge_flats, split_field
        from .device import DevHier, BSAM_FIELD_Q
        from .flat import FIELD_Q
        parts = [it[2]['flat'] for it in items]
        opts = dict(items[0][2]['opts'])
        b = merge_flats(parts)
        dh = DevHier(self.ctxs[slot], b, opts)
        dh.setup_levels()
        for i, it in enumerate(items):
            o = it[2]['opts']
            if o['MaxVCycles'] != opts['MaxVCycles'] or o['RelTol'] != opts['RelTol']:
                dh.set_stop(i, int(o['MaxVCycles']), float(o['RelTol']))
        dh.solve_cycles(int(max(it[2]['opts']['MaxVCycles'] for it in items)) + 2)
        Q = dh.get(BSAM_FIELD_Q, b.Q.size)
        out = []
        for i, it in enumerate(items):
            r = dh.batch_result(i, int(it[2]['opts']['MaxVCycles']) + 2)
            out.append((split_field(b, FIELD_Q, Q, i),) + tuple(r))
        del dh
        return out

    def _run_wave(self, slot, items, used):
        t0 = time.perf_counter()
        try:
            for _, _, _, times in items:
                times['wave_start'] = t0
            res = self._solve(slot, items)
            t1 = time.perf_counter()
            self.waves_run.append({'size': len(items), 'start': t0, 'end': t1, 'bytes': used})
            for i, (rid, spec, built, times) in enumerate(items):
                times['done'] = time.perf_counter()
                q, it, hist, rel, vis = res[i]
                r = Result(rid, spec, q, built['flat'], it, hist, rel, vis, times)
                r.solution = built.get('solution')
                self.futures.pop(rid).set_result(r)
        except Exception as e:  # noqa: BLE001 -- every request of the wave learns of it
            self.errors.append(repr(e))
            for rid, _, _, _ in items:
                f = self.futures.pop(rid, None)
                if f is not None:
                    f.set_exception(e)
        finally:
            with self.lock:
                self.inflight -= used
                self.free_slots.append(slot)
                self.lock.notify_all()


def run_stream(server, specs, rate, seed=0):
    """Submit `specs` with Poisson arrivals at `rate` requests/s; returns the
    results and the wall time from the first submission to the last result."""
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    gaps = rng.exponential(1.0 / rate, len(specs))
    t0 = time.perf_counter()
    futs = []
    tnext = t0
    for s, g in zip(specs, gaps):
        now = time.perf_counter()
        if tnext > now:
            time.sleep(tnext - now)
        futs.append(server.submit(s))
        tnext += g
    results = [f.result() for f in futs]
    return results, time.perf_counter() - t0


def summarize(results, wall):
    lat = np.array([r.latency_s for r in results]) * 1e3
    build = np.array([r.times['built'] - r.times['submit'] for r in results]) * 1e3
    wait = np.array([r.times['wave_start'] - r.times['built'] for r in results]) * 1e3
    solve = np.array([r.times['done'] - r.times['wave_start'] for r in results]) * 1e3
    return {'requests': len(results), 'wall_s': wall, 'solves_per_s': len(results) / wall,
            'p50_ms': float(np.percentile(lat, 50)), 'p99_ms': float(np.percentile(lat, 99)),
            'build_p50_ms': float(np.percentile(build, 50)), 'queue_p50_ms': float(np.percentile(wait, 50)),
            'wave_p50_ms': float(np.percentile(solve, 50)),
            'max_final_rel': float(max(r.final_rel for r in results))}
