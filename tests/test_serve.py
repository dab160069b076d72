"""Serving loop (bsam.serve): request recipe, admission by device footprint,
continuous batching, and the same result alone and in a mix.

The host logic runs on CPU with a fake builder and a fake wave runner; the
GPU tests serve real diffuse-domain star requests.
"""
import threading
import time

import numpy as np
import pytest

from bsam.serve import Server, star_request, run_stream, summarize


def test_star_request_recipe():
    seen_k, seen_ml = set(), set()
    for s in range(300):
        r = star_request(s)
        assert r == star_request(s)
        assert 3 <= r['k'] <= 7 and 0.3 <= r['b'] <= 0.8 and 0.8 <= r['a0'] <= 1.2
        assert 0 <= r['th0'] < 2 * np.pi and 0.02 <= r['eps'] <= 0.08 and r['MaxLevels'] in (3, 4, 5)
        assert r['a0'] * (1 + r['b']) <= 1.9
        seen_k.add(r['k'])
        seen_ml.add(r['MaxLevels'])
    assert seen_k == {3, 4, 5, 6, 7} and seen_ml == {3, 4, 5}


class FakeServer(Server):
    """Waves 'run' by sleeping; records the bytes and waves in flight."""

    def __init__(self, **kw):
        self.peak_bytes = 0
        self.peak_waves = 0
        self.running = 0
        self.wave_members = []
        self.mon = threading.Lock()
        super().__init__(device=None, **kw)

    def _solve(self, slot, items):
        with self.mon:
            self.running += 1
            self.peak_waves = max(self.peak_waves, self.running)
            self.peak_bytes = max(self.peak_bytes, self.inflight)
            self.wave_members.append([it[1]['name'] for it in items])
        time.sleep(0.03)
        with self.mon:
            self.running -= 1
        return [(np.zeros(1), 1, np.zeros(2), 0.0, 1) for _ in items]


def _fake_build(spec):
    return {'flat': None, 'opts': {}, 'key': spec['key'], 'footprint': spec['bytes'], 'build_s': 0.0}


def test_admission_respects_the_memory_budget_and_groups():
    srv = FakeServer(waves=3, wave_size=4, budget_bytes=1000, build_fn=_fake_build)
    specs = [{'name': f'r{i}', 'key': 'A' if i % 3 else 'B', 'bytes': 150 + 10 * (i % 5)} for i in range(40)]
    futs = [srv.submit(s) for s in specs]
    res = [f.result(timeout=30) for f in futs]
    srv.close()
    assert len(res) == 40
    assert srv.peak_bytes <= 1000
    assert srv.peak_waves >= 2                       # waves overlap
    for members in srv.wave_members:
        assert len(members) <= 4
        keys = {specs[int(m[1:])]['key'] for m in members}
        assert len(keys) == 1                        # one level ladder per wave
        idx = [int(m[1:]) for m in members]
        assert idx == sorted(idx)                    # FIFO within a wave


def test_oversized_request_is_rejected():
    srv = FakeServer(waves=1, wave_size=4, budget_bytes=100, build_fn=_fake_build)
    f = srv.submit({'name': 'r0', 'key': 'A', 'bytes': 500})
    with pytest.raises(MemoryError, match='bsam_serve:footprint'):
        f.result(timeout=10)
    ok = srv.submit({'name': 'r1', 'key': 'A', 'bytes': 50})
    assert ok.result(timeout=10).vcycles == 1
    srv.close()


def test_poisson_stream_driver():
    srv = FakeServer(waves=2, wave_size=8, budget_bytes=10 ** 6, build_fn=_fake_build)
    specs = [{'name': f'r{i}', 'key': 'A', 'bytes': 10} for i in range(20)]
    res, wall = run_stream(srv, specs, rate=200.0, seed=1)
    srv.close()
    for r in res:
        r.final_rel = 0.0
    s = summarize(res, wall)
    assert s['requests'] == 20 and s['p99_ms'] >= s['p50_ms'] > 0


@pytest.mark.gpu
def test_served_result_same_alone_and_in_mix():
    from bsam.serve import build_spec
    specs = [dict(star_request(s), MaxLevels=3) for s in (11, 12, 13)]
    alone = Server(waves=1, wave_size=1, build_fn=build_spec)
    ra = alone.submit(specs[0]).result(timeout=600)
    alone.close()
    mix = Server(waves=1, wave_size=3, build_fn=build_spec)
    # hold the dispatcher until all three are ready, so they share one wave
    with mix.lock:
        futs = [mix.submit(s) for s in specs]
    rm = [f.result(timeout=600) for f in futs]
    mix.close()
    assert len(mix.waves_run) == 1 and mix.waves_run[0]['size'] == 3
    assert ra.final_rel <= 1e-10 and all(r.final_rel <= 1e-10 for r in rm)
    assert ra.vcycles == rm[0].vcycles
    np.testing.assert_array_equal(ra.hist, rm[0].hist)
    np.testing.assert_array_equal(ra.Q, rm[0].Q)


@pytest.mark.gpu
def test_served_stream_with_builder_processes():
    srv = Server(builders=2, waves=2, wave_size=8)
    specs = [dict(star_request(s), MaxLevels=3) for s in range(4)]
    res, wall = run_stream(srv, specs, rate=50.0, seed=3)
    srv.close()
    s = summarize(res, wall)
    assert s['requests'] == 4 and s['max_final_rel'] <= 1e-10


@pytest.mark.gpu
def test_deferred_setup_equals_setup_on_device():
    """A hierarchy built without a device (set-up steps deferred) and then
    set up on the device holds the same fields as one whose set-up steps ran
    on the device as it was built."""
    import warnings
    from bsam import ebOptions
    from bsam.ddm import StarGeometry, ddTransmissionProblem, starfish_q, starfish_h, starfish_tag
    from bsam.device import DeviceBackend, DeferredBackend, DevHier, BSAM_FIELD_Q, BSAM_FIELD_QC
    from bsam.flat import flatten
    from bsam.solve import build_hierarchy
    from bsam.batch import merge_flats, split_field
    from bsam.flat import FIELD_Q, FIELD_QC
    from cases import vardc_problem
    be = DeviceBackend.get(0)
    flats = []
    for backend in (be, DeferredBackend()):
        g = StarGeometry(3000, 1.0, 1.0, 0.5, 4.0, 0.3)
        data = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'q': starfish_q, 'h': starfish_h, 'g': 4}
        prob, _ = ddTransmissionProblem(g, 0.04, [-2, 2, -2, 2], data)
        o = ebOptions('BaseCells', 64, 'MaxLevels', 4, 'Indicator', 'fun', 'TagFunction', starfish_tag(g, 0.04),
                      'TagBuffer', 2, 'Verbose', 0)
        band = lambda x, y: np.abs(x - y) < 0.15
        o2 = ebOptions('BaseCells', 32, 'MaxLevels', 3, 'Indicator', 'fun', 'Verbose', 0, 'TagFunction', band)
        o3 = ebOptions('BaseCells', 64, 'MaxLevels', 2, 'Indicator', 'fun', 'Verbose', 0, 'TagFunction', band)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            flats.append((flatten(build_hierarchy(prob, o, backend)),
                          flatten(build_hierarchy(vardc_problem(), o2, backend)),
                          flatten(build_hierarchy(vardc_problem(), o3, backend)), o))
    (a1, a2, a3, o), (b1, b2, b3, _) = flats
    for fa, fb in ((a1, b1), (a2, b2), (a3, b3)):   # alone
        dh = DevHier(be.ctx, fb, o)
        dh.setup_levels()
        np.testing.assert_array_equal(dh.get(BSAM_FIELD_Q, fb.Q.size), fa.Q)
        np.testing.assert_array_equal(dh.get(BSAM_FIELD_QC, fb.QC.size), fa.QC)
    # in a batch of instances with different roots (32^2 and 64^2 bases)
    # the deferred steps of each instance still run in its own order
    assert b2.rootIdx != b3.rootIdx
    bb = merge_flats([b2, b3])
    dh = DevHier(be.ctx, bb, o)
    dh.setup_levels()
    Q = dh.get(BSAM_FIELD_Q, bb.Q.size)
    for i, fa in enumerate((a2, a3)):
        np.testing.assert_array_equal(split_field(bb, FIELD_Q, Q, i), fa.Q)


@pytest.mark.gpu
def test_parabolic_request_same_alone_and_beside_waves():
    """A served parabolic run holds one wave slot with its state resident on
    that stream; beside concurrent diffuse-domain waves it gives the same
    steps and solution as alone, and the same as ebpSolve on the default
    stream."""
    from bsam.serve import build_spec, heat_request, run_parabolic
    from bsam.device import DeviceBackend
    spec = heat_request(7)
    direct = run_parabolic(spec, DeviceBackend.get(0))
    alone = Server(waves=1, wave_size=4, build_fn=build_spec)
    ra = alone.submit(spec).result(timeout=600)
    alone.close()
    mix = Server(waves=3, wave_size=4, build_fn=build_spec)
    with mix.lock:
        futs = [mix.submit(spec)] + [mix.submit(dict(star_request(s), MaxLevels=3)) for s in (21, 22)]
    rm = [f.result(timeout=600) for f in futs]
    mix.close()
    for r in (ra, rm[0]):
        np.testing.assert_array_equal(r.solution['cycles'], direct['cycles'])
        np.testing.assert_array_equal(r.solution['relres'], direct['relres'])
        for k in range(1, direct['H'].nlev + 1):
            for qa, qb in zip(direct['H'].lev[k].Q, r.solution['H'].lev[k].Q):
                np.testing.assert_array_equal(qa[1:-1, 1:-1], qb[1:-1, 1:-1])
    assert all(r.final_rel <= 1e-10 for r in rm[1:])


def _brute_dist2(verts, x, y, best):
    """Squared distance to the closed polygon by brute force (a stand-in for
    the device minimum in a CPU test of the service's plumbing)."""
    a, b = verts[:-1], verts[1:]
    for i in range(x.size):
        px, py = x[i], y[i]
        dx, dy = b[:, 0] - a[:, 0], b[:, 1] - a[:, 1]
        t = np.clip(((px - a[:, 0]) * dx + (py - a[:, 1]) * dy) / (dx * dx + dy * dy), 0, 1)
        ex, ey = a[:, 0] + t * dx - px, a[:, 1] + t * dy - py
        best[i] = min(best[i], float(np.min(ex * ex + ey * ey)))
    return best


def _remote_distances(n):
    from bsam import serve
    from bsam.ddm import StarGeometry
    g = StarGeometry(200, 0.9, 1.2, 0.5, 4.0, 0.3, device=serve._REMOTE)
    rng = np.random.Generator(np.random.PCG64(n))
    X, Y = rng.uniform(-2, 2, (2, 50))
    return X, Y, g.signedDistance(X, Y), serve._REMOTE is not None


def test_distance_service_plumbing():
    """Builder processes hand their polygon distances to the server's
    service through shared memory and get the minima back in place."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from bsam import serve
    from bsam.ddm import StarGeometry
    spawn = mp.get_context('spawn')
    svc = serve.DistanceService(spawn, 2, dist2=_brute_dist2)
    with cf.ProcessPoolExecutor(2, mp_context=spawn, initializer=serve._worker_init,
                                initargs=svc.initargs()) as pool:
        out = list(pool.map(_remote_distances, [1, 2, 3]))
    svc.close()
    host = StarGeometry(200, 0.9, 1.2, 0.5, 4.0, 0.3)
    for X, Y, d, remote in out:
        assert remote
        np.testing.assert_allclose(d, host.signedDistance(X, Y), rtol=0, atol=1e-13)
    assert svc.calls == 3 and svc.points == 150


@pytest.mark.gpu
def test_gpu_distance_builds_equal_host_builds():
    """Requests built by builder processes whose polygon distances run on
    the GPU (the server's DistanceService) solve to the same bits as
    requests built with the host distance."""
    specs = [dict(star_request(s), MaxLevels=3) for s in (21, 22)]
    out = {}
    for gpu in (True, False):
        srv = Server(builders=2, waves=1, wave_size=1, gpu_distance=gpu)
        futs = [srv.submit(s) for s in specs]
        out[gpu] = [f.result(timeout=600) for f in futs]
        if gpu:
            assert srv.distance is not None and srv.distance.calls > 0
        else:
            assert srv.distance is None
        srv.close()
    for a, b in zip(out[True], out[False]):
        for name in ('FTrue', 'DeW', 'DnS', 'CC', 'InvDiagS'):
            np.testing.assert_array_equal(getattr(a.flat, name), getattr(b.flat, name))
        np.testing.assert_array_equal(a.Q, b.Q)
        assert a.vcycles == b.vcycles and a.final_rel <= 1e-10


@pytest.mark.gpu
def test_elliptic_request_same_alone_and_beside_another_wave():
    """An elliptic request solved on one wave slot while a wave of another
    hierarchy runs on a second slot gives the same bits as when it runs
    alone."""
    from bsam.serve import build_spec
    a = dict(star_request(31), MaxLevels=3)
    b = dict(star_request(32), MaxLevels=5)
    alone = Server(waves=1, wave_size=1, build_fn=build_spec)
    ra = alone.submit(a).result(timeout=600)
    alone.close()
    mix = Server(waves=2, wave_size=1, build_fn=build_spec)
    with mix.lock:          # both ready before the dispatcher takes either
        fb = mix.submit(b)
        fa = mix.submit(a)
    rb, rm = fb.result(timeout=600), fa.result(timeout=600)
    mix.close()
    w = mix.waves_run
    assert len(w) == 2 and max(x['start'] for x in w) < min(x['end'] for x in w), w   # the waves overlapped
    assert rb.final_rel <= 1e-10 and rm.final_rel <= 1e-10
    assert rm.vcycles == ra.vcycles
    np.testing.assert_array_equal(rm.hist, ra.hist)
    np.testing.assert_array_equal(rm.Q, ra.Q)
