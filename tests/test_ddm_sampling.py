"""Diffuse-domain coefficient sampling (ddStarfishGeometry.m:140-177 signed
distance, ddTransmissionProblem.m:14-19 coefficients).

CPU: the sampled-point cache returns exactly what a fresh evaluation gives.
GPU: with the segment minimum on the device (bsam_polygon_dist2) the signed
distance equals the host restatement bit for bit, at random points and at
every sample point of the starfish hierarchy, whose uploaded tables are then
identical to the host-built ones.
"""
import numpy as np
import pytest

from bsam.ddm import StarGeometry, ddStarfishGeometry


def _points(n, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-2, 2, n), rng.uniform(-2, 2, n)


def test_distance_cache_is_exact():
    g = ddStarfishGeometry(400)
    X, Y = _points(5000)
    d1 = g.signedDistance(X, Y)
    d2 = g.signedDistance(X.copy(), Y.copy())          # served from the cache
    np.testing.assert_array_equal(d1, d2)
    X2 = X.copy()
    X2[17] += 1e-3
    d3 = g.signedDistance(X2, Y)
    assert d3[17] != d1[17]
    np.testing.assert_array_equal(np.delete(d3, 17), np.delete(d1, 17))
    fresh = StarGeometry(400, 0.9, 1.2, 0.7, 5.0, 0.0)
    np.testing.assert_array_equal(fresh.signedDistance(X2, Y), d3)


@pytest.mark.gpu
@pytest.mark.parametrize('params', [(0.9, 1.2, 0.7, 5.0, 0.0), (1.1, 1.0, 0.6, 3.0, 2.1), (0.8, 1.0, 0.3, 7.0, 4.4)])
def test_device_distance_equals_host(params):
    from bsam.device import DeviceBackend
    ctx = DeviceBackend.get(0).ctx
    host = StarGeometry(3000, *params)
    dev = StarGeometry(3000, *params, device=ctx)
    X, Y = _points(200000, seed=int(params[3]))
    # points on and next to the polygon too
    v = host.vertices
    X = np.concatenate([X, v[:, 0], v[:, 0] * (1 + 1e-9), 0.5 * (v[:-1, 0] + v[1:, 0])])
    Y = np.concatenate([Y, v[:, 1], v[:, 1] * (1 + 1e-9), 0.5 * (v[:-1, 1] + v[1:, 1])])
    np.testing.assert_array_equal(dev.signedDistance(X, Y), host.signedDistance(X, Y))


@pytest.mark.gpu
def test_starfish_hierarchy_device_sampling_identical():
    import warnings
    from bsam import ebOptions
    from bsam.ddm import ddTransmissionProblem, starfish_q, starfish_h, starfish_tag
    from bsam.device import DeviceBackend
    from bsam.flat import flatten
    from bsam.solve import build_hierarchy
    from bsam_oracle import OracleBackend
    be = DeviceBackend.get(0)
    data = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'q': starfish_q, 'h': starfish_h, 'g': 4}
    fls = []
    for device in (None, be.ctx):
        g = StarGeometry(3000, 0.9, 1.2, 0.7, 5.0, 0.0, device=device)
        prob, aux = ddTransmissionProblem(g, 0.05, [-2, 2, -2, 2], data)
        opts = ebOptions('BaseCells', 64, 'MaxLevels', 3, 'Indicator', 'fun', 'TagFunction', starfish_tag(g),
                         'TagBuffer', 2, 'RelTol', 1e-10, 'Verbose', 0)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            fls.append(flatten(build_hierarchy(prob, opts, OracleBackend())))
    a, b = fls
    np.testing.assert_array_equal(a.patches, b.patches)
    for name in ('DeW', 'DnS', 'CC', 'InvDiagS', 'FTrue', 'Q', 'pcoef', 'cfd', 'Ainv'):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)


@pytest.mark.parametrize('order', ['grid', 'reversed', 'shuffled'])
def test_distance_equals_brute_force_in_any_point_order(order):
    """Each point's search starts from its predecessor's nearest segment; the
    result is still the minimum over all segments, bit for bit, whatever
    the order of the points."""
    g = StarGeometry(3000, 0.9, 1.2, 0.7, 5.0, 0.0)
    c = -2 + (np.arange(48) + 0.5) * 4 / 48
    X, Y = np.meshgrid(c, c, indexing='ij')
    x, y = X.ravel(order='F'), Y.ravel(order='F')
    if order == 'reversed':
        x, y = x[::-1].copy(), y[::-1].copy()
    elif order == 'shuffled':
        p = np.random.Generator(np.random.PCG64(3)).permutation(x.size)
        x, y = x[p], y[p]
    d = g.signedDistance(x, y)
    v = g.vertices
    a, e = v[:-1], v[1:] - v[:-1]
    len2 = e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]
    best = np.full(x.size, np.inf)
    for j in range(a.shape[0]):            # same operation order as the library's segment distance
        dxa, dya = x - a[j, 0], y - a[j, 1]
        t = np.clip((dxa * e[j, 0] + dya * e[j, 1]) / len2[j], 0.0, 1.0)
        px, py = dxa - t * e[j, 0], dya - t * e[j, 1]
        best = np.minimum(best, px * px + py * py)
    np.testing.assert_array_equal(np.abs(d), np.sqrt(best))


def test_level_prefetch_builds_the_same_hierarchy(monkeypatch):
    """make_level hands a level's sample points to the geometry first; the
    hierarchy (every uploaded table) is the one the per-patch calls build."""
    import warnings
    from bsam import ebOptions
    from bsam.ddm import ddTransmissionProblem, starfish_q, starfish_h, starfish_tag
    from bsam.flat import flatten
    from bsam.solve import build_hierarchy
    from bsam_oracle import OracleBackend
    data = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'q': starfish_q, 'h': starfish_h, 'g': 4}
    fls = []
    for pre, threads in ((True, '4'), (False, '1')):
        monkeypatch.setenv('BSAM_HOST_THREADS', threads)
        g = StarGeometry(3000, 0.9, 1.2, 0.7, 5.0, 0.0)
        prob, _ = ddTransmissionProblem(g, 0.05, [-2, 2, -2, 2], data)
        if not pre:
            del prob['prefetch']
        opts = ebOptions('BaseCells', 64, 'MaxLevels', 3, 'Indicator', 'fun', 'TagFunction', starfish_tag(g),
                         'TagBuffer', 2, 'Verbose', 0)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            fls.append(flatten(build_hierarchy(prob, opts, OracleBackend())))
    a, b = fls
    for name, v in vars(a).items():
        if isinstance(v, np.ndarray):
            np.testing.assert_array_equal(v, getattr(b, name), err_msg=name)


def test_threaded_distance_equals_serial(monkeypatch):
    g = StarGeometry(3000, 1.1, 1.0, 0.6, 3.0, 2.1)
    X, Y = _points(300000, seed=5)
    monkeypatch.setenv('BSAM_HOST_THREADS', '1')
    d1 = g._distance(np.ascontiguousarray(X), np.ascontiguousarray(Y))
    monkeypatch.setenv('BSAM_HOST_THREADS', '7')
    d7 = g._distance(np.ascontiguousarray(X), np.ascontiguousarray(Y))
    np.testing.assert_array_equal(d1, d7)
