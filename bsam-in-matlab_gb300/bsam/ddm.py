"""Diffuse-domain problems (host set-up): the starfish geometry and the
two-sided transmission coefficients.

``ddStarfishGeometry`` follows ``DiffuseDomainBSAM/src/ddStarfishGeometry.m``
(polygon, bounding-box tree, exact segment distance, radial sign test; the
arithmetic is in ``csrc/bsam_host.c``).  ``ddTransmissionProblem`` follows
``DiffuseDomainBSAM/src/ddTransmissionProblem.m:14-23``:

    phi   = (1 + tanh(d/eps))/2,  delta = sech(d/eps)^2/(2 eps)
    D = alpha + (1-alpha) phi
    C = beta + (gamma-beta) phi + kappa delta
    F = h (1-phi) + q phi - g delta

Transcendentals go through the C library (``bsam.hostlib``) so sampled
coefficients carry the same bits on every host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import hostlib
from .problem import ebProblem


class StarGeometry:
    """Closed polygon r(theta) = s0 (s1 + s2 sin(k theta + th0)) with n
    points (last = first), signed distance positive inside."""

    def __init__(self, n=3000, s0=0.9, s1=1.2, s2=0.7, k=5.0, th0=0.0, name=None, device=None):
        if n < 32:
            raise ValueError('dd_starfish:n: n must be an integer >= 32')
        self.n = int(n)
        self.params = (s0, s1, s2, k, th0)
        self._h = hostlib.lib().bsam_starfish_new(int(n), float(s0), float(s1), float(s2), float(k), float(th0))
        self.name = name or f'star: r = {s0}({s1} + {s2} sin({k} theta + {th0}))'
        # a bsam.device.Context, or a serving builder's RemoteDistance: the
        # segment minimum runs on the GPU
        self.device = device
        self._cache = []              # recent (key, d): phi, delta, D, C, F sample the same points
        self._pref = {}               # key -> (x, y, d) of the point sets handed to prefetch()

    def __del__(self):
        try:
            hostlib.lib().bsam_starfish_free(self._h)
        except Exception:
            pass

    @property
    def vertices(self):
        nv = hostlib.lib().bsam_starfish_nvert(self._h)
        out = np.empty(2 * nv)
        hostlib.lib().bsam_starfish_vertices(self._h, out.ctypes.data)
        return out.reshape(nv, 2)

    def signedDistance(self, X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        if X.shape != Y.shape:
            raise ValueError('X and Y must have equal size.')
        x = np.ascontiguousarray(X.ravel(order='F'))
        y = np.ascontiguousarray(Y.ravel(order='F'))
        key = (x.size, hash(x.tobytes()), hash(y.tobytes()))
        for k, (kk, xx, yy, dd) in enumerate(self._cache):
            if kk == key and np.array_equal(xx, x) and np.array_equal(yy, y):
                return dd.reshape(X.shape, order='F').copy()
        hit = self._pref.get(key)
        if hit is not None and np.array_equal(hit[0], x) and np.array_equal(hit[1], y):
            d = hit[2]
        else:
            d = self._distance(x, y)
        self._cache.insert(0, (key, x, y, d))
        del self._cache[6:]
        return d.reshape(X.shape, order='F').copy()

    def _distance(self, x, y):
        if self.device is None:
            d = np.empty_like(x)
            hostlib.lib().bsam_starfish_distance_mt(self._h, x.ctypes.data, y.ctypes.data, d.ctypes.data, x.size,
                                                    hostlib.host_threads())
            return d
        best = np.empty_like(x)
        sign = np.empty_like(x)
        hostlib.lib().bsam_starfish_init_sign(self._h, x.ctypes.data, y.ctypes.data, best.ctypes.data,
                                              sign.ctypes.data, x.size)
        if hasattr(self.device, 'dist2'):     # a builder process: the server's GPU distance service
            self.device.dist2(self.vertices, x, y, best)
        else:
            from .device import polygon_dist2
            polygon_dist2(self.device, self.vertices, x, y, best)
        return sign * np.sqrt(best)

    def prefetch(self, sets):
        """Compute the distances of many point sets (pairs of X, Y arrays)
        in one call -- on every host thread, or in one device launch -- and
        keep them until the next prefetch, so the per-patch calls that
        follow are lookups.  Each point's distance is its own minimum over
        the segments, so the values are the ones a call per set gives."""
        self._pref = {}
        xs, ys = [], []
        for X, Y in sets:
            xs.append(np.asarray(X, dtype=np.float64).ravel(order='F'))
            ys.append(np.asarray(Y, dtype=np.float64).ravel(order='F'))
        if not xs:
            return
        d = self._distance(np.ascontiguousarray(np.concatenate(xs)), np.ascontiguousarray(np.concatenate(ys)))
        o = 0
        for x, y in zip(xs, ys):
            x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
            self._pref[(x.size, hash(x.tobytes()), hash(y.tobytes()))] = (x, y, d[o:o + x.size])
            o += x.size

    def psi(self, X, Y):
        return -self.signedDistance(X, Y)

    def inside(self, X, Y):
        return self.signedDistance(X, Y) >= 0


def ddStarfishGeometry(n=3000):
    """The five-armed starfish r = 0.9 (1.2 + 0.7 sin 5 theta)."""
    return StarGeometry(n, 0.9, 1.2, 0.7, 5.0, 0.0,
                        name='Helmholtz starfish: r = 0.9(1.2 + 0.7 sin(5 theta))')


def starfish_q(x, y):
    """q(x,y) = 15 - x^2 (demoStarfish.m:13)."""
    return 15 - x ** 2


def starfish_h(x, y):
    """h(x,y) = 2.5 sin x + exp(cos y) (demoStarfish.m:13)."""
    return 2.5 * hostlib.sin(x) + hostlib.exp(hostlib.cos(y))


def _tofun(v):
    if callable(v):
        return v
    vv = float(v)
    return lambda X, Y: vv + np.zeros(np.shape(X))


def ddTransmissionProblem(geom, epsilon, box, data):
    """Two-sided diffuse-domain transmission problem (``ddTransmissionProblem.m``)."""
    if not (np.isscalar(epsilon) and epsilon > 0 and np.isfinite(epsilon)):
        raise ValueError('dd_transmission:epsilon: epsilon must be a positive finite scalar')
    if not data['alpha'] > 0:
        raise ValueError('dd_transmission:alpha: alpha must be positive')
    for f in ('beta', 'gamma', 'kappa'):
        if data[f] < 0:
            raise ValueError(f'dd_transmission:{f}: {f} must be nonnegative')
    eps = float(epsilon)
    recent = []            # (X, Y, phi, delta) of the last point sets: D, C and F sample the same points

    def _fields(X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        for XX, YY, ph, de in recent:
            if XX.shape == X.shape and np.array_equal(XX, X) and np.array_equal(YY, Y):
                return ph, de
        d = geom.signedDistance(X, Y)
        ph = (1 + hostlib.tanh(d / eps)) / 2
        de = (1.0 / hostlib.cosh(d / eps)) ** 2 / (2 * eps)
        recent.insert(0, (X.copy(), Y.copy(), ph, de))
        del recent[3:]
        return ph, de

    def phi(X, Y):
        return _fields(X, Y)[0].copy()

    def delta(X, Y):
        return _fields(X, Y)[1].copy()

    q, h, g = _tofun(data['q']), _tofun(data['h']), _tofun(data['g'])
    al, be, ga, ka = float(data['alpha']), float(data['beta']), float(data['gamma']), float(data['kappa'])

    def D(X, Y):
        return al + (1 - al) * phi(X, Y)

    def Cf(X, Y):
        return be + (ga - be) * phi(X, Y) + ka * delta(X, Y)

    def Ff(X, Y):
        return h(X, Y) * (1 - phi(X, Y)) + q(X, Y) * phi(X, Y) - g(X, Y) * delta(X, Y)

    bc = data.get('OuterBC', ('neumann', 0))
    prob = ebProblem(box, D, Cf, Ff, bc, data.get('exact'))
    prob.prefetch = geom.prefetch       # make_level hands over a level's sample points first
    aux = {'phi': phi, 'delta': delta, 'epsilon': eps, 'signedDistance': geom.signedDistance,
           'vertices': geom.vertices}
    return prob, aux


def starfish_problem(n=3000, epsilon=0.05):
    """The starfish transmission problem of examples/demoStarfish.m:11-14."""
    g = ddStarfishGeometry(n)
    data = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'q': starfish_q, 'h': starfish_h, 'g': 4}
    prob, aux = ddTransmissionProblem(g, epsilon, [-2, 2, -2, 2], data)
    return prob, aux, g


def starfish_tag(g, epsilon=0.05, base=64):
    """Tag rule of demoStarfish.m:16: |d| < max(3 eps, 3*4/(base 2^(L-1)))."""
    def tag(x, y, L):
        return np.abs(g.signedDistance(x, y)) < max(3 * epsilon, 3 * 4 / (base * 2 ** (L - 1)))
    return tag
