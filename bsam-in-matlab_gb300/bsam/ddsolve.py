"""Diffuse-domain problems posed on an internal domain Omega_1 (host set-up):
level-set geometries, the one-sided diffuse-domain reformulation and the
driver that solves it with the adaptive solver.

``ddGeometry`` follows ``DiffuseDomainBSAM/src/ddGeometry.m:21-172``
(circle, ellipse, Feng et al.'s star, generic polar curves, flower3,
peanut, regular polygons with the exact signed distance), ``ddProblem``
``ddProblem.m:29-78`` (Neumann via |grad phi| g, Dirichlet penalty),
``ddSolve`` ``ddSolve.m:14-50`` and ``ddErrorInside`` ``ddErrorInside.m``.
The phase field is phi = (1 - tanh(3 psi / eps)) / 2, phi ~ 1 inside.
Transcendentals go through the C library (``bsam.hostlib``) so sampled
coefficients carry the same bits on every host.
"""
from __future__ import annotations

import numpy as np

from . import hostlib
from .options import ebOptions
from .problem import ebProblem


class Geometry:
    """psi(X, Y) < 0 inside Omega_1, gpsi(X, Y) -> (psix, psiy), gpsimag."""

    def __init__(self, psi, gpsi, gpsimag, name, vertices=None):
        self.psi, self.gpsi, self.gpsimag, self.name = psi, gpsi, gpsimag, name
        self.vertices = vertices


def _arr(X):
    return np.asarray(X, dtype=np.float64)


def _polar(Rf, Rpf, name):
    """Simple closed polar curve r = R(theta) > 0: psi = r - R(theta)."""
    def psi(X, Y):
        X, Y = _arr(X), _arr(Y)
        return hostlib.hypot(X, Y) - Rf(hostlib.atan2(Y, X))

    def gpsi(X, Y):
        X, Y = _arr(X), _arr(Y)
        r = np.maximum(hostlib.hypot(X, Y), 1e-10)
        Rp = Rpf(hostlib.atan2(Y, X))
        return X / r + Rp * Y / r ** 2, Y / r - Rp * X / r ** 2

    def gpsimag(X, Y):
        gx, gy = gpsi(X, Y)
        return hostlib.hypot(gx, gy)

    return Geometry(psi, gpsi, gpsimag, name)


def _poly_core(X, Y, vx, vy):
    """Exact signed distance to a convex polygon (CCW vertices) and its
    gradient (ddGeometry.m:126-161)."""
    X, Y = _arr(X), _arr(Y)
    sz = X.shape
    px, py = X.ravel(order='F'), Y.ravel(order='F')
    n = len(vx)
    dmin = np.full(px.size, np.inf)
    dvx, dvy = np.zeros(px.size), np.zeros(px.size)
    enx, eny = np.zeros(px.size), np.zeros(px.size)
    inside = np.ones(px.size, dtype=bool)
    for k in range(n):
        ax, ay = vx[k], vy[k]
        kb = (k + 1) % n
        bx, by = vx[kb], vy[kb]
        ex, ey = bx - ax, by - ay
        t = ((px - ax) * ex + (py - ay) * ey) / (ex ** 2 + ey ** 2)
        t = np.minimum(np.maximum(t, 0), 1)
        dx = px - (ax + t * ex)
        dy = py - (ay + t * ey)
        d = hostlib.hypot(dx, dy)
        m = d < dmin
        dmin[m], dvx[m], dvy[m] = d[m], dx[m], dy[m]
        elen = float(hostlib.hypot(ex, ey))
        enx[m], eny[m] = ey / elen, -ex / elen
        inside &= (ex * (py - ay) - ey * (px - ax)) >= 0
    s = np.ones(px.size)
    s[inside] = -1
    psi = (s * dmin).reshape(sz, order='F')
    dn = np.maximum(dmin, np.finfo(float).tiny)
    gx = s * dvx / dn
    gy = s * dvy / dn
    # on an edge the closest-point displacement vanishes; the edge normal
    # is the gradient there
    big = max(1.0, float(np.max(np.abs(np.concatenate([vx, vy])))))
    on = dmin <= 64 * np.spacing(big)
    gx[on], gy[on] = enx[on], eny[on]
    return psi, gx.reshape(sz, order='F'), gy.reshape(sz, order='F')


def ddGeometry(kind, *args):
    """Level-set description of Omega_1 (``ddGeometry.m:21-79``)."""
    kind = str(kind).lower()
    if kind == 'circle':
        R0 = float(args[0])
        cx, cy = (float(args[1]), float(args[2])) if len(args) >= 3 else (0.0, 0.0)

        def psi(X, Y):
            return hostlib.hypot(_arr(X) - cx, _arr(Y) - cy) - R0

        def gpsi(X, Y):
            X, Y = _arr(X) - cx, _arr(Y) - cy
            r = np.maximum(hostlib.hypot(X, Y), 1e-12)
            return X / r, Y / r

        return Geometry(psi, gpsi, lambda X, Y: np.ones(np.shape(X)), f'circle R={R0:g}')
    if kind == 'ellipse':
        a, b = float(args[0]), float(args[1])
        cx, cy = (float(args[2]), float(args[3])) if len(args) >= 4 else (0.0, 0.0)

        def psi(X, Y):
            return hostlib.hypot((_arr(X) - cx) / a, (_arr(Y) - cy) / b) - 1

        def gpsi(X, Y):
            X, Y = _arr(X) - cx, _arr(Y) - cy
            r = np.maximum(hostlib.hypot(X / a, Y / b), 1e-12)
            return X / (a ** 2 * r), Y / (b ** 2 * r)

        def gmag(X, Y):
            gx, gy = gpsi(X, Y)
            return hostlib.hypot(gx, gy)

        return Geometry(psi, gpsi, gmag, f'ellipse a={a:g} b={b:g}')
    if kind == 'star':
        bpar = float(args[0]) if args else 0.5
        A3, A5 = float(hostlib.exp(2 * bpar)) / 10, float(hostlib.exp(6 * bpar)) / 50
        return _polar(lambda th: (A3 * hostlib.cos(3 * th) + A5 * hostlib.cos(5 * th)) + 1,
                      lambda th: -3 * A3 * hostlib.sin(3 * th) - 5 * A5 * hostlib.sin(5 * th), f'star b={bpar:g}')
    if kind == 'polar':
        return _polar(args[0], args[1], args[2])
    if kind == 'flower3':
        return _polar(lambda th: 1 + 0.25 * hostlib.cos(3 * th), lambda th: -0.75 * hostlib.sin(3 * th),
                      'flower3 r=1+0.25cos3t')
    if kind == 'peanut':
        return _polar(lambda th: 1 + 0.40 * hostlib.cos(2 * th), lambda th: -0.80 * hostlib.sin(2 * th),
                      'peanut r=1+0.4cos2t')
    if kind in ('polygon', 'pentagon'):
        if kind == 'pentagon':
            Nv, R = 5, float(args[0])
            rot = float(args[1]) if len(args) >= 2 else np.pi / 2
        else:
            Nv, R = int(args[0]), float(args[1])
            rot = float(args[2]) if len(args) >= 3 else np.pi / 2
        th = rot + 2 * np.pi * np.arange(Nv) / Nv
        vx, vy = R * hostlib.cos(th), R * hostlib.sin(th)
        return Geometry(lambda X, Y: _poly_core(X, Y, vx, vy)[0],
                        lambda X, Y: _poly_core(X, Y, vx, vy)[1:],
                        lambda X, Y: np.ones(np.shape(X)), f'regular {Nv}-gon R={R:g}',
                        np.stack([vx, vy], axis=1))
    raise ValueError(f'dd_geometry:kind: unknown geometry {kind}')


def _tof(v):
    if callable(v):
        return v
    vv = float(v)
    return lambda X, Y: vv * np.ones(np.shape(X))


def _get(data, f, d):
    v = data.get(f) if isinstance(data, dict) else getattr(data, f, None)
    return d if v is None else v


def ddProblem(geom, eps, box, bctype, data, PhiFloor=1e-8, Mu=1.0, OuterBC=('neumann', 0)):
    """The diffuse-domain reformulation on the box (``ddProblem.m:29-78``):
    -div(Ddd grad u) + Cdd u = fdd with phi = (1 - tanh(3 psi/eps))/2."""
    if not (np.isscalar(eps) and eps > 0 and np.isfinite(eps)):
        raise ValueError('dd_problem:eps: eps must be a positive finite scalar')
    if not (0 <= PhiFloor < 1):
        raise ValueError('dd_problem:phifloor: PhiFloor must lie in [0, 1)')
    if not Mu > 0:
        raise ValueError('dd_problem:mu: Mu must be positive')
    eps = float(eps)
    Dfun, ffun, gfun = _tof(_get(data, 'D', 1)), _tof(_get(data, 'f', 0)), _tof(_get(data, 'g', 0))
    psi = geom.psi
    recent = []            # the last point sets: D, C and f sample the same points

    def _entry(X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        for e in recent:
            if e['X'].shape == X.shape and np.array_equal(e['X'], X) and np.array_equal(e['Y'], Y):
                return e
        e = {'X': X.copy(), 'Y': Y.copy(), 'psi': np.asarray(psi(X, Y), dtype=np.float64)}
        recent.insert(0, e)
        del recent[3:]
        return e

    def phi(X, Y):
        e = _entry(X, Y)
        if 'phi' not in e:
            e['phi'] = 0.5 * (1 - hostlib.tanh(3 * e['psi'] / eps))
        return e['phi'].copy()

    def gphimag(X, Y):
        e = _entry(X, Y)
        if 'gpm' not in e:
            e['gpm'] = (3 / (2 * eps)) * (1.0 / hostlib.cosh(3 * e['psi'] / eps)) ** 2 * geom.gpsimag(X, Y)
        return e['gpm'].copy()

    def phifl(X, Y):
        return np.maximum(phi(X, Y), PhiFloor)

    bt = str(bctype).lower()
    if bt == 'neumann':
        Cfun = _tof(_get(data, 'C', 1))

        def Ddd(X, Y):
            return phifl(X, Y) * Dfun(X, Y)

        def Cdd(X, Y):
            return phifl(X, Y) * Cfun(X, Y)

        def fdd(X, Y):
            return phi(X, Y) * ffun(X, Y) + gphimag(X, Y) * gfun(X, Y)
    elif bt == 'dirichlet':
        Cfun = _tof(_get(data, 'C', 0))
        pen = Mu / eps ** 3

        def Ddd(X, Y):
            return phifl(X, Y) * Dfun(X, Y)

        def Cdd(X, Y):
            return phi(X, Y) * Cfun(X, Y) + pen * (1 - phi(X, Y))

        def fdd(X, Y):
            return phi(X, Y) * ffun(X, Y) + pen * (1 - phi(X, Y)) * gfun(X, Y)
    else:
        raise ValueError('dd_problem:bctype: bctype must be neumann or dirichlet')
    prob = ebProblem(box, Ddd, Cdd, fdd, OuterBC, _get(data, 'exact', None))
    aux = {'phi': phi, 'gradphimag': gphimag, 'psi': psi, 'epsi': eps,
           'inside': lambda X, Y: psi(X, Y) < 0,
           'tagfun': lambda width: (lambda X, Y: np.abs(psi(X, Y)) < width * eps)}
    return prob, aux


def ddErrorInside(H, uexact, aux):
    """Composite error norms on the visible cells inside Omega_1
    (``ddErrorInside.m``)."""
    dom = H.prob.domain
    linf = l2sq = 0.0
    ncell = 0
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        da = lev.h[0] * lev.h[1]
        for p in range(lev.np):
            b = lev.box[p]
            xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0]
            yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1]
            XC, YC = np.meshgrid(xc, yc, indexing='ij')
            vis = ~lev.covered[p] & (aux['psi'](XC, YC) < 0)
            if not vis.any():
                continue
            E = lev.Q[p][1:-1, 1:-1] - uexact(XC, YC)
            e = E.ravel(order='F')[vis.ravel(order='F')]
            linf = max(linf, float(np.max(np.abs(e))))
            l2sq = l2sq + float(np.sum(e ** 2)) * da
            ncell += e.size
    return {'linf': linf, 'l2': float(np.sqrt(l2sq)), 'ncell': ncell}


def ddToUniform(H, N0):
    """Project the composite solution onto a uniform N0 x N0 grid
    (``ddToUniform.m``): finer visible cells are averaged into each uniform
    cell, coarser ones are replicated; the visible cells must tile the
    domain.  Returns (U, X, Y) with X, Y the uniform cell centres."""
    dom = H.prob.domain
    U = np.zeros((N0, N0))
    W = np.zeros((N0, N0))
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        n = int(lev.n[0])
        if int(lev.n[1]) != n:
            raise ValueError('dd_to_uniform:square: square grids only.')
        for p in range(lev.np):
            b = lev.box[p]
            Qi = lev.Q[p][1:-1, 1:-1]
            vis = ~lev.covered[p]
            if not vis.any():
                continue
            if n >= N0:
                if n % N0:
                    raise ValueError(f'dd_to_uniform:align: N0 incompatible with level size {n}.')
                f = n // N0
                gi, gj = np.meshgrid(np.arange(b[0], b[1] + 1), np.arange(b[2], b[3] + 1), indexing='ij')
                vf = vis.ravel(order='F')
                s1 = -(-gi.ravel(order='F')[vf] // f)
                s2 = -(-gj.ravel(order='F')[vf] // f)
                lin = (s1 - 1) + (s2 - 1) * N0
                acc = np.zeros(N0 * N0)
                np.add.at(acc, lin, Qi.ravel(order='F')[vf] / f ** 2)
                wacc = np.zeros(N0 * N0)
                np.add.at(wacc, lin, np.ones(lin.size) / f ** 2)
                U += acc.reshape((N0, N0), order='F')
                W += wacc.reshape((N0, N0), order='F')
            else:
                if N0 % n:
                    raise ValueError(f'dd_to_uniform:align: N0 incompatible with level size {n}.')
                f = N0 // n
                R = np.repeat(np.repeat(Qi, f, axis=0), f, axis=1)
                M = np.repeat(np.repeat(vis, f, axis=0), f, axis=1)
                rows = slice((b[0] - 1) * f, b[1] * f)
                cols = slice((b[2] - 1) * f, b[3] * f)
                Ub, Wb = U[rows, cols], W[rows, cols]
                Ub[M] += R[M]
                Wb[M] += 1
    if np.max(np.abs(W - 1)) > 1e-10:
        raise ValueError('dd_to_uniform:tile: visible cells do not tile the domain.')
    U = U / W
    hx0 = (dom[1] - dom[0]) / N0
    hy0 = (dom[3] - dom[2]) / N0
    X, Y = np.meshgrid(dom[0] + (np.arange(1, N0 + 1) - 0.5) * hx0, dom[2] + (np.arange(1, N0 + 1) - 0.5) * hy0,
                       indexing='ij')
    return U, X, Y


def ddSolve(geom, eps, box, bctype, data, *args, backend=None):
    """Solve the diffuse-domain problem with the adaptive solver
    (``ddSolve.m:14-50``): ddProblem's options (PhiFloor, Mu, OuterBC),
    TagWidth (2.5: refine where |psi| < TagWidth * eps) and every ebOptions
    option as name-value pairs; Indicator 'fun' with the geometric band."""
    from .solve import ebSolve
    if len(args) % 2:
        raise ValueError('dd_solve:pairs: Options must be name-value pairs.')
    dd, rest, width = {}, [], 2.5
    for name, val in zip(args[0::2], args[1::2]):
        if str(name).lower() in ('phifloor', 'mu', 'outerbc'):
            dd[{'phifloor': 'PhiFloor', 'mu': 'Mu', 'outerbc': 'OuterBC'}[str(name).lower()]] = val
        elif str(name).lower() == 'tagwidth':
            width = val
        else:
            rest += [name, val]
    if not (np.isscalar(width) and np.isfinite(width) and width > 0):
        raise ValueError('dd_solve:tagwidth: TagWidth must be a positive finite scalar')
    prob, aux = ddProblem(geom, eps, box, bctype, data, **dd)
    opts = ebOptions('Indicator', 'fun', 'TagFunction', aux['tagfun'](width), *rest)
    sol = ebSolve(prob, opts, backend=backend)
    sol['aux'] = aux
    exact = _get(data, 'exact', None)
    sol['errInside'] = ddErrorInside(sol['H'], exact, aux) if exact is not None else None
    return sol
