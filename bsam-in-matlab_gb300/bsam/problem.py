"""Problem definition, mirroring ``EllipticBSAM/src/ebProblem.m:1-63``.

    -div(D(x,y) grad u) + C(x,y) u = f(x,y)   on [a,b] x [c,d]

``D``, ``C``, ``f`` (and the boundary data ``g`` and ``exact``) are callables
``fn(X, Y) -> ndarray`` evaluated on ndgrid-shaped arrays, or scalars (which
become constant fields exactly like the reference's ``tofun``).  Boundary
conditions are either one ``(type, g)`` pair applied to all four sides or a
dict with keys ``west/east/south/north``.
"""
from __future__ import annotations

import numpy as np

SIDES = ('west', 'east', 'south', 'north')


class Problem(dict):
    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError as e:
            raise AttributeError(name) from e

    def __setattr__(self, name, value):
        self[name] = value


def tofun(v, label):
    """Scalar -> constant field; callable passes through (``ebProblem.m:54-63``)."""
    if callable(v):
        return v
    if np.isscalar(v) and np.isreal(v):
        vv = float(v)
        return lambda X, Y: vv * np.ones(np.shape(X))
    raise ValueError(f'eb_problem:badinput: {label} must be a function handle or scalar.')


def ebProblem(domain, D, C, f, bc, exact=None) -> Problem:
    domain = [float(v) for v in domain]
    if len(domain) != 4 or domain[1] <= domain[0] or domain[3] <= domain[2]:
        raise ValueError('eb_problem:domain: domain must be [a b c d] with b>a, d>c.')
    prob = Problem()
    prob.domain = domain
    prob.D = tofun(D, 'D')
    prob.C = tofun(C, 'C')
    prob.f = tofun(f, 'f')
    if isinstance(bc, (list, tuple)) and len(bc) == 2 and isinstance(bc[0], str):
        bc = {s: bc for s in SIDES}
    sides = []
    for s in SIDES:
        if s not in bc:
            raise ValueError(f'eb_problem:bc: bc missing side {s}')
        t = str(bc[s][0]).lower()
        if t not in ('dirichlet', 'neumann'):
            raise ValueError('eb_problem:bc: bc type must be dirichlet or neumann')
        sides.append({'type': t, 'g': tofun(bc[s][1], 'g_' + s)})
    prob.bc = sides
    prob.exact = tofun(exact, 'exact') if exact is not None else None
    return prob


def ebtProblem(domain, D, C, f, bc, exact=None) -> Problem:
    """``ebtProblem`` (``EllipticBSAMTree/src/ebtProblem.m``): the same
    problem; its errors carry the tree identifiers (``ebt_problem:*``)."""
    try:
        return ebProblem(domain, D, C, f, bc, exact)
    except ValueError as e:
        m = str(e)
        if m.startswith('eb_problem:'):
            raise ValueError('ebt_' + m[3:]) from None
        raise
