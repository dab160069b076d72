"""Solve drivers: ``ebSolve`` / ``ebtSolve`` / ``ebSolveCycles``.

Host sequencing follows ``EllipticBSAM/src/ebSolve.m:22-94`` (and the tree
copy ``EllipticBSAMTree/src/ebtSolve.m``): set-up, then either geometry-
driven refinement followed by one solve (``Indicator='fun'``) or
solve / tag / add level / re-solve.  Every ``ebSolveCycles`` call -- the
reference's hot path -- runs on the GPU through the C-ABI library
(``bsam.device``); the set-up ghost fills and the new-level prolongation
run there too.
"""
from __future__ import annotations

import math

import numpy as np

from . import hierarchy as hier
from .options import ebOptions, ebtOptions
from .tagcluster import tag_cluster


class Solution(dict):
    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError as e:
            raise AttributeError(name) from e


def default_backend(opts):
    from .device import DeviceBackend
    return DeviceBackend.get(int(opts.get('Device', 0)))


def ebSolveCycles(H, backend=None):
    """Run V-cycles on H until ``rel <= RelTol`` or ``MaxVCycles``
    (``EllipticBSAM/src/ebSolveCycles.m:1-80``); appends one stage record."""
    backend = backend or default_backend(H.opts)
    it, hist, rel, vis = backend.solve_cycles(H)
    ncellTot = 0
    for k in range(H.rootIdx, H.nlev + 1):
        ncellTot += sum(f.size for f in H.lev[k].F)
    stage = {
        'amrLevels': H.nlev - H.rootIdx + 1,
        'nlev': H.nlev,
        'vcycles': int(it),
        'resHist': np.asarray(hist),
        'finalRel': float(rel),
        'visibleCells': int(vis),
        'totalCells': int(ncellTot),
    }
    if len(hist) >= 2:
        stage['avgFactor'] = (hist[-1] / max(hist[0], np.finfo(float).tiny)) ** (1.0 / (len(hist) - 1))
    else:
        stage['avgFactor'] = math.nan
    H.stats['stages'].append(stage)
    if H.opts.Verbose >= 1:
        print(f"[ebsam] stage {len(H.stats['stages'])}: {stage['amrLevels']} AMR level(s), {it} V-cycle(s), "
              f"|r|/|f| = {rel:.2e}, avg factor {stage['avgFactor']:.3f}, {vis} visible cells")
    return H


ebtSolveCycles = ebSolveCycles


def build_hierarchy(prob, opts, backend, tree=False):
    """The geometry-driven ('fun') hierarchy: set-up, then tag/cluster/add
    level until MaxLevels (``ebSolve.m:30-37``); no solve."""
    H = hier.setup(prob, opts, backend, tree=tree)
    while (H.nlev - H.rootIdx + 1) < opts.MaxLevels:
        boxes = tag_cluster(H, backend)
        if boxes.shape[0] == 0:
            break
        H = hier.add_level(H, boxes, backend)
    return H


def _solve(prob, args, kwargs, tree, backend):
    parse = ebtOptions if tree else ebOptions
    if len(args) == 1 and isinstance(args[0], dict) and not kwargs:
        opts = parse(args[0])
    else:
        opts = parse(*args, **kwargs)
    backend = backend or default_backend(opts)
    H = hier.setup(prob, opts, backend, tree=tree)
    if str(opts.Indicator).lower() == 'fun':
        while (H.nlev - H.rootIdx + 1) < opts.MaxLevels:
            boxes = tag_cluster(H, backend)
            if boxes.shape[0] == 0:
                break
            H = hier.add_level(H, boxes, backend)
        H = ebSolveCycles(H, backend)
    else:
        H = ebSolveCycles(H, backend)
        while (H.nlev - H.rootIdx + 1) < opts.MaxLevels:
            boxes = tag_cluster(H, backend)
            if boxes.shape[0] == 0:
                if opts.Verbose >= 1:
                    print(f'[ebsam] no cells tagged; stopping at {H.nlev - H.rootIdx + 1} AMR level(s)')
                break
            H = hier.add_level(H, boxes, backend)
            H = ebSolveCycles(H, backend)
    mz = opts.MeanZero
    if isinstance(mz, str) and mz.lower() == 'auto':
        mz = H.coarsest['singular']
    if mz:
        m, _ = backend.composite_mean(H)
        for k in range(1, H.nlev + 1):
            for p in range(H.lev[k].np):
                H.lev[k].Q[p] = H.lev[k].Q[p] - m
        H.touch()
    sol = Solution()
    sol['H'] = H
    sol['stats'] = H.stats
    sol['err'] = error_norms(H) if prob.exact is not None else None
    sol['mass'] = backend.mass_check(H)
    levels = []
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        d = {'n': lev.n, 'h': lev.h, 'np': lev.np, 'cells': sum(f.size for f in lev.F), 'box': lev.box.copy()}
        if tree:
            d['parent'] = lev.parent.copy()
            d['mbounds'] = lev.mbounds.copy()
        levels.append(d)
    sol['levels'] = levels
    return sol


def ebSolve(prob, *args, backend=None, **kwargs):
    """Adaptive FAS multigrid solve (``EllipticBSAM/src/ebSolve.m``)."""
    return _solve(prob, args, kwargs, False, backend)


def ebtSolve(prob, *args, backend=None, **kwargs):
    """Tree-form adaptive solve (``EllipticBSAMTree/src/ebtSolve.m``)."""
    return _solve(prob, args, kwargs, True, backend)


def error_norms(H, ufun=None):
    """``ebErrorNorms`` (``EllipticBSAM/src/ebErrorNorms.m``): composite error
    of the visible cells against the exact solution; the singular
    all-Neumann problem is compared modulo its composite mean."""
    ufun = ufun or H.prob.exact
    if ufun is None:
        raise ValueError(('ebt' if H.tree else 'eb') + '_error_norms:noexact: no exact solution available.')
    dom = H.prob.domain
    E = {}
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        for p in range(lev.np):
            b = lev.box[p]
            xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0]
            yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1]
            XC, YC = np.meshgrid(xc, yc, indexing='ij')
            E[(k, p)] = lev.Q[p][1:-1, 1:-1] - ufun(XC, YC)
    m = 0.0
    if H.coarsest['singular']:
        tot = area = 0.0
        for (k, p), e in E.items():
            da = H.lev[k].h[0] * H.lev[k].h[1]
            vis = ~H.lev[k].covered[p]
            tot += float(np.sum(e[vis])) * da
            area += np.count_nonzero(vis) * da
        m = tot / max(area, np.finfo(float).tiny)
        E = {key: e - m for key, e in E.items()}
    linf = l2sq = 0.0
    dof = 0
    for (k, p), e in E.items():
        da = H.lev[k].h[0] * H.lev[k].h[1]
        ev = e[~H.lev[k].covered[p]]
        if ev.size:
            linf = max(linf, float(np.max(np.abs(ev))))
            l2sq += float(np.sum(ev ** 2)) * da
            dof += ev.size
    return {'linf': linf, 'l2': math.sqrt(l2sq), 'dof': dof, 'meanShift': m}


def ebSample(H, xq, yq):
    """Bilinear sample of the composite solution at points (``ebSample.m``,
    tree copy ``ebtSample.m``): each point takes the finest patch that
    contains it (boundary included), interpolating the padded Q, ghosts
    included, at its fractional cell-centre index."""
    xq = np.asarray(xq, dtype=np.float64)
    yq = np.asarray(yq, dtype=np.float64)
    dom = H.prob.domain
    vals = np.full(xq.shape, np.nan)
    assigned = np.zeros(xq.shape, dtype=bool)
    for k in range(H.nlev, H.rootIdx - 1, -1):
        lev = H.lev[k]
        hx, hy = lev.h
        for p in range(lev.np):
            b = lev.box[p]
            x0 = dom[0] + (b[0] - 1) * hx
            x1 = dom[0] + b[1] * hx
            y0 = dom[2] + (b[2] - 1) * hy
            y1 = dom[2] + b[3] * hy
            inside = ~assigned & (xq >= x0) & (xq <= x1) & (yq >= y0) & (yq <= y1)
            if not inside.any():
                continue
            Q = lev.Q[p]
            m2, n2 = Q.shape
            s = (xq[inside] - x0) / hx + 1.5          # fractional 1-based padded index
            t = (yq[inside] - y0) / hy + 1.5
            i0 = np.minimum(np.maximum(np.floor(s), 1), m2 - 1).astype(np.int64)
            j0 = np.minimum(np.maximum(np.floor(t), 1), n2 - 1).astype(np.int64)
            fr = s - i0
            ft = t - j0
            vals[inside] = ((1 - fr) * (1 - ft) * Q[i0 - 1, j0 - 1] + fr * (1 - ft) * Q[i0, j0 - 1]
                            + (1 - fr) * ft * Q[i0 - 1, j0] + fr * ft * Q[i0, j0])
            assigned[inside] = True
    if not assigned.all():
        raise ValueError(('ebt' if H.tree else 'eb') + '_sample:cover: query points outside the domain.')
    return vals


ebtSample = ebSample
