"""Hierarchy construction on the host (the reference keeps this in MATLAB).

Everything here is static set-up: level creation and coefficient sampling,
coefficient fill-down, boundary folds, transfer index tables, parent
coefficient windows, the coarsest-level operator and the singular-Neumann
source projection.  Nothing in this module runs inside a V-cycle; the solve
path is the CUDA library reached through ``bsam.device``.

Arrays follow the reference layout exactly: per patch, MATLAB column-major
(Fortran order, x fastest) with one ghost cell on every side of ``Q`` and
``QC``.  Boxes are 1-based ``[ilo ihi jlo jhi]`` in level-global cells.
Linear indices stored in tables are 0-based (``sub2ind - 1``).

Both hierarchy forms are built here:
  * QC-ring (``EllipticBSAM``): multi-parent gathers resolved per cell
    (``ebBuildOps.m:17-200``);
  * single-parent tree (``EllipticBSAMTree``): every patch owns exactly one
    parent, all parent transfers are slices of that parent's padded arrays
    (``ebtBuildOps.m:1-189``).
"""
from __future__ import annotations

import hashlib
import threading
from collections import OrderedDict

import numpy as np

F = 'F'  # array order used for every patch array


class Level:
    """One level of the hierarchy (``H.lev{k}`` in the reference)."""

    def __init__(self):
        self.n = None
        self.h = None
        self.np = 0
        self.box = np.zeros((0, 4), dtype=np.int64)
        self.sourceShift = 0.0
        self.Q, self.F, self.FTrue = [], [], []
        self.DeW, self.DnS, self.CC, self.InvDiagS = [], [], [], []
        self.QC = []
        self.par0 = []
        self.faceInternal = []
        self.bc = []
        self.covered = []
        self.children, self.parents = [], []
        self.cornerClass = []
        self.land = []
        self.sameOps = []
        self.ops = []
        self.cfD = []
        # tree lineage (EllipticBSAMTree): parent index (1-based) + mbounds
        self.parent = None
        self.mbounds = None


class Hierarchy:
    """``H`` of the reference: ``lev[1..nlev]`` (index 0 unused)."""

    def __init__(self, prob, opts, tree=False):
        self.prob = prob
        self.opts = opts
        self.tree = tree
        self.lev = [None]
        self.nlev = 0
        self.rootIdx = 0
        self.coarsest = {}
        self.stats = {'stages': []}
        self.compatibility = None
        self.version = 0        # bumped on every structural change
        self._dev = None        # resident device copy (bsam.device)
        self.dirty = set()      # fields edited on the host since the last sync

    def __deepcopy__(self, memo):
        """A deep copy owns no device state: the resident copy (whose handle
        only this hierarchy frees) is left out, and the copy uploads its own
        arrays when it is next solved.  A copy whose host arrays are older
        than the device (``host_stale``) keeps that flag, so using it fails
        loudly until the original is synced."""
        import copy
        new = self.__class__.__new__(self.__class__)
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            setattr(new, k, None if k == '_dev' else copy.deepcopy(v, memo))
        return new

    def touch(self):
        self.version += 1

    def mark_dirty(self, *fields):
        """Record host edits of Q / F / FTrue / QC for the resident copy."""
        self.dirty.update(fields)


# ---------------------------------------------------------------------------
# kernels used at set-up time (host): same formulas as ebKernels.m
# ---------------------------------------------------------------------------
def restrict2(A):
    """``restrict2`` (``ebKernels.m:98-102``): 0.25*(a+b+c+d), left to right."""
    return 0.25 * (((A[0::2, 0::2] + A[1::2, 0::2]) + A[0::2, 1::2]) + A[1::2, 1::2])


def invdiag2d(DeW, DnS, CC, hx, hy):
    """``invdiag2d`` (``ebKernels.m:28-34``)."""
    mx, my = CC.shape
    den = ((DeW[1:mx + 1, :] + DeW[0:mx, :]) / (hx * hx)
           + (DnS[:, 1:my + 1] + DnS[:, 0:my]) / (hy * hy)) + CC
    return 1.0 / den


def op2d(Q, DeW, DnS, CC, hx, hy):
    """``op2d`` (``ebKernels.m:13-25``): flux-form -div(D grad u) + C u."""
    mx, my = CC.shape
    feW = DeW * (Q[1:mx + 2, 1:my + 1] - Q[0:mx + 1, 1:my + 1])
    fnS = DnS * (Q[1:mx + 1, 1:my + 2] - Q[1:mx + 1, 0:my + 1])
    return ((-(feW[1:mx + 1, :] - feW[0:mx, :])) / (hx * hx)
            - (fnS[:, 1:my + 1] - fnS[:, 0:my]) / (hy * hy)) + CC * Q[1:mx + 1, 1:my + 1]


def prolong_bilin(W):
    """``prolongBilin`` (``ebKernels.m:105-123``)."""
    cm, cn = W.shape[0] - 2, W.shape[1] - 2
    C = W[1:cm + 1, 1:cn + 1]
    Wm, Wp = W[0:cm, 1:cn + 1], W[2:cm + 2, 1:cn + 1]
    Sm, Sp = W[1:cm + 1, 0:cn], W[1:cm + 1, 2:cn + 2]
    Dmm, Dpm = W[0:cm, 0:cn], W[2:cm + 2, 0:cn]
    Dmp, Dpp = W[0:cm, 2:cn + 2], W[2:cm + 2, 2:cn + 2]
    out = np.zeros((2 * cm, 2 * cn), order=F)
    out[0::2, 0::2] = (((9 * C + 3 * Wm) + 3 * Sm) + Dmm) / 16
    out[1::2, 0::2] = (((9 * C + 3 * Wp) + 3 * Sm) + Dpm) / 16
    out[0::2, 1::2] = (((9 * C + 3 * Wm) + 3 * Sp) + Dmp) / 16
    out[1::2, 1::2] = (((9 * C + 3 * Wp) + 3 * Sp) + Dpp) / 16
    return out


# ---------------------------------------------------------------------------
def rect_isect(a, b):
    r = [max(a[0], b[0]), min(a[1], b[1]), max(a[2], b[2]), min(a[3], b[3])]
    if r[0] > r[1] or r[2] > r[3]:
        return None
    return r


def near_boxes(boxes, r, pad=1):
    """Indices (ascending) of the boxes [i0, i1, j0, j1] that intersect the
    rectangle r grown by `pad` cells on every side: a superset of the boxes
    that any face- or cell-rectangle test against r can hit, so a loop over
    these in order does what the reference's loop over every patch does
    (the others intersect nothing and are skipped)."""
    b = np.asarray(boxes).reshape(-1, 4)
    m = (b[:, 0] <= r[1] + pad) & (b[:, 1] >= r[0] - pad) & (b[:, 2] <= r[3] + pad) & (b[:, 3] >= r[2] - pad)
    return np.nonzero(m)[0].tolist()


def sub2ind(m, i, j):
    """0-based linear index of 1-based (i, j) in an m-row column-major array."""
    return (np.asarray(i) - 1) + (np.asarray(j) - 1) * m


def _eid(tree, tail):
    """Error identifier: the tree copies (EllipticBSAMTree) raise ``ebt_*``."""
    return ('ebt_' if tree else 'eb_') + tail


def _evalgrid(fh, X, Y, tree=False):
    v = fh(X, Y)
    if np.isscalar(v) or np.ndim(v) == 0:
        v = float(v) * np.ones(X.shape)
    v = np.asarray(v, dtype=np.float64)
    if v.shape != X.shape:
        raise ValueError(_eid(tree, 'make_level:eval: coefficient function returned wrong size.'))
    if not np.all(np.isfinite(v)):
        raise ValueError(_eid(tree, 'make_level:eval: coefficient function returned non-finite values.'))
    return np.asfortranarray(v)


def _gauss_legendre(n):
    if n == 1:
        return np.array([0.0]), np.array([2.0])
    k = np.arange(1, n)
    beta = 0.5 / np.sqrt(1 - (2.0 * k) ** (-2))
    T = np.diag(beta, 1) + np.diag(beta, -1)
    d, V = np.linalg.eigh(T)
    idx = np.argsort(d)
    return d[idx], 2 * V[0, idx] ** 2


def _srcquad(fh, XC, YC, hx, hy, nq, tree=False):
    """``srcquad`` (``ebMakeLevel.m:108-131``)."""
    if nq <= 1:
        return _evalgrid(fh, XC, YC, tree)
    xi, w = _gauss_legendre(int(nq))
    w = w / 2
    out = np.zeros(XC.shape, order=F)
    for i in range(int(nq)):
        for j in range(int(nq)):
            out = out + (w[i] * w[j]) * _evalgrid(fh, XC + xi[i] * hx / 2, YC + xi[j] * hy / 2, tree)
    return out


def _bc_side(prob, side, xv, yv, isvert):
    """``bcSide`` (``ebMakeLevel.m:78-92``)."""
    bcs = prob.bc[side]
    if isvert:
        yv = np.asarray(yv, dtype=np.float64)
        g = bcs['g'](xv * np.ones(yv.shape), yv)
        nn = yv.size
    else:
        xv = np.asarray(xv, dtype=np.float64)
        g = bcs['g'](xv, yv * np.ones(xv.shape))
        nn = xv.size
    g = np.asarray(g, dtype=np.float64).reshape(-1)
    if g.size == 1 and nn != 1:
        g = g[0] * np.ones(nn)
    code = 1 if bcs['type'] == 'dirichlet' else 2
    return {'code': code, 'g': np.ascontiguousarray(g)}


def bc_fold(lev, p):
    """``ebBcFold`` (``ebBcFold.m:12-42``): Dirichlet +2D/h^2, Neumann -D/h^2."""
    bcd = lev.bc[p]
    CC = lev.CC[p]
    mx, my = CC.shape
    hx2 = lev.h[0] * lev.h[0]
    hy2 = lev.h[1] * lev.h[1]
    add = np.zeros((mx, my), order=F)
    DeW, DnS = lev.DeW[p], lev.DnS[p]
    if bcd[0]['code'] == 1:
        add[0, :] = add[0, :] + 2 * DeW[0, :] / hx2
    elif bcd[0]['code'] == 2:
        add[0, :] = add[0, :] - DeW[0, :] / hx2
    if bcd[1]['code'] == 1:
        add[mx - 1, :] = add[mx - 1, :] + 2 * DeW[mx, :] / hx2
    elif bcd[1]['code'] == 2:
        add[mx - 1, :] = add[mx - 1, :] - DeW[mx, :] / hx2
    if bcd[2]['code'] == 1:
        add[:, 0] = add[:, 0] + 2 * DnS[:, 0] / hy2
    elif bcd[2]['code'] == 2:
        add[:, 0] = add[:, 0] - DnS[:, 0] / hy2
    if bcd[3]['code'] == 1:
        add[:, my - 1] = add[:, my - 1] + 2 * DnS[:, my] / hy2
    elif bcd[3]['code'] == 2:
        add[:, my - 1] = add[:, my - 1] - DnS[:, my] / hy2
    return add


def _invdiags(lev, p):
    ID = invdiag2d(lev.DeW[p], lev.DnS[p], lev.CC[p], lev.h[0], lev.h[1])
    return np.asfortranarray(1.0 / (1.0 / ID + bc_fold(lev, p)))


# ---------------------------------------------------------------------------
def make_level(H, k, n, boxes, parents=None):
    """``ebMakeLevel`` (``ebMakeLevel.m:1-75``) / ``ebtMakeLevel`` (tree)."""
    prob = H.prob
    dom = prob.domain
    lev = Level()
    lev.n = [int(n[0]), int(n[1])]
    lev.h = [(dom[1] - dom[0]) / lev.n[0], (dom[3] - dom[2]) / lev.n[1]]
    boxes = np.asarray(boxes, dtype=np.int64).reshape(-1, 4)
    lev.np = boxes.shape[0]
    lev.box = boxes.copy()
    lev.sourceShift = 0.0
    if H.tree:
        lev.parent = (np.zeros(lev.np, dtype=np.int64) if parents is None
                      else np.asarray(parents, dtype=np.int64).reshape(-1))
        lev.mbounds = np.zeros((lev.np, 4), dtype=np.int64)
    pre = prob.get('prefetch') if isinstance(prob, dict) else None
    if callable(pre):
        # a problem whose coefficients share one costly point function (a
        # geometry's distance) takes every sample point of the level at once;
        # the per-patch evaluations below are unchanged
        sets = []
        hx, hy = lev.h
        for b in boxes:
            xf = dom[0] + np.arange(b[0] - 1, b[1] + 1) * hx
            yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * hy
            xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * hx
            yf = dom[2] + np.arange(b[2] - 1, b[3] + 1) * hy
            sets += [np.meshgrid(xf, yc, indexing='ij'), np.meshgrid(xc, yf, indexing='ij'),
                     np.meshgrid(xc, yc, indexing='ij')]
        pre(sets)
    for p in range(lev.np):
        b = [int(v) for v in boxes[p]]
        if (b[0] < 1 or b[0] > n[0] or b[1] < 1 or b[1] > n[0] or b[2] < 1 or b[2] > n[1]
                or b[3] < 1 or b[3] > n[1] or b[0] > b[1] or b[2] > b[3]):
            raise ValueError(_eid(H.tree, 'make_level:box: invalid patch box.'))
        if H.tree and k > 1:
            if b[0] % 2 != 1 or b[1] % 2 != 0 or b[2] % 2 != 1 or b[3] % 2 != 0:
                raise ValueError(f'ebt_make_level:align: patch {p+1} of level {k} not aligned to parent cells.')
            q = int(lev.parent[p])
            if q < 1 or q > H.lev[k - 1].np:
                raise ValueError(f'ebt_make_level:parent: patch {p+1} of level {k} has invalid parent index {q}.')
            qb = [int(v) for v in H.lev[k - 1].box[q - 1]]
            fp = [(b[0] + 1) // 2, b[1] // 2, (b[2] + 1) // 2, b[3] // 2]
            mb = [fp[0] - qb[0] + 1, fp[1] - qb[0] + 1, fp[2] - qb[2] + 1, fp[3] - qb[2] + 1]
            pmx, pmy = qb[1] - qb[0] + 1, qb[3] - qb[2] + 1
            if mb[0] < 1 or mb[1] > pmx or mb[2] < 1 or mb[3] > pmy:
                raise ValueError(f'ebt_make_level:containment: patch {p+1} of level {k} is not contained '
                                 f'in its parent patch {q} - single-parent lineage violated.')
            lev.mbounds[p] = mb
        mx, my = b[1] - b[0] + 1, b[3] - b[2] + 1
        lev.Q.append(np.zeros((mx + 2, my + 2), order=F))
        hx, hy = lev.h
        xf = dom[0] + np.arange(b[0] - 1, b[1] + 1) * hx
        yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * hy
        xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * hx
        yf = dom[2] + np.arange(b[2] - 1, b[3] + 1) * hy
        XF, YCF = np.meshgrid(xf, yc, indexing='ij')
        lev.DeW.append(_evalgrid(prob.D, XF, YCF, H.tree))
        XCF, YF = np.meshgrid(xc, yf, indexing='ij')
        lev.DnS.append(_evalgrid(prob.D, XCF, YF, H.tree))
        XC, YC = np.meshgrid(xc, yc, indexing='ij')
        lev.CC.append(_evalgrid(prob.C, XC, YC, H.tree))
        ft = _srcquad(prob.f, XC, YC, hx, hy, H.opts.SourceQuad, H.tree)
        lev.FTrue.append(ft)
        lev.F.append(ft.copy(order=F))
        if np.any(lev.DeW[p] <= 0) or np.any(lev.DnS[p] <= 0):
            raise ValueError(_eid(H.tree, 'make_level:D: D(x,y) must be strictly positive at faces.'))
        lev.par0.append((b[0] + b[2]) % 2)
        fint = (b[0] > 1, b[1] < n[0], b[2] > 1, b[3] < n[1])
        lev.faceInternal.append(fint)
        bcdat = [{'code': 0, 'g': None} for _ in range(4)]
        if not fint[0]:
            bcdat[0] = _bc_side(prob, 0, dom[0], yc, True)
        if not fint[1]:
            bcdat[1] = _bc_side(prob, 1, dom[1], yc, True)
        if not fint[2]:
            bcdat[2] = _bc_side(prob, 2, xc, dom[2], False)
        if not fint[3]:
            bcdat[3] = _bc_side(prob, 3, xc, dom[3], False)
        lev.bc.append(bcdat)
        lev.InvDiagS.append(None)
        lev.covered.append(np.zeros((mx, my), dtype=bool, order=F))
        lev.children.append([])
        lev.parents.append([])
        lev.cornerClass.append([1, 1, 1, 1])
        lev.land.append({'W': np.ones(my, np.int8), 'E': np.ones(my, np.int8),
                         'S': np.ones(mx, np.int8), 'N': np.ones(mx, np.int8)})
        lev.sameOps.append([])
        lev.ops.append(None)
        lev.cfD.append(None)
        lev.QC.append(np.zeros((mx // 2 + 2, my // 2 + 2), order=F) if k > 1 else None)
    for p in range(lev.np):
        lev.InvDiagS[p] = _invdiags(lev, p)
    return lev


# ---------------------------------------------------------------------------
def coeff_filldown(H):
    """``ebCoeffFilldown`` (``ebCoeffFilldown.m:8-56``) and the tree variant
    (``ebtCoeffFilldown.m:12-76``, including the shared-face push)."""
    for k in range(H.nlev, 1, -1):
        levF, levC = H.lev[k], H.lev[k - 1]
        if H.tree:
            OC = _owner_map(levC)
        for p in range(levF.np):
            b = [int(v) for v in levF.box[p]]
            mx, my = b[1] - b[0] + 1, b[3] - b[2] + 1
            DeW, DnS = levF.DeW[p], levF.DnS[p]
            cDeW = 0.5 * (DeW[0:mx + 1:2, 0:my - 1:2] + DeW[0:mx + 1:2, 1:my:2])
            cDnS = 0.5 * (DnS[0:mx - 1:2, 0:my + 1:2] + DnS[1:mx:2, 0:my + 1:2])
            cCC = restrict2(levF.CC[p])
            if H.tree:
                q = int(levF.parent[p])
                qb = [int(v) for v in levC.box[q - 1]]
                pmx, pmy = qb[1] - qb[0] + 1, qb[3] - qb[2] + 1
                Il, Ih, Jl, Jh = [int(v) for v in levF.mbounds[p]]
                levC.CC[q - 1][Il - 1:Ih, Jl - 1:Jh] = cCC
                levC.DeW[q - 1][Il - 1:Ih + 1, Jl - 1:Jh] = cDeW
                levC.DnS[q - 1][Il - 1:Ih, Jl - 1:Jh + 1] = cDnS
                if Il == 1 and qb[0] > 1:
                    _push_face_x(levC, OC, qb[0], range(qb[2] + Jl - 1, qb[2] + Jh), qb[0] - 1, cDeW[0, :])
                if Ih == pmx and qb[1] < levC.n[0]:
                    _push_face_x(levC, OC, qb[1] + 1, range(qb[2] + Jl - 1, qb[2] + Jh), qb[1] + 1, cDeW[-1, :])
                if Jl == 1 and qb[2] > 1:
                    _push_face_y(levC, OC, range(qb[0] + Il - 1, qb[0] + Ih), qb[2], qb[2] - 1, cDnS[:, 0])
                if Jh == pmy and qb[3] < levC.n[1]:
                    _push_face_y(levC, OC, range(qb[0] + Il - 1, qb[0] + Ih), qb[3] + 1, qb[3] + 1, cDnS[:, -1])
                continue
            Il, Ih, Jl, Jh = (b[0] + 1) // 2, b[1] // 2, (b[2] + 1) // 2, b[3] // 2
            for q in near_boxes(levC.box, [Il, Ih, Jl, Jh]):
                qb = [int(v) for v in levC.box[q]]
                r = rect_isect([Il, Ih, Jl, Jh], qb)
                if r is not None:
                    levC.CC[q][r[0] - qb[0]:r[1] - qb[0] + 1, r[2] - qb[2]:r[3] - qb[2] + 1] = \
                        cCC[r[0] - Il:r[1] - Il + 1, r[2] - Jl:r[3] - Jl + 1]
                rf = rect_isect([Il, Ih + 1, Jl, Jh], [qb[0], qb[1] + 1, qb[2], qb[3]])
                if rf is not None:
                    levC.DeW[q][rf[0] - qb[0]:rf[1] - qb[0] + 1, rf[2] - qb[2]:rf[3] - qb[2] + 1] = \
                        cDeW[rf[0] - Il:rf[1] - Il + 1, rf[2] - Jl:rf[3] - Jl + 1]
                rf = rect_isect([Il, Ih, Jl, Jh + 1], [qb[0], qb[1], qb[2], qb[3] + 1])
                if rf is not None:
                    levC.DnS[q][rf[0] - qb[0]:rf[1] - qb[0] + 1, rf[2] - qb[2]:rf[3] - qb[2] + 1] = \
                        cDnS[rf[0] - Il:rf[1] - Il + 1, rf[2] - Jl:rf[3] - Jl + 1]
    for k in range(1, H.nlev + 1):
        lev = H.lev[k]
        for p in range(lev.np):
            lev.InvDiagS[p] = _invdiags(lev, p)


def _push_face_x(levC, OC, faceG, jGs, nbrI, vals):
    jGs = list(jGs)
    own = np.array([OC[nbrI - 1, j - 1] for j in jGs], dtype=np.int64)
    for s in np.unique(own[own > 0]):
        ii = np.nonzero(own == s)[0]
        sb = [int(v) for v in levC.box[s - 1]]
        fl = faceG - sb[0] + 1
        for t in ii:
            levC.DeW[s - 1][fl - 1, jGs[t] - sb[2]] = vals[t]


def _push_face_y(levC, OC, iGs, faceG, nbrJ, vals):
    iGs = list(iGs)
    own = np.array([OC[i - 1, nbrJ - 1] for i in iGs], dtype=np.int64)
    for s in np.unique(own[own > 0]):
        ii = np.nonzero(own == s)[0]
        sb = [int(v) for v in levC.box[s - 1]]
        fl = faceG - sb[2] + 1
        for t in ii:
            levC.DnS[s - 1][iGs[t] - sb[0], fl - 1] = vals[t]


def _owner_map(lev):
    O = np.zeros((lev.n[0], lev.n[1]), dtype=np.int64, order=F)
    for q in range(lev.np):
        b = lev.box[q]
        O[b[0] - 1:b[1], b[2] - 1:b[3]] = q + 1
    return O


# ---------------------------------------------------------------------------
def _add_face_ops(same, levF, nb, gi, gj, dstAll):
    """``addFaceOps`` (``ebBuildOps.m:203-218``)."""
    idx = np.nonzero(nb > 0)[0]
    if idx.size == 0:
        return
    gi = np.broadcast_to(np.asarray(gi), nb.shape)
    gj = np.broadcast_to(np.asarray(gj), nb.shape)
    for s in np.unique(nb[idx]):
        ii = idx[nb[idx] == s]
        sb = levF.box[s - 1]
        msx = int(sb[1] - sb[0] + 1)
        src = sub2ind(msx + 2, gi[ii] - sb[0] + 2, gj[ii] - sb[2] + 2)
        same.append((int(s), np.asarray(src, np.int64), np.asarray(dstAll[ii], np.int64)))


def _landscape(H, k, p, OF):
    """Ghost classes, corner classes and same-level copies for patch p of
    level k (``ebBuildOps.m:47-113``; identical in ``ebtBuildOps.m:60-124``)."""
    levF = H.lev[k]
    nF = levF.n
    ilo, ihi, jlo, jhi = [int(v) for v in levF.box[p]]
    mx, my = ihi - ilo + 1, jhi - jlo + 1
    land = {'W': np.ones(my, np.int8), 'E': np.ones(my, np.int8),
            'S': np.ones(mx, np.int8), 'N': np.ones(mx, np.int8)}
    same = []
    gj = np.arange(jlo, jhi + 1)
    gi = np.arange(ilo, ihi + 1)
    if ilo > 1:
        nb = OF[ilo - 2, jlo - 1:jhi]
        land['W'][nb > 0] = 2
        land['W'][nb == 0] = 3
        _add_face_ops(same, levF, nb, ilo - 1, gj, sub2ind(mx + 2, np.ones(my, np.int64), np.arange(2, my + 2)))
    if ihi < nF[0]:
        nb = OF[ihi, jlo - 1:jhi]
        land['E'][nb > 0] = 2
        land['E'][nb == 0] = 3
        _add_face_ops(same, levF, nb, ihi + 1, gj,
                      sub2ind(mx + 2, (mx + 2) * np.ones(my, np.int64), np.arange(2, my + 2)))
    if jlo > 1:
        nb = OF[ilo - 1:ihi, jlo - 2]
        land['S'][nb > 0] = 2
        land['S'][nb == 0] = 3
        _add_face_ops(same, levF, nb, gi, jlo - 1, sub2ind(mx + 2, np.arange(2, mx + 2), np.ones(mx, np.int64)))
    if jhi < nF[1]:
        nb = OF[ilo - 1:ihi, jhi]
        land['N'][nb > 0] = 2
        land['N'][nb == 0] = 3
        _add_face_ops(same, levF, nb, gi, jhi + 1,
                      sub2ind(mx + 2, np.arange(2, mx + 2), (my + 2) * np.ones(mx, np.int64)))
    cdef = [(ilo - 1, jlo - 1, 1, 1), (ihi + 1, jlo - 1, mx + 2, 1),
            (ilo - 1, jhi + 1, 1, my + 2), (ihi + 1, jhi + 1, mx + 2, my + 2)]
    cclass = [1, 1, 1, 1]
    for c in range(4):
        cgi, cgj, li, lj = cdef[c]
        if cgi < 1 or cgi > nF[0] or cgj < 1 or cgj > nF[1]:
            cclass[c] = 1
        else:
            s = int(OF[cgi - 1, cgj - 1])
            if s > 0:
                cclass[c] = 2
                sb = levF.box[s - 1]
                msx = int(sb[1] - sb[0] + 1)
                same.append((s, np.array([sub2ind(msx + 2, cgi - sb[0] + 2, cgj - sb[2] + 2)], np.int64),
                             np.array([sub2ind(mx + 2, li, lj)], np.int64)))
            else:
                cclass[c] = 3
    levF.land[p] = land
    levF.cornerClass[p] = cclass
    levF.sameOps[p] = same
    return land


def _resolve_cells(levC, OC, gis, gjs, Il, Jl, cmx, cmy):
    """``resolveCells`` (``ebBuildOps.m:221-252``): for each ring cell its
    owning parent patch and the padded source / destination indices,
    grouped by parent in ascending order (cell order kept inside a group).
    The first offending cell raises, as the per-cell loop does."""
    nC = levC.n
    gi = np.asarray(gis, dtype=np.int64).ravel()
    gj = np.asarray(gjs, dtype=np.int64).ravel()
    if gi.size == 0:
        return []
    sp = OC[np.clip(gi, 1, nC[0]) - 1, np.clip(gj, 1, nC[1]) - 1].astype(np.int64)
    unc = sp == 0
    qb = np.asarray(levC.box, dtype=np.int64)[np.where(unc, 1, sp) - 1]
    li, lj = gi - qb[:, 0] + 2, gj - qb[:, 2] + 2
    mqx, mqy = qb[:, 1] - qb[:, 0] + 1, qb[:, 3] - qb[:, 2] + 1
    over = ~unc & ((li < 1) | (li > mqx + 2) | (lj < 1) | (lj > mqy + 2))
    bad = np.nonzero(unc | over)[0]
    if bad.size:
        t = int(bad[0])
        if unc[t]:
            raise ValueError(f'eb_build_ops:ring: parent cell ({gi[t]},{gj[t]}) not covered - proper nesting '
                             f'violated.')
        raise ValueError('eb_build_ops:overhang: ring cell overhang exceeds ghost ring.')
    src = sub2ind(mqx + 2, li, lj)
    dst = sub2ind(cmx + 2, gi - Il + 2, gj - Jl + 2)
    ops = []
    for q in np.unique(sp):
        ii = sp == q
        ops.append((int(q), src[ii], dst[ii]))
    return ops


def _corr_face(levC, OC, mask, gis, gjs, tree=False):
    """``corrFace`` (``ebBuildOps.m:255-281``)."""
    cs = {'mask': mask, 'ops': []}
    idx = np.nonzero(mask)[0]
    if idx.size == 0:
        return cs
    gi = np.broadcast_to(np.asarray(gis), mask.shape)[idx].astype(np.int64)
    gj = np.broadcast_to(np.asarray(gjs), mask.shape)[idx].astype(np.int64)
    dp = OC[gi - 1, gj - 1].astype(np.int64)
    if (dp == 0).any():
        raise ValueError(_eid(tree, 'build_ops:corr: mass-correction target cell uncovered.'))
    qb = np.asarray(levC.box, dtype=np.int64)[dp - 1]
    dst = sub2ind(qb[:, 1] - qb[:, 0] + 1, gi - qb[:, 0] + 1, gj - qb[:, 2] + 1)
    for q in np.unique(dp):
        ii = dp == q
        cs['ops'].append((int(q), idx[ii].astype(np.int64), dst[ii]))
    return cs


def build_ops(H, k):
    """``ebBuildOps`` (``ebBuildOps.m:17-200``) or ``ebtBuildOps`` (tree)."""
    levF, levC = H.lev[k], H.lev[k - 1]
    OF = _owner_map(levF)
    OC = _owner_map(levC)
    for p in range(levF.np):
        ilo, ihi, jlo, jhi = [int(v) for v in levF.box[p]]
        mx, my = ihi - ilo + 1, jhi - jlo + 1
        if ilo % 2 != 1 or ihi % 2 != 0 or jlo % 2 != 1 or jhi % 2 != 0:
            raise ValueError('eb_build_ops:align: patch not aligned to parent cells.')
        land = _landscape(H, k, p, OF)
        ops = {}
        if H.tree:
            q = int(levF.parent[p])
            Il, Ih, Jl, Jh = [int(v) for v in levF.mbounds[p]]
            cmx, cmy = Ih - Il + 1, Jh - Jl + 1
            if cmx != mx // 2 or cmy != my // 2:
                raise ValueError('ebt_build_ops:mbounds: mbounds inconsistent with patch size.')
            ops['sp'] = q
            ops['win'] = [Il, Ih + 2, Jl, Jh + 2]
            ops['tree'] = True
            fpg = [(ilo + 1) // 2, ihi // 2, (jlo + 1) // 2, jhi // 2]
            ops['corrW'] = _corr_face(levC, OC, land['W'][1::2] == 3, fpg[0] - 1, np.arange(fpg[2], fpg[3] + 1), True)
            ops['corrE'] = _corr_face(levC, OC, land['E'][1::2] == 3, fpg[1] + 1, np.arange(fpg[2], fpg[3] + 1), True)
            ops['corrS'] = _corr_face(levC, OC, land['S'][1::2] == 3, np.arange(fpg[0], fpg[1] + 1), fpg[2] - 1, True)
            ops['corrN'] = _corr_face(levC, OC, land['N'][1::2] == 3, np.arange(fpg[0], fpg[1] + 1), fpg[3] + 1, True)
            levF.ops[p] = ops
            continue
        Il, Ih, Jl, Jh = (ilo + 1) // 2, ihi // 2, (jlo + 1) // 2, jhi // 2
        cmx, cmy = Ih - Il + 1, Jh - Jl + 1
        ringGi = np.concatenate([(Il - 1) * np.ones(cmy + 2, np.int64), (Ih + 1) * np.ones(cmy + 2, np.int64),
                                 np.arange(Il, Ih + 1), np.arange(Il, Ih + 1)])
        ringGj = np.concatenate([np.arange(Jl - 1, Jh + 2), np.arange(Jl - 1, Jh + 2),
                                 (Jl - 1) * np.ones(cmx, np.int64), (Jh + 1) * np.ones(cmx, np.int64)])
        ops['ring'] = _resolve_cells(levC, OC, ringGi, ringGj, Il, Jl, cmx, cmy)
        ops['winrect'] = []
        ncov = sum(len(t[2]) for t in ops['ring'])
        for q in near_boxes(levC.box, [Il, Ih, Jl, Jh]):
            qb = [int(v) for v in levC.box[q]]
            r = rect_isect([Il, Ih, Jl, Jh], qb)
            if r is None:
                continue
            ops['winrect'].append((q + 1, [r[0] - qb[0] + 2, r[1] - qb[0] + 2, r[2] - qb[2] + 2, r[3] - qb[2] + 2],
                                   [r[0] - Il + 2, r[1] - Il + 2, r[2] - Jl + 2, r[3] - Jl + 2]))
            ncov += (r[1] - r[0] + 1) * (r[3] - r[2] + 1)
        if ncov != (cmx + 2) * (cmy + 2):
            raise ValueError(f'eb_build_ops:nesting: patch {p+1} at level {k}: parent window not fully covered '
                             f'({ncov} of {(cmx+2)*(cmy+2)}) - proper nesting violated.')
        ops['usc'], ops['fsc'] = [], []
        for q in near_boxes(levC.box, [Il, Ih, Jl, Jh]):
            qb = [int(v) for v in levC.box[q]]
            r = rect_isect([Il, Ih, Jl, Jh], qb)
            if r is None:
                continue
            sr = [r[0] - Il + 1, r[1] - Il + 1, r[2] - Jl + 1, r[3] - Jl + 1]
            ops['usc'].append((q + 1, sr, [r[0] - qb[0] + 2, r[1] - qb[0] + 2, r[2] - qb[2] + 2, r[3] - qb[2] + 2]))
            ops['fsc'].append((q + 1, sr, [r[0] - qb[0] + 1, r[1] - qb[0] + 1, r[2] - qb[2] + 1, r[3] - qb[2] + 1]))
        ops['corrW'] = _corr_face(levC, OC, land['W'][1::2] == 3, Il - 1, np.arange(Jl, Jh + 1))
        ops['corrE'] = _corr_face(levC, OC, land['E'][1::2] == 3, Ih + 1, np.arange(Jl, Jh + 1))
        ops['corrS'] = _corr_face(levC, OC, land['S'][1::2] == 3, np.arange(Il, Ih + 1), Jl - 1)
        ops['corrN'] = _corr_face(levC, OC, land['N'][1::2] == 3, np.arange(Il, Ih + 1), Jh + 1)
        ops['tree'] = False
        levF.ops[p] = ops

    # children / parents bookkeeping and covered masks
    if H.tree:
        for q in range(levC.np):
            levC.children[q] = []
            qb = levC.box[q]
            levC.covered[q] = np.zeros((int(qb[1] - qb[0] + 1), int(qb[3] - qb[2] + 1)), dtype=bool, order=F)
        for p in range(levF.np):
            q = int(levF.parent[p])
            mb = levF.mbounds[p]
            levC.children[q - 1].append(p + 1)
            levC.covered[q - 1][mb[0] - 1:mb[1], mb[2] - 1:mb[3]] = True
        return
    fboxes = np.asarray(levF.box).reshape(-1, 4).astype(np.int64)
    fps = np.stack([(fboxes[:, 0] + 1) // 2, fboxes[:, 1] // 2, (fboxes[:, 2] + 1) // 2, fboxes[:, 3] // 2], axis=1)
    for q in range(levC.np):
        levC.children[q] = []
        qb = [int(v) for v in levC.box[q]]
        cov = np.zeros((qb[1] - qb[0] + 1, qb[3] - qb[2] + 1), dtype=bool, order=F)
        for p in near_boxes(fps, qb, pad=0):
            fp = [int(v) for v in fps[p]]
            r = rect_isect(fp, qb)
            if r is not None:
                levC.children[q].append(p + 1)
                cov[r[0] - qb[0]:r[1] - qb[0] + 1, r[2] - qb[2]:r[3] - qb[2] + 1] = True
        levC.covered[q] = cov
    for p in range(levF.np):
        b = levF.box[p]
        fp = [(int(b[0]) + 1) // 2, int(b[1]) // 2, (int(b[2]) + 1) // 2, int(b[3]) // 2]
        levF.parents[p] = [q + 1 for q in near_boxes(levC.box, fp, pad=0)
                           if rect_isect(fp, list(levC.box[q])) is not None]


# ---------------------------------------------------------------------------
def parent_coeffs(H, k, p):
    """``ebParentCoeffs`` (``ebParentCoeffs.m:1-31``) / ``ebtParentCoeffs``:
    the parent coefficients over the footprint of patch p of level k."""
    levF, levC = H.lev[k], H.lev[k - 1]
    b = levF.box[p]
    cmx, cmy = int(b[1] - b[0] + 1) // 2, int(b[3] - b[2] + 1) // 2
    if H.tree:
        q = int(levF.parent[p]) - 1
        Il, Ih, Jl, Jh = [int(v) for v in levF.mbounds[p]]
        PDeW = levC.DeW[q][Il - 1:Ih + 1, Jl - 1:Jh].copy(order=F)
        PDnS = levC.DnS[q][Il - 1:Ih, Jl - 1:Jh + 1].copy(order=F)
        PCC = levC.CC[q][Il - 1:Ih, Jl - 1:Jh].copy(order=F)
        return PDeW, PDnS, PCC
    Il, Ih, Jl, Jh = (int(b[0]) + 1) // 2, int(b[1]) // 2, (int(b[2]) + 1) // 2, int(b[3]) // 2
    PDeW = np.full((cmx + 1, cmy), np.nan, order=F)
    PDnS = np.full((cmx, cmy + 1), np.nan, order=F)
    PCC = np.full((cmx, cmy), np.nan, order=F)
    for q in near_boxes(levC.box, [Il, Ih, Jl, Jh]):
        qb = [int(v) for v in levC.box[q]]
        r = rect_isect([Il, Ih, Jl, Jh], qb)
        if r is not None:
            PCC[r[0] - Il:r[1] - Il + 1, r[2] - Jl:r[3] - Jl + 1] = \
                levC.CC[q][r[0] - qb[0]:r[1] - qb[0] + 1, r[2] - qb[2]:r[3] - qb[2] + 1]
        rf = rect_isect([Il, Ih + 1, Jl, Jh], [qb[0], qb[1] + 1, qb[2], qb[3]])
        if rf is not None:
            PDeW[rf[0] - Il:rf[1] - Il + 1, rf[2] - Jl:rf[3] - Jl + 1] = \
                levC.DeW[q][rf[0] - qb[0]:rf[1] - qb[0] + 1, rf[2] - qb[2]:rf[3] - qb[2] + 1]
        rf = rect_isect([Il, Ih, Jl, Jh + 1], [qb[0], qb[1], qb[2], qb[3] + 1])
        if rf is not None:
            PDnS[rf[0] - Il:rf[1] - Il + 1, rf[2] - Jl:rf[3] - Jl + 1] = \
                levC.DnS[q][rf[0] - qb[0]:rf[1] - qb[0] + 1, rf[2] - qb[2]:rf[3] - qb[2] + 1]
    return PDeW, PDnS, PCC


def gather_parent_coeffs(H):
    """``ebGatherParentCoeffs`` (``ebGatherParentCoeffs.m:12-63``): interface
    face diffusivities ``cfD`` per patch (W/E/S/N)."""
    for k in range(2, H.nlev + 1):
        levF = H.lev[k]
        for p in range(levF.np):
            PDeW, PDnS, _ = parent_coeffs(H, k, p)
            if np.any(np.isnan(PDeW)) or np.any(np.isnan(PDnS)):
                if H.tree:
                    raise ValueError(f'ebt_gather_parent_coeffs:size: parent coefficient window of patch {p+1} '
                                     f'level {k} has wrong size.')
                raise ValueError(f'eb_gather_parent_coeffs:cover: footprint of patch {p+1} level {k} '
                                 f'not covered by parent level.')
            levF.cfD[p] = {'W': PDeW[0, :].copy(), 'E': PDeW[-1, :].copy(),
                           'S': PDnS[:, 0].copy(), 'N': PDnS[:, -1].copy()}


# ---------------------------------------------------------------------------
def coarsest_assemble(H):
    """``ebCoarsest('assemble')`` (``ebCoarsest.m:14-77``).

    Builds the ghost-eliminated 5-point operator of level 1 and its boundary
    right-hand side.  The factorisation used by the device is the explicit
    inverse (``Ainv``), so that each coarsest solve is one dense
    matrix-vector product with a fixed summation order shared by the device
    kernel and the CPU oracle; the singular all-Neumann, C == 0 case keeps
    the reference's one-row/one-column KKT augmentation and stores the
    leading N x N block of the augmented inverse.
    """
    lev = H.lev[1]
    n1, n2 = lev.n
    N = n1 * n2
    if N > 16384:
        raise ValueError(f'eb_coarsest:size: coarsest level has {N} unknowns; the device coarsest solve '
                         f'supports at most 16384 (raise CoarsestCells or use even BaseCells).')
    hx, hy = lev.h
    hx2, hy2 = hx * hx, hy * hy
    DeW, DnS, CC = lev.DeW[0], lev.DnS[0], lev.CC[0]
    bcd = lev.bc[0]
    A = np.zeros((N, N))
    idx = np.arange(N).reshape((n1, n2), order=F)
    A[idx.ravel(order=F), idx.ravel(order=F)] += CC.ravel(order=F)
    bcRhs = np.zeros(N)
    c = DeW[1:n1, :] / hx2
    iL, iR = idx[0:n1 - 1, :], idx[1:n1, :]
    np.add.at(A, (iL.ravel(F), iL.ravel(F)), c.ravel(F))
    np.add.at(A, (iR.ravel(F), iR.ravel(F)), c.ravel(F))
    np.add.at(A, (iL.ravel(F), iR.ravel(F)), -c.ravel(F))
    np.add.at(A, (iR.ravel(F), iL.ravel(F)), -c.ravel(F))
    c = DnS[:, 1:n2] / hy2
    iL, iR = idx[:, 0:n2 - 1], idx[:, 1:n2]
    np.add.at(A, (iL.ravel(F), iL.ravel(F)), c.ravel(F))
    np.add.at(A, (iR.ravel(F), iR.ravel(F)), c.ravel(F))
    np.add.at(A, (iL.ravel(F), iR.ravel(F)), -c.ravel(F))
    np.add.at(A, (iR.ravel(F), iL.ravel(F)), -c.ravel(F))

    def bface(code, d, g, i1, i2, h, h2):
        if code == 1:
            np.add.at(A, (i1, i1), 3 * d / h2)
            np.add.at(A, (i1, i2), -d / (3 * h2))
            np.add.at(bcRhs, i1, (8 / 3) * d * g / h2)
        elif code == 2:
            np.add.at(bcRhs, i1, d * g / h)

    bface(bcd[0]['code'], DeW[0, :], bcd[0]['g'], idx[0, :], idx[1, :], hx, hx2)
    bface(bcd[1]['code'], DeW[n1, :], bcd[1]['g'], idx[n1 - 1, :], idx[n1 - 2, :], hx, hx2)
    bface(bcd[2]['code'], DnS[:, 0], bcd[2]['g'], idx[:, 0], idx[:, 1], hy, hy2)
    bface(bcd[3]['code'], DnS[:, n2], bcd[3]['g'], idx[:, n2 - 1], idx[:, n2 - 2], hy, hy2)

    allneu = all(s['code'] != 1 for s in bcd)
    cmax = 0.0
    for k in range(1, H.nlev + 1):
        for p in range(H.lev[k].np):
            cmax = max(cmax, float(np.max(np.abs(H.lev[k].CC[p]))))
    singular = allneu and cmax == 0
    if singular:
        e = np.ones((N, 1))
        K = np.block([[A, e], [e.T, np.zeros((1, 1))]])
        Ainv = dense_inverse(K)[:N, :N]
    else:
        Ainv = dense_inverse(A)
    H.coarsest = {'singular': bool(singular), 'bcRhs': bcRhs, 'Ainv': np.ascontiguousarray(Ainv), 'A': A}


_INV_LOCK = threading.Lock()
_INV_CACHE = OrderedDict()


def dense_inverse(A):
    """np.linalg.inv of the coarsest operator, memoised by the matrix's
    bytes (a rebuilt hierarchy with the same coarsest coefficients -- every
    regrid of a time-independent problem, every served request of one recipe
    -- gets the very same inverse without recomputing it) and serialised: the
    threaded BLAS behind it stalled for about a second whenever two host
    threads entered it at once."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    key = (A.shape, hashlib.sha1(A.tobytes()).digest())
    with _INV_LOCK:
        hit = _INV_CACHE.get(key)
        if hit is not None and np.array_equal(hit[0], A):
            _INV_CACHE.move_to_end(key)
            return hit[1].copy()
        inv = np.linalg.inv(A)
        _INV_CACHE[key] = (A.copy(), inv.copy())
        while len(_INV_CACHE) > 16:
            _INV_CACHE.popitem(last=False)
    return inv


def compat_project(H):
    """``ebCompatProject`` (``ebCompatProject.m:33-111``)."""
    if not H.coarsest:
        return
    if not H.coarsest['singular']:
        for k in range(1, H.nlev + 1):
            lev = H.lev[k]
            old = lev.sourceShift
            if old == 0:
                continue
            for p in range(lev.np):
                lev.FTrue[p] = lev.FTrue[p] + old
                lev.F[p] = lev.FTrue[p].copy(order=F)
            lev.sourceShift = 0.0
        H.compatibility = {'sourceShift': 0.0, 'unprojectedDefect': 0.0}
        return
    S = Av = R = 0.0
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        old = lev.sourceShift
        hx, hy = lev.h
        da = hx * hy
        for p in range(lev.np):
            cov = lev.covered[p]
            vis = ~cov
            S = S + (np.sum(lev.FTrue[p][vis]) + old * np.count_nonzero(vis)) * da
            Av = Av + np.count_nonzero(vis) * da
            mx, my = cov.shape
            bcd = lev.bc[p]
            if bcd[0]['code'] == 2:
                m = ~cov[0, :]
                R = R + np.sum((lev.DeW[p][0, :] * bcd[0]['g'])[m]) * hy
            if bcd[1]['code'] == 2:
                m = ~cov[mx - 1, :]
                R = R + np.sum((lev.DeW[p][mx, :] * bcd[1]['g'])[m]) * hy
            if bcd[2]['code'] == 2:
                m = ~cov[:, 0]
                R = R + np.sum((lev.DnS[p][:, 0] * bcd[2]['g'])[m]) * hx
            if bcd[3]['code'] == 2:
                m = ~cov[:, my - 1]
                R = R + np.sum((lev.DnS[p][:, my] * bcd[3]['g'])[m]) * hx
    c = (S + R) / max(Av, np.finfo(float).tiny)
    for k in range(1, H.nlev + 1):
        lev = H.lev[k]
        old = lev.sourceShift
        for p in range(lev.np):
            lev.FTrue[p] = lev.FTrue[p] - (c - old)
            lev.F[p] = lev.FTrue[p].copy(order=F)
        lev.sourceShift = c
    H.compatibility = {'sourceShift': c, 'unprojectedDefect': S + R}


# ---------------------------------------------------------------------------
def setup(prob, opts, backend, tree=False):
    """``ebSetup`` (``ebSetup.m:10-69``) / ``ebtSetup``."""
    H = Hierarchy(prob, opts, tree=tree)
    n0 = list(opts.BaseCells)
    sizes = [n0]
    ns = list(n0)
    while all(v % 2 == 0 for v in ns) and min(ns) / 2 >= 4 and min(ns) > opts.CoarsestCells:
        ns = [v // 2 for v in ns]
        sizes.insert(0, ns)
    H.rootIdx = len(sizes)
    H.nlev = H.rootIdx
    for k in range(1, H.nlev + 1):
        sz = sizes[k - 1]
        par = [1] if (tree and k > 1) else None
        H.lev.append(make_level(H, k, sz, [[1, sz[0], 1, sz[1]]], par))
    coeff_filldown(H)
    for k in range(2, H.nlev + 1):
        build_ops(H, k)
    gather_parent_coeffs(H)
    ig = opts.InitialGuess
    if ig is not None:
        dom = prob.domain
        for k in range(1, H.nlev + 1):
            lev = H.lev[k]
            for p in range(lev.np):
                b = lev.box[p]
                xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0]
                yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1]
                XC, YC = np.meshgrid(xc, yc, indexing='ij')
                lev.Q[p][1:-1, 1:-1] = ig(XC, YC)
    coarsest_assemble(H)
    H.touch()
    backend.run(H, [('fill', k) for k in range(1, H.nlev + 1)])
    compat_project(H)
    H.touch()
    return H


def add_level(H, boxes, backend):
    """``ebAddLevel`` (``ebAddLevel.m:6-32``) / ``ebtAddLevel`` (boxes carry
    the parent index in column 0 for the tree form)."""
    kNew = H.nlev + 1
    nNew = [2 * v for v in H.lev[H.nlev].n]
    boxes = np.asarray(boxes, dtype=np.int64)
    if H.tree:
        parents = boxes[:, 0]
        cb = boxes[:, 1:5]
    else:
        parents = None
        cb = boxes
    fineBoxes = np.stack([2 * cb[:, 0] - 1, 2 * cb[:, 1], 2 * cb[:, 2] - 1, 2 * cb[:, 3]], axis=1)
    H.nlev = kNew
    H.lev.append(make_level(H, kNew, nNew, fineBoxes, parents))
    coeff_filldown(H)
    build_ops(H, kNew)
    gather_parent_coeffs(H)
    coarsest_assemble(H)
    compat_project(H)
    H.touch()
    backend.run(H, [('fill', kNew - 1), ('prolong', kNew), ('fill', kNew)])
    if H.opts.Verbose >= 1:
        lev = H.lev[kNew]
        ncell = sum(f.size for f in lev.F)
        tag = '[ebtsam]' if H.tree else '[ebsam]'
        print(f'{tag} added level {kNew - H.rootIdx + 1} ({lev.np} patch(es), {ncell} cells, h = {lev.h[0]:.3e})')
    return H
