"""Tagging and Berger-Rigoutsos clustering (host, integer-exact).

Restates ``EllipticBSAM/src/ebTagCluster.m:24-380`` (QC-ring: one global
clustering) and ``EllipticBSAMTree/src/ebtTagCluster.m`` (tree: the same
clustering run inside every patch of the finest level, global buffering).
The box order produced here is the reference's order (explicit LIFO stacks,
first-minimum tie breaks, stable sorts), because patch numbering fixes the
order of the flux-correction sums downstream.

Boxes are 1-based ``[ilo ihi jlo jhi]`` in the finest level's index space.
"""
from __future__ import annotations

import inspect
import warnings

import numpy as np

from .hierarchy import op2d, restrict2


def _nargin(fn):
    """Number of positional parameters (MATLAB ``nargin(fh)``)."""
    try:
        ps = inspect.signature(fn).parameters.values()
    except (TypeError, ValueError):
        return 2
    if any(p.kind == p.VAR_POSITIONAL for p in ps):
        return 3
    return sum(1 for p in ps if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD))


def _dilate(M, b):
    """``dilate`` (``ebTagCluster.m:113-127``)."""
    if b <= 0:
        return M
    n1, n2 = M.shape
    P = np.zeros((n1 + 2 * b, n2 + 2 * b), dtype=bool)
    P[b:b + n1, b:b + n2] = M
    acc = np.zeros((n1, n2), dtype=bool)
    for dx in range(-b, b + 1):
        for dy in range(-b, b + 1):
            acc |= P[b + dx:b + n1 + dx, b + dy:b + n2 + dy]
    return acc


def _erode8(Cm):
    """``erode8`` (``ebTagCluster.m:130-141``)."""
    n1, n2 = Cm.shape
    P = np.ones((n1 + 2, n2 + 2), dtype=bool)
    P[1:n1 + 1, 1:n2 + 1] = Cm
    A = np.ones((n1, n2), dtype=bool)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            A &= P[1 + dx:n1 + 1 + dx, 1 + dy:n2 + 1 + dy]
    return A


def _tight_bbox(T, bb):
    sub = T[bb[0] - 1:bb[1], bb[2] - 1:bb[3]]
    rows = np.any(sub, axis=1)
    cols = np.any(sub, axis=0)
    if not rows.any():
        return None
    ri = np.nonzero(rows)[0]
    ci = np.nonzero(cols)[0]
    return [bb[0] + int(ri[0]), bb[0] + int(ri[-1]), bb[2] + int(ci[0]), bb[2] + int(ci[-1])]


def _pick_split(sig, minW):
    """``pickSplit`` (``ebTagCluster.m:211-236``); returns (s, quality)."""
    n = len(sig)
    holes = np.nonzero(sig == 0)[0] + 1
    holes = holes[(holes > minW) & (holes <= n - minW)]
    if holes.size:
        ii = int(np.argmin(np.abs(holes - n / 2)))
        return int(holes[ii]), 2
    if n < 2 * minW:
        return 0, 0
    sig = sig.astype(np.int64)
    d2 = sig[2:n] - 2 * sig[1:n - 1] + sig[0:n - 2]      # d2[t] <-> MATLAB d2(t+1)
    best = -1
    s = 0
    for i in range(2, n - 1):                              # MATLAB i = 2:len-2
        j = abs(int(d2[i - 1]) - int(d2[i - 2]))
        cut = i
        if cut >= minW and (n - cut) >= minW and j > best:
            best = j
            s = cut
    return s, (1 if s > 0 else 0)


def _br_cluster(T, minW, eff):
    """``brCluster`` (``ebTagCluster.m:144-198``)."""
    out = []
    stack = [_tight_bbox(T, [1, T.shape[0], 1, T.shape[1]])]
    while stack:
        bb = stack.pop()
        if bb is None:
            continue
        bb = _tight_bbox(T, bb)
        if bb is None:
            continue
        w = [bb[1] - bb[0] + 1, bb[3] - bb[2] + 1]
        sub = T[bb[0] - 1:bb[1], bb[2] - 1:bb[3]]
        fill = np.count_nonzero(sub) / sub.size
        if fill >= eff or (w[0] <= minW and w[1] <= minW):
            out.append(bb)
            continue
        sigx = sub.sum(axis=1)
        sigy = sub.sum(axis=0)
        sx, qx = _pick_split(sigx, minW)
        sy, qy = _pick_split(sigy, minW)
        if qx == 0 and qy == 0:
            if w[0] >= 2 * minW or w[1] >= 2 * minW:
                if w[0] >= w[1]:
                    s = w[0] // 2
                    stack.append([bb[0], bb[0] + s - 1, bb[2], bb[3]])
                    stack.append([bb[0] + s, bb[1], bb[2], bb[3]])
                else:
                    s = w[1] // 2
                    stack.append([bb[0], bb[1], bb[2], bb[2] + s - 1])
                    stack.append([bb[0], bb[1], bb[2] + s, bb[3]])
            else:
                out.append(bb)
            continue
        usex = qx > qy or (qx == qy and w[0] >= w[1])
        if qx == 0:
            usex = False
        if qy == 0:
            usex = True
        if usex:
            stack.append([bb[0], bb[0] + sx - 1, bb[2], bb[3]])
            stack.append([bb[0] + sx, bb[1], bb[2], bb[3]])
        else:
            stack.append([bb[0], bb[1], bb[2], bb[2] + sy - 1])
            stack.append([bb[0], bb[1], bb[2] + sy, bb[3]])
    return out


def _clip_allowed(boxes, T, allowed):
    """``clipAllowed`` (``ebTagCluster.m:239-264``)."""
    out = []
    stack = [list(b) for b in boxes]
    while stack:
        bb = stack.pop()
        sub = T[bb[0] - 1:bb[1], bb[2] - 1:bb[3]]
        if not sub.any():
            continue
        ok = allowed[bb[0] - 1:bb[1], bb[2] - 1:bb[3]]
        if ok.all():
            out.append(bb)
            continue
        w = [bb[1] - bb[0] + 1, bb[3] - bb[2] + 1]
        if w[0] >= w[1]:
            s = w[0] // 2
            stack.append([bb[0], bb[0] + s - 1, bb[2], bb[3]])
            stack.append([bb[0] + s, bb[1], bb[2], bb[3]])
        else:
            s = w[1] // 2
            stack.append([bb[0], bb[1], bb[2], bb[2] + s - 1])
            stack.append([bb[0], bb[1], bb[2] + s, bb[3]])
    return out


def _strip_ok(boxes, allowed, b, dim, pos):
    """``stripOk`` (``ebTagCluster.m:359-380``)."""
    bb = boxes[b]
    if dim == 0:
        strip = allowed[pos - 1, bb[2] - 1:bb[3]]
        s = [pos, pos, bb[2], bb[3]]
    else:
        strip = allowed[bb[0] - 1:bb[1], pos - 1]
        s = [bb[0], bb[1], pos, pos]
    if not strip.all():
        return False
    for o, ob in enumerate(boxes):
        if o == b:
            continue
        if s[0] <= ob[1] and s[1] >= ob[0] and s[2] <= ob[3] and s[3] >= ob[2]:
            return False
    return True


def _grow_min(boxes, allowed, minW, n):
    """``growMin`` (``ebTagCluster.m:267-297``)."""
    boxes = [list(b) for b in boxes]
    for b in range(len(boxes)):
        for dim in range(2):
            lo, hi = boxes[b][2 * dim], boxes[b][2 * dim + 1]
            nd = n[dim]
            side = 0
            while hi - lo + 1 < minW:
                grown = False
                for tryside in (side, 1 - side):
                    if tryside == 0 and lo > 1:
                        if _strip_ok(boxes, allowed, b, dim, lo - 1):
                            lo -= 1
                            grown = True
                            break
                    elif tryside == 1 and hi < nd:
                        if _strip_ok(boxes, allowed, b, dim, hi + 1):
                            hi += 1
                            grown = True
                            break
                if not grown:
                    break
                side = 1 - side
            boxes[b][2 * dim], boxes[b][2 * dim + 1] = lo, hi
    return boxes


def _merge_or_drop_thin(boxes, allowed, tree=False):
    """``mergeOrDropThin`` (``ebTagCluster.m:299-356``)."""
    boxes = [list(b) for b in boxes]

    def thin(bb):
        return (bb[1] - bb[0] + 1 < 2) or (bb[3] - bb[2] + 1 < 2)

    b = 0
    while b < len(boxes):
        if not thin(boxes[b]):
            b += 1
            continue
        merged = False
        nb = len(boxes)
        areab = (boxes[b][1] - boxes[b][0] + 1) * (boxes[b][3] - boxes[b][2] + 1)
        ua = np.full(nb, np.inf)
        for o in range(nb):
            if o == b:
                continue
            u = [min(boxes[b][0], boxes[o][0]), max(boxes[b][1], boxes[o][1]),
                 min(boxes[b][2], boxes[o][2]), max(boxes[b][3], boxes[o][3])]
            ua[o] = (u[1] - u[0] + 1) * (u[3] - u[2] + 1)
        order = np.argsort(ua, kind='stable')
        for o in order:
            o = int(o)
            if o == b or not np.isfinite(ua[o]):
                continue
            sb, ob = boxes[b], boxes[o]
            if not (sb[0] - 1 <= ob[1] and sb[1] + 1 >= ob[0] and sb[2] - 1 <= ob[3] and sb[3] + 1 >= ob[2]):
                continue
            u = [min(sb[0], ob[0]), max(sb[1], ob[1]), min(sb[2], ob[2]), max(sb[3], ob[3])]
            areao = (ob[1] - ob[0] + 1) * (ob[3] - ob[2] + 1)
            if ua[o] > 1.5 * (areab + areao):
                continue
            if not allowed[u[0] - 1:u[1], u[2] - 1:u[3]].all():
                continue
            clash = False
            for t in range(nb):
                if t == b or t == o:
                    continue
                tb = boxes[t]
                if u[0] <= tb[1] and u[1] >= tb[0] and u[2] <= tb[3] and u[3] >= tb[2]:
                    clash = True
                    break
            if clash:
                continue
            boxes[o] = u
            del boxes[b]
            merged = True
            break
        if not merged:
            warnings.warn(('ebt' if tree else 'eb') + '_tag_cluster:dropthin: dropping an ungrowable sliver '
                          'cluster box (less local refinement)', RuntimeWarning, stacklevel=2)
            del boxes[b]
    return boxes


def rte_indicator(H, k, p):
    """``ebRte`` (``EllipticBSAM/src/ebRte.m:14-41``)."""
    lev = H.lev[k]
    Q = lev.Q[p]
    mx, my = Q.shape[0] - 2, Q.shape[1] - 2
    cmx, cmy = mx // 2, my // 2
    hx, hy = lev.h
    Lh = op2d(Q, lev.DeW[p], lev.DnS[p], lev.CC[p], hx, hy)
    RLh = restrict2(Lh)
    Rpad = np.zeros((cmx + 2, cmy + 2), order='F')
    Rpad[1:-1, 1:-1] = restrict2(Q[1:-1, 1:-1])
    j = np.arange(1, cmy + 1)
    Rpad[0, j] = 0.5 * (Q[0, 2 * j - 1] + Q[0, 2 * j])
    Rpad[cmx + 1, j] = 0.5 * (Q[mx + 1, 2 * j - 1] + Q[mx + 1, 2 * j])
    i = np.arange(1, cmx + 1)
    Rpad[i, 0] = 0.5 * (Q[2 * i - 1, 0] + Q[2 * i, 0])
    Rpad[i, cmy + 1] = 0.5 * (Q[2 * i - 1, my + 1] + Q[2 * i, my + 1])
    DeW, DnS = lev.DeW[p], lev.DnS[p]
    cDeW = 0.5 * (DeW[0:mx + 1:2, 0:my - 1:2] + DeW[0:mx + 1:2, 1:my:2])
    cDnS = 0.5 * (DnS[0:mx - 1:2, 0:my + 1:2] + DnS[1:mx:2, 0:my + 1:2])
    cCC = restrict2(lev.CC[p])
    tau = op2d(Rpad, cDeW, cDnS, cCC, 2 * hx, 2 * hy) - RLh
    return np.repeat(np.repeat(np.abs(tau), 2, axis=0), 2, axis=1)


def tag_cluster(H, backend=None):
    """``ebTagCluster`` / ``ebtTagCluster``: boxes (nb x 4, or nb x 5 with the
    1-based parent index first for the tree form) for a new finest level.
    With a device backend the solution-driven indicators ('ulap', 'rte')
    and the buffering run on the GPU, where the solution is, and only the
    tag mask comes back."""
    opts = H.opts
    k = H.nlev
    lev = H.lev[k]
    n = lev.n
    T = np.zeros((n[0], n[1]), dtype=bool)
    dom = H.prob.domain
    ind = str(opts.Indicator).lower()
    device = backend is not None and hasattr(backend, 'tag_mask') and ind in ('ulap', 'rte') and \
        not (ind == 'rte' and k == 1)
    if device:
        thr = opts.TagThreshold
        if callable(thr):
            thr = thr(k - H.rootIdx + 1)
        T = backend.tag_mask(H, ind, float(thr), int(opts.TagBuffer))
    for p in range(0 if device else lev.np):
        b = [int(v) for v in lev.box[p]]
        if ind == 'fun':
            if opts.TagFunction is None:
                raise ValueError(('ebt' if H.tree else 'eb') + '_tag_cluster:tagfun: Indicator=fun needs TagFunction.')
            xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0]
            yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1]
            XC, YC = np.meshgrid(xc, yc, indexing='ij')
            if _nargin(opts.TagFunction) >= 3:
                tp = np.asarray(opts.TagFunction(XC, YC, k - H.rootIdx + 1), dtype=bool)
            else:
                tp = np.asarray(opts.TagFunction(XC, YC), dtype=bool)
        elif ind == 'ulap':
            Q = lev.Q[p]
            mx, my = b[1] - b[0] + 1, b[3] - b[2] + 1
            sdx = (Q[2:mx + 2, 1:my + 1] - 2 * Q[1:mx + 1, 1:my + 1]) + Q[0:mx, 1:my + 1]
            sdy = (Q[1:mx + 1, 2:my + 2] - 2 * Q[1:mx + 1, 1:my + 1]) + Q[1:mx + 1, 0:my]
            s = np.sqrt(sdx ** 2 + sdy ** 2)
            thr = opts.TagThreshold
            if callable(thr):
                thr = thr(k - H.rootIdx + 1)
            tp = s > thr
        elif ind == 'rte':
            s = rte_indicator(H, k, p)
            thr = opts.TagThreshold
            if callable(thr):
                thr = thr(k - H.rootIdx + 1)
            tp = s > thr
        else:
            raise ValueError(('ebt' if H.tree else 'eb') + f'_tag_cluster:ind: unknown Indicator {opts.Indicator}')
        T[b[0] - 1:b[1], b[2] - 1:b[3]] |= tp
    cover = np.zeros((n[0], n[1]), dtype=bool)
    for p in range(lev.np):
        b = lev.box[p]
        cover[b[0] - 1:b[1], b[2] - 1:b[3]] = True
    allowed = _erode8(cover)
    if not device:
        T = _dilate(T, int(opts.TagBuffer))
        T &= allowed
    ncol = 5 if H.tree else 4
    if not T.any():
        return np.zeros((0, ncol), dtype=np.int64)
    minW, eff = int(opts.MinBoxWidth), float(opts.MinFillRatio)
    if not H.tree:
        boxes = _br_cluster(T, minW, eff)
        boxes = _clip_allowed(boxes, T, allowed)
        boxes = _grow_min(boxes, allowed, minW, n)
        boxes = _merge_or_drop_thin(boxes, allowed)
        return np.array(boxes, dtype=np.int64).reshape(-1, 4)
    out = []
    for q in range(lev.np):
        b = [int(v) for v in lev.box[q]]
        Tq = T[b[0] - 1:b[1], b[2] - 1:b[3]]
        if not Tq.any():
            continue
        Aq = allowed[b[0] - 1:b[1], b[2] - 1:b[3]]
        nq = [b[1] - b[0] + 1, b[3] - b[2] + 1]
        bq = _br_cluster(Tq, minW, eff)
        bq = _clip_allowed(bq, Tq, Aq)
        bq = _grow_min(bq, Aq, minW, nq)
        bq = _merge_or_drop_thin(bq, Aq, True)
        for bb in bq:
            out.append([q + 1, bb[0] + b[0] - 1, bb[1] + b[0] - 1, bb[2] + b[2] - 1, bb[3] + b[2] - 1])
    return np.array(out, dtype=np.int64).reshape(-1, 5)
