"""Batches of independent hierarchies solved in one device hierarchy.

The reference solves one hierarchy per ``ebSolveCycles`` call.  On the GPU a
single small hierarchy leaves most of the 152 SMs idle (a 16x16 coarsest
level is one block), so many instances are merged into one upload: merged
level k holds the level-k patches of every instance, instance by instance,
and every launch of the V-cycle covers all of them.  Each instance keeps its
own coarsest inverse, root level, residual norms and stop test, and an
instance that has converged is frozen (its stores are predicated off) while
the others continue, so each instance's result equals its solve alone.

Instances may differ in patches, levels, root, coefficients and data; they
must share the cell size of every level they have (``hs``), which holds for
instances on equal domains with equal coarsest grids.
"""
from __future__ import annotations

import numpy as np

from .flat import (Flat, flatten, scatter_field, LD, LD_N0, LD_N1, LD_P0, LD_P1, LD_CELL0, LD_CELL1, LD_Q0, LD_Q1,
                   PD_LEVEL, PD_MX, PD_MY, PD_QOFF, PD_COFF, PD_DEWOFF, PD_DNSOFF, PD_QCOFF, PD_BCGOFF, PD_CFDOFF,
                   PD_PCOFF, PD_SAME0, PD_SAME1, PD_RING0, PD_RING1, PD_WIN0, PD_FP0, PD_CORR0, PD_PARENT,
                   FIELD_Q, FIELD_QC, FIELD_F)


def _extents(r):
    """Per-patch block lengths in each flat array: q, cells, dew, dns, qc,
    bcg, cfd, pcoef, win, fp, corr."""
    mx, my, k = int(r[PD_MX]), int(r[PD_MY]), int(r[PD_LEVEL])
    n = {'q': (mx + 2) * (my + 2), 'c': mx * my, 'dew': (mx + 1) * my, 'dns': mx * (my + 1),
         'bcg': 2 * (mx + my), 'qc': 0, 'cfd': 0, 'pc': 0, 'win': 0, 'fp': 0, 'corr': 0}
    if k > 1:
        cmx, cmy = mx // 2, my // 2
        n.update(qc=(cmx + 2) * (cmy + 2), cfd=2 * (cmx + cmy),
                 pc=(cmx + 1) * cmy + cmx * (cmy + 1) + cmx * cmy, win=(cmx + 2) * (cmy + 2), fp=cmx * cmy,
                 corr=2 * (cmx + cmy))
    return n


_OFFCOL = {'q': PD_QOFF, 'c': PD_COFF, 'dew': PD_DEWOFF, 'dns': PD_DNSOFF, 'qc': PD_QCOFF, 'bcg': PD_BCGOFF,
           'cfd': PD_CFDOFF, 'pc': PD_PCOFF, 'win': PD_WIN0, 'fp': PD_FP0, 'corr': PD_CORR0}


def merge_flats(parts):
    """Merge per-instance flat tables (``flatten`` output) into one batch
    table.  Returns a Flat with the extra attributes ``ninst``,
    ``patch_inst``, ``inst_root`` and, per instance, the index maps from its
    own flat arrays into the merged ones (``maps[i][name]``)."""
    ninst = len(parts)
    if ninst < 1:
        raise ValueError('bsam_batch:empty: no instances')
    nlev = max(p.nlev for p in parts)
    for k in range(1, nlev + 1):
        hk = [tuple(p.hs[k - 1]) for p in parts if p.nlev >= k]
        if any(h != hk[0] for h in hk):
            raise ValueError(f'bsam_batch:spacing: instances differ in the cell size of level {k}')
    for p in parts:
        if int(p.patches[:, PD_LEVEL].tolist().count(1)) != 1:
            raise ValueError('bsam_batch:coarsest: every instance needs exactly one level-1 patch')
    # merged order of patches: level, instance, patch
    order = []
    for k in range(1, nlev + 1):
        for i, fl in enumerate(parts):
            if fl.nlev < k:
                continue
            L = fl.levels[k - 1]
            order.extend((i, g) for g in range(int(L[LD_P0]), int(L[LD_P1])))
    newidx = [np.full(fl.npatch, -1, dtype=np.int64) for fl in parts]
    for ng, (i, g) in enumerate(order):
        newidx[i][g] = ng
    # new offsets per patch and block
    names = ('q', 'c', 'dew', 'dns', 'qc', 'bcg', 'cfd', 'pc', 'win', 'fp', 'corr')
    tot = dict.fromkeys(names, 0)
    rows = np.zeros((len(order), parts[0].patches.shape[1]), dtype=np.int64)
    maps = [{nm: np.full(_size(fl, nm), -1, dtype=np.int64) for nm in ('q', 'c', 'qc')} for fl in parts]
    moves = []                       # (inst, name, old_off, new_off, length)
    for ng, (i, g) in enumerate(order):
        r = parts[i].patches[g].astype(np.int64).copy()
        ext = _extents(r)
        for nm in names:
            if ext[nm] == 0:
                continue
            col = _OFFCOL[nm]
            moves.append((i, nm, int(r[col]), tot[nm], ext[nm]))
            if nm in maps[i]:
                maps[i][nm][int(r[col]):int(r[col]) + ext[nm]] = np.arange(tot[nm], tot[nm] + ext[nm])
            r[col] = tot[nm]
            tot[nm] += ext[nm]
        if r[PD_PARENT] >= 0:
            r[PD_PARENT] = newidx[i][int(r[PD_PARENT])]
        rows[ng] = r
    for nm in ('q', 'c', 'qc'):
        if tot[nm] >= 2 ** 31:
            raise ValueError(f'bsam_batch:size: merged {nm} has {tot[nm]} entries; the upload format indexes with int32')
    out = Flat()
    fields = {'Q': 'q', 'F': 'c', 'FTrue': 'c', 'CC': 'c', 'InvDiagS': 'c', 'covered': 'c', 'DeW': 'dew',
              'DnS': 'dns', 'QC': 'qc', 'bcg': 'bcg', 'cfd': 'cfd', 'pcoef': 'pc'}
    for f, nm in fields.items():
        setattr(out, f, np.zeros(tot[nm], dtype=getattr(parts[0], f).dtype))
    for (i, nm, o, no, n) in moves:
        for f, fnm in fields.items():
            if fnm == nm:
                getattr(out, f)[no:no + n] = getattr(parts[i], f)[o:o + n]
    # index tables, patch by patch in the merged order
    same, ring, win, fp, corr = [], [], [], [], []
    ns = nr = nw = nf = nc = 0
    for ng, (i, g) in enumerate(order):
        fl, mp, r0, r = parts[i], maps[i], parts[i].patches[g], rows[ng]
        s0, s1 = int(r0[PD_SAME0]), int(r0[PD_SAME1])
        t = fl.same[s0:s1]
        same.append(np.stack([mp['q'][t[:, 0]], mp['q'][t[:, 1]]], axis=1) if len(t) else np.zeros((0, 2), np.int64))
        r[PD_SAME0], r[PD_SAME1] = ns, ns + (s1 - s0)
        ns += s1 - s0
        if int(r0[PD_LEVEL]) == 1:
            continue
        ext = _extents(r0)
        a0, a1 = int(r0[PD_RING0]), int(r0[PD_RING1])
        t = fl.ring[a0:a1]
        ring.append(np.stack([mp['q'][t[:, 0]], mp['qc'][t[:, 1]]], axis=1) if len(t) else np.zeros((0, 2), np.int64))
        r[PD_RING0], r[PD_RING1] = nr, nr + (a1 - a0)
        nr += a1 - a0
        w0 = int(r0[PD_WIN0])
        win.append(mp['q'][fl.win[w0:w0 + ext['win']]])
        r[PD_WIN0] = nw
        nw += ext['win']
        f0 = int(r0[PD_FP0])
        t = fl.fp[f0:f0 + ext['fp']]
        fp.append(np.stack([mp['q'][t[:, 0]], mp['c'][t[:, 1]]], axis=1))
        r[PD_FP0] = nf
        nf += ext['fp']
        c0 = int(r0[PD_CORR0])
        t = fl.corr[c0:c0 + ext['corr']].astype(np.int64)
        m = np.where(t >= 0, mp['c'][np.maximum(t, 0)], -1)
        if np.any((m < 0) != (t < 0)):
            raise ValueError('bsam_batch:index: a correction target points outside its instance')
        corr.append(m)
        r[PD_CORR0] = nc
        nc += ext['corr']
    for nm, tab in (('same', same), ('ring', ring), ('win', win), ('fp', fp)):
        if any(np.any(a < 0) for a in tab):
            raise ValueError(f'bsam_batch:index: a {nm} entry points outside its instance')

    def cat(lst, shape):
        return np.ascontiguousarray(np.concatenate(lst).astype(np.int32)) if lst else np.zeros(shape, np.int32)

    out.same = cat(same, (0, 2)).reshape(-1, 2)
    out.ring = cat(ring, (0, 2)).reshape(-1, 2)
    out.win = cat(win, (0,))
    out.fp = cat(fp, (0, 2)).reshape(-1, 2)
    out.corr = cat(corr, (0,))
    out.patches = np.ascontiguousarray(rows.astype(np.int32))
    # levels
    levels = np.zeros((nlev, LD), dtype=np.int32)
    hs = np.zeros((nlev, 2))
    pk = rows[:, PD_LEVEL]
    for k in range(1, nlev + 1):
        idx = np.nonzero(pk == k)[0]
        first = next(fl for fl in parts if fl.nlev >= k)
        levels[k - 1, LD_N0], levels[k - 1, LD_N1] = first.levels[k - 1, LD_N0], first.levels[k - 1, LD_N1]
        levels[k - 1, LD_P0], levels[k - 1, LD_P1] = idx[0], idx[-1] + 1
        lastr = rows[idx[-1]]
        levels[k - 1, LD_CELL0] = rows[idx[0], PD_COFF]
        levels[k - 1, LD_CELL1] = lastr[PD_COFF] + lastr[PD_MX] * lastr[PD_MY]
        levels[k - 1, LD_Q0] = rows[idx[0], PD_QOFF]
        levels[k - 1, LD_Q1] = lastr[PD_QOFF] + (lastr[PD_MX] + 2) * (lastr[PD_MY] + 2)
        hs[k - 1] = first.hs[k - 1]
    out.levels, out.hs = levels, hs
    out.Ainv = np.ascontiguousarray(np.concatenate([np.asarray(fl.Ainv, dtype=np.float64).ravel() for fl in parts]))
    out.bcRhs = np.ascontiguousarray(np.concatenate([np.asarray(fl.bcRhs, dtype=np.float64).ravel() for fl in parts]))
    out.singular = 0
    out.nlev = nlev
    out.rootIdx = min(int(fl.rootIdx) for fl in parts)
    out.npatch = len(order)
    out.ninst = ninst
    out.patch_inst = np.ascontiguousarray(np.array([i for (i, g) in order], dtype=np.int32))
    out.inst_root = np.ascontiguousarray(np.array([fl.rootIdx for fl in parts], dtype=np.int32))
    out.maps = maps
    out.parts = parts
    out.pglob = None
    return out


def _size(fl, nm):
    return {'q': fl.Q.size, 'c': fl.F.size, 'qc': fl.QC.size}[nm]


def flatten_batch(Hs):
    """Flatten every hierarchy of ``Hs`` and merge them (see merge_flats)."""
    return merge_flats([flatten(H) for H in Hs])


def split_field(bfl, which, arr, i):
    """Instance i's own flat copy of a merged field (Q, QC, F/FTrue)."""
    nm = {FIELD_Q: 'q', FIELD_QC: 'qc', FIELD_F: 'c'}.get(which, 'c')
    return np.asarray(arr)[bfl.maps[i][nm]]


def join_field(bfl, which, arrs):
    """Merged flat field from every instance's own flat copy."""
    nm = {FIELD_Q: 'q', FIELD_QC: 'qc', FIELD_F: 'c'}.get(which, 'c')
    n = sum(m[nm].size for m in bfl.maps)
    out = np.zeros(n)
    for m, a in zip(bfl.maps, arrs):
        out[m[nm]] = a
    return out


def solve_batch(Hs, backend=None):
    """``ebSolveCycles`` of every hierarchy in ``Hs`` as one batch on the
    device.  Each H receives its solution (Q, QC, F) as a solve of it alone
    would leave it; returns [(vcycles, resHist, finalRel, visibleCells)]."""
    from .device import DeviceBackend, DevHier, BSAM_FIELD_Q, BSAM_FIELD_QC, BSAM_FIELD_F
    backend = backend or DeviceBackend.get(0)
    opts = Hs[0].opts
    for H in Hs[1:]:
        for key in ('NPre', 'NPost', 'Omega', 'GhostInterp', 'MassCorrection', 'Precision'):
            if H.opts[key] != opts[key]:
                raise ValueError(f'bsam_batch:opts: instances of a batch share {key}')
    bfl = flatten_batch(Hs)
    dh = DevHier(backend.ctx, bfl, opts)
    for i, H in enumerate(Hs[1:], 1):
        if H.opts is not opts:
            dh.set_stop(i, int(H.opts.MaxVCycles), float(H.opts.RelTol))
    dh.solve_cycles(int(opts.MaxVCycles) + 2)
    Q = dh.get(BSAM_FIELD_Q, bfl.Q.size)
    QC = dh.get(BSAM_FIELD_QC, bfl.QC.size)
    F = dh.get(BSAM_FIELD_F, bfl.F.size)
    out = []
    for i, H in enumerate(Hs):
        fl = bfl.parts[i]
        fl.pglob = getattr(fl, 'pglob', None)
        scatter_field(H, fl, FIELD_Q, split_field(bfl, FIELD_Q, Q, i))
        scatter_field(H, fl, FIELD_QC, split_field(bfl, FIELD_QC, QC, i))
        scatter_field(H, fl, FIELD_F, split_field(bfl, FIELD_F, F, i))
        H.dirty.clear()
        out.append(dh.batch_result(i, int(H.opts.MaxVCycles) + 2))
    return out
