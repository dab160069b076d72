"""Flat patch-descriptor tables: the upload format of the device C-ABI.

One hierarchy ``H`` is flattened into

  * ``levels``  int32 [nlev, LD]   per-level descriptor (``LD_*`` columns)
  * ``hs``      float64 [nlev, 2]  cell sizes (hx, hy)
  * ``patches`` int32 [npatch, PD] per-patch descriptor (``PD_*`` columns)
  * field arrays (float64) with every patch of every level concatenated:
    ``Q`` (padded), ``F``, ``FTrue``, ``CC``, ``InvDiagS`` (cells),
    ``DeW`` (x faces), ``DnS`` (y faces), ``QC`` (padded coarse shadow),
    ``bcg`` (boundary data W,E,S,N), ``cfd`` (interface D W,E,S,N),
    ``pcoef`` (parent coefficients over the footprint: PDeW,PDnS,PCC),
    ``covered`` (uint8 per cell)
  * index tables (int32, global flat indices):
      ``same``  [n,2]  (src Q, dst Q)       same-level ghost copies
      ``ring``  [n,2]  (src Q, dst QC)      parent -> QC ring gathers
      ``win``   [n]    src Q per parent-window cell (ring + interior)
      ``fp``    [n,2]  (parent Q, parent cell) per footprint cell
      ``corr``  [n]    correction target cell per coarse interface face, -1
                       where the face is not coarse-fine (W,E,S,N blocks)
  * the coarsest operator: ``Ainv`` (N x N), ``bcRhs`` (N)

These are the reference's own tables (``ebBuildOps.m`` ring/same/usc/fsc/
winrect/corr*, ``ebtBuildOps.m`` slices, ``ebGatherParentCoeffs.m`` cfD and
``ebParentCoeffs.m`` windows) with patch-local indices turned into global
ones; nothing is precompiled for a particular kernel design.  The CUDA
library derives its execution plan (ghost programs, tiles, gather-form
correction lists) from them at upload time.
"""
from __future__ import annotations

import numpy as np

from .hierarchy import parent_coeffs

# per-level descriptor columns
LD_N0, LD_N1, LD_P0, LD_P1, LD_CELL0, LD_CELL1, LD_Q0, LD_Q1 = range(8)
LD = 8

# per-patch descriptor columns
(PD_LEVEL, PD_ILO, PD_IHI, PD_JLO, PD_JHI, PD_MX, PD_MY, PD_PAR0,
 PD_BCW, PD_BCE, PD_BCS, PD_BCN, PD_FIW, PD_FIE, PD_FIS, PD_FIN,
 PD_CCSW, PD_CCSE, PD_CCNW, PD_CCNE,
 PD_QOFF, PD_COFF, PD_DEWOFF, PD_DNSOFF, PD_QCOFF, PD_BCGOFF, PD_CFDOFF, PD_PCOFF,
 PD_SAME0, PD_SAME1, PD_RING0, PD_RING1, PD_WIN0, PD_FP0, PD_CORR0, PD_PARENT) = range(36)
PD = 36

FIELD_Q, FIELD_F, FIELD_FTRUE, FIELD_QC = 0, 1, 2, 3


class Flat:
    pass


def flatten(H):
    """Flatten ``H`` into the upload format (see module docstring)."""
    nlev = H.nlev
    # ---- offsets ----------------------------------------------------------
    pglob = {}          # (k, p) -> global patch index
    rows = []
    qoff = coff = dewoff = dnsoff = qcoff = bcgoff = cfdoff = pcoff = 0
    levels = np.zeros((nlev, LD), dtype=np.int32)
    hs = np.zeros((nlev, 2))
    for k in range(1, nlev + 1):
        lev = H.lev[k]
        levels[k - 1, LD_N0], levels[k - 1, LD_N1] = lev.n
        levels[k - 1, LD_P0] = len(rows)
        levels[k - 1, LD_CELL0] = coff
        levels[k - 1, LD_Q0] = qoff
        hs[k - 1] = lev.h
        for p in range(lev.np):
            b = [int(v) for v in lev.box[p]]
            mx, my = b[1] - b[0] + 1, b[3] - b[2] + 1
            r = np.full(PD, -1, dtype=np.int64)
            r[PD_LEVEL] = k
            r[PD_ILO:PD_JHI + 1] = [b[0], b[1], b[2], b[3]]
            r[PD_MX], r[PD_MY] = mx, my
            r[PD_PAR0] = lev.par0[p]
            for s in range(4):
                r[PD_BCW + s] = lev.bc[p][s]['code']
                r[PD_FIW + s] = int(bool(lev.faceInternal[p][s]))
                r[PD_CCSW + s] = lev.cornerClass[p][s]
            r[PD_QOFF] = qoff
            r[PD_COFF] = coff
            r[PD_DEWOFF] = dewoff
            r[PD_DNSOFF] = dnsoff
            r[PD_BCGOFF] = bcgoff
            qoff += (mx + 2) * (my + 2)
            coff += mx * my
            dewoff += (mx + 1) * my
            dnsoff += mx * (my + 1)
            bcgoff += 2 * (mx + my)
            if k > 1:
                cmx, cmy = mx // 2, my // 2
                r[PD_QCOFF] = qcoff
                r[PD_CFDOFF] = cfdoff
                r[PD_PCOFF] = pcoff
                qcoff += (cmx + 2) * (cmy + 2)
                cfdoff += 2 * (cmx + cmy)
                pcoff += (cmx + 1) * cmy + cmx * (cmy + 1) + cmx * cmy
            pglob[(k, p)] = len(rows)
            rows.append(r)
        levels[k - 1, LD_P1] = len(rows)
        levels[k - 1, LD_CELL1] = coff
        levels[k - 1, LD_Q1] = qoff
    patches = np.array(rows, dtype=np.int64)
    for name, tot in (('Q', qoff), ('cells', coff), ('DeW', dewoff), ('DnS', dnsoff), ('QC', qcoff)):
        if tot >= 2 ** 31:
            raise ValueError(f'bsam_flat:size: {name} has {tot} entries; the upload format indexes with int32')

    fl = Flat()
    fl.levels, fl.hs = levels, hs
    fl.Q = np.zeros(qoff)
    fl.F = np.zeros(coff)
    fl.FTrue = np.zeros(coff)
    fl.CC = np.zeros(coff)
    fl.InvDiagS = np.zeros(coff)
    fl.covered = np.zeros(coff, dtype=np.uint8)
    fl.DeW = np.zeros(dewoff)
    fl.DnS = np.zeros(dnsoff)
    fl.QC = np.zeros(qcoff)
    fl.bcg = np.zeros(bcgoff)
    fl.cfd = np.zeros(cfdoff)
    fl.pcoef = np.zeros(pcoff)
    same, ring, win, fp, corr = [], [], [], [], []
    nsame = nring = nwin = nfp = ncorr = 0

    def R(k, p):
        return patches[pglob[(k, p)]]

    for k in range(1, nlev + 1):
        lev = H.lev[k]
        for p in range(lev.np):
            r = R(k, p)
            mx, my = int(r[PD_MX]), int(r[PD_MY])
            qo, co = int(r[PD_QOFF]), int(r[PD_COFF])
            fl.Q[qo:qo + (mx + 2) * (my + 2)] = lev.Q[p].ravel(order='F')
            fl.F[co:co + mx * my] = lev.F[p].ravel(order='F')
            fl.FTrue[co:co + mx * my] = lev.FTrue[p].ravel(order='F')
            fl.CC[co:co + mx * my] = lev.CC[p].ravel(order='F')
            fl.InvDiagS[co:co + mx * my] = lev.InvDiagS[p].ravel(order='F')
            fl.covered[co:co + mx * my] = lev.covered[p].ravel(order='F')
            o = int(r[PD_DEWOFF])
            fl.DeW[o:o + (mx + 1) * my] = lev.DeW[p].ravel(order='F')
            o = int(r[PD_DNSOFF])
            fl.DnS[o:o + mx * (my + 1)] = lev.DnS[p].ravel(order='F')
            o = int(r[PD_BCGOFF])
            for s, nn in enumerate((my, my, mx, mx)):
                g = lev.bc[p][s]['g']
                if lev.bc[p][s]['code'] != 0:
                    fl.bcg[o:o + nn] = g
                o += nn
            # same-level copies
            r[PD_SAME0] = nsame
            for (sp, src, dst) in lev.sameOps[p]:
                so = int(R(k, sp - 1)[PD_QOFF])
                same.append(np.stack([so + src, qo + dst], axis=1))
                nsame += len(src)
            r[PD_SAME1] = nsame
            if k == 1:
                continue
            cmx, cmy = mx // 2, my // 2
            qco = int(r[PD_QCOFF])
            fl.QC[qco:qco + (cmx + 2) * (cmy + 2)] = lev.QC[p].ravel(order='F')
            o = int(r[PD_CFDOFF])
            cfD = lev.cfD[p]
            fl.cfd[o:o + cmy] = cfD['W']
            fl.cfd[o + cmy:o + 2 * cmy] = cfD['E']
            fl.cfd[o + 2 * cmy:o + 2 * cmy + cmx] = cfD['S']
            fl.cfd[o + 2 * cmy + cmx:o + 2 * (cmx + cmy)] = cfD['N']
            PDeW, PDnS, PCC = parent_coeffs(H, k, p)
            o = int(r[PD_PCOFF])
            n1, n2, n3 = (cmx + 1) * cmy, cmx * (cmy + 1), cmx * cmy
            fl.pcoef[o:o + n1] = PDeW.ravel(order='F')
            fl.pcoef[o + n1:o + n1 + n2] = PDnS.ravel(order='F')
            fl.pcoef[o + n1 + n2:o + n1 + n2 + n3] = PCC.ravel(order='F')
            ops = lev.ops[p]
            levC = H.lev[k - 1]
            # ring gathers, window gathers, footprint scatters
            r[PD_RING0] = nring
            W = np.full((cmx + 2) * (cmy + 2), -1, dtype=np.int64)
            fpq = np.full(cmx * cmy, -1, dtype=np.int64)
            fpc = np.full(cmx * cmy, -1, dtype=np.int64)
            if ops['tree']:
                q = int(ops['sp']) - 1
                rq = R(k - 1, q)
                pmx = int(rq[PD_MX])
                pqo, pco = int(rq[PD_QOFF]), int(rq[PD_COFF])
                r[PD_PARENT] = pglob[(k - 1, q)]
                Il, Ih2, Jl, Jh2 = ops['win']            # padded parent range
                ii, jj = np.meshgrid(np.arange(Il, Ih2 + 1), np.arange(Jl, Jh2 + 1), indexing='ij')
                W = (pqo + (ii - 1) + (jj - 1) * (pmx + 2)).ravel(order='F')
                # ring = perimeter of the window slice (W/E columns, then S/N rows)
                wi, wj = np.meshgrid(np.arange(1, cmx + 3), np.arange(1, cmy + 3), indexing='ij')
                wi, wj = wi.ravel(order='F'), wj.ravel(order='F')
                widx = np.arange(W.size)
                sel = []
                for (ci, cj) in ((wi == 1, None), (wi == cmx + 2, None)):
                    sel.append(widx[ci])
                sel.append(widx[(wj == 1) & (wi > 1) & (wi < cmx + 2)])
                sel.append(widx[(wj == cmy + 2) & (wi > 1) & (wi < cmx + 2)])
                for s in sel:
                    ring.append(np.stack([W[s], qco + s], axis=1))
                    nring += len(s)
                ci, cj = np.meshgrid(np.arange(cmx), np.arange(cmy), indexing='ij')
                mb = [int(v) for v in H.lev[k].mbounds[p]]
                fpq = (pqo + (mb[0] + ci) + (mb[2] + cj) * (pmx + 2)).ravel(order='F')
                fpc = (pco + (mb[0] - 1 + ci) + (mb[2] - 1 + cj) * pmx).ravel(order='F')
            else:
                for (sp, src, dst) in ops['ring']:
                    rq = R(k - 1, sp - 1)
                    ring.append(np.stack([int(rq[PD_QOFF]) + src, qco + dst], axis=1))
                    nring += len(src)
                    W[dst] = int(rq[PD_QOFF]) + src
                for (sp, sr, dr) in ops['winrect']:
                    rq = R(k - 1, sp - 1)
                    pmx = int(rq[PD_MX])
                    si, sj = np.meshgrid(np.arange(sr[0], sr[1] + 1), np.arange(sr[2], sr[3] + 1), indexing='ij')
                    di, dj = np.meshgrid(np.arange(dr[0], dr[1] + 1), np.arange(dr[2], dr[3] + 1), indexing='ij')
                    W[((di - 1) + (dj - 1) * (cmx + 2)).ravel()] = \
                        int(rq[PD_QOFF]) + ((si - 1) + (sj - 1) * (pmx + 2)).ravel()
                for (dp, sr, dr) in ops['usc']:
                    rq = R(k - 1, dp - 1)
                    pmx = int(rq[PD_MX])
                    si, sj = np.meshgrid(np.arange(sr[0], sr[1] + 1), np.arange(sr[2], sr[3] + 1), indexing='ij')
                    di, dj = np.meshgrid(np.arange(dr[0], dr[1] + 1), np.arange(dr[2], dr[3] + 1), indexing='ij')
                    fpq[((si - 1) + (sj - 1) * cmx).ravel()] = \
                        int(rq[PD_QOFF]) + ((di - 1) + (dj - 1) * (pmx + 2)).ravel()
                for (dp, sr, dr) in ops['fsc']:
                    rq = R(k - 1, dp - 1)
                    pmx = int(rq[PD_MX])
                    si, sj = np.meshgrid(np.arange(sr[0], sr[1] + 1), np.arange(sr[2], sr[3] + 1), indexing='ij')
                    di, dj = np.meshgrid(np.arange(dr[0], dr[1] + 1), np.arange(dr[2], dr[3] + 1), indexing='ij')
                    fpc[((si - 1) + (sj - 1) * cmx).ravel()] = \
                        int(rq[PD_COFF]) + ((di - 1) + (dj - 1) * pmx).ravel()
            if np.any(W < 0) or np.any(fpq < 0) or np.any(fpc < 0):
                raise ValueError(f'bsam_flat:cover: incomplete parent tables for patch {p+1} of level {k}')
            r[PD_RING1] = nring
            r[PD_WIN0] = nwin
            win.append(W)
            nwin += W.size
            r[PD_FP0] = nfp
            fp.append(np.stack([fpq, fpc], axis=1))
            nfp += fpq.size
            # flux-correction targets, one per coarse interface face
            r[PD_CORR0] = ncorr
            for f, key, nn in ((0, 'corrW', cmy), (1, 'corrE', cmy), (2, 'corrS', cmx), (3, 'corrN', cmx)):
                t = np.full(nn, -1, dtype=np.int64)
                for (dp, src, dst) in ops[key]['ops']:
                    t[src] = int(R(k - 1, dp - 1)[PD_COFF]) + dst
                corr.append(t)
                ncorr += nn

    def cat(lst, shape):
        return np.ascontiguousarray(np.concatenate(lst).astype(np.int32)) if lst else np.zeros(shape, np.int32)

    fl.patches = np.ascontiguousarray(patches.astype(np.int32))
    fl.same = cat(same, (0, 2)).reshape(-1, 2)
    fl.ring = cat(ring, (0, 2)).reshape(-1, 2)
    fl.win = cat(win, (0,))
    fl.fp = cat(fp, (0, 2)).reshape(-1, 2)
    fl.corr = cat(corr, (0,))
    fl.Ainv = np.ascontiguousarray(H.coarsest['Ainv'], dtype=np.float64)
    fl.bcRhs = np.ascontiguousarray(H.coarsest['bcRhs'], dtype=np.float64)
    fl.singular = int(H.coarsest['singular'])
    fl.nlev, fl.rootIdx = nlev, H.rootIdx
    fl.npatch = patches.shape[0]
    fl.pglob = pglob
    return fl


def scatter_field(H, fl, which, arr):
    """Write a downloaded flat field back into the per-patch arrays of H."""
    for (k, p), g in fl.pglob.items():
        r = fl.patches[g]
        mx, my = int(r[PD_MX]), int(r[PD_MY])
        lev = H.lev[k]
        if which == FIELD_Q:
            o = int(r[PD_QOFF])
            lev.Q[p][...] = arr[o:o + (mx + 2) * (my + 2)].reshape((mx + 2, my + 2), order='F')
        elif which == FIELD_QC:
            if k == 1:
                continue
            o = int(r[PD_QCOFF])
            cmx, cmy = mx // 2, my // 2
            lev.QC[p] = arr[o:o + (cmx + 2) * (cmy + 2)].reshape((cmx + 2, cmy + 2), order='F').copy(order='F')
        elif which == FIELD_F:
            o = int(r[PD_COFF])
            lev.F[p] = arr[o:o + mx * my].reshape((mx, my), order='F').copy(order='F')
        elif which == FIELD_FTRUE:
            o = int(r[PD_COFF])
            lev.FTrue[p] = arr[o:o + mx * my].reshape((mx, my), order='F').copy(order='F')


def gather_field(H, fl, which):
    """Flat copy of one field of H in the layout of ``fl`` (the inverse of
    scatter_field); used to refresh a resident hierarchy after host edits."""
    sizes = {FIELD_Q: fl.Q.size, FIELD_QC: fl.QC.size, FIELD_F: fl.F.size, FIELD_FTRUE: fl.F.size}
    out = np.zeros(sizes[which])
    for (k, p), g in fl.pglob.items():
        r = fl.patches[g]
        lev = H.lev[k]
        if which == FIELD_Q:
            a, o = lev.Q[p], int(r[PD_QOFF])
        elif which == FIELD_QC:
            if k == 1:
                continue
            a, o = lev.QC[p], int(r[PD_QCOFF])
        elif which == FIELD_F:
            a, o = lev.F[p], int(r[PD_COFF])
        else:
            a, o = lev.FTrue[p], int(r[PD_COFF])
        out[o:o + a.size] = np.asarray(a).ravel(order='F')
    return out


def visible_q_index(fl):
    """Q indices of the visible cells (levels >= root, not covered by a finer
    level), in cell order: the cells the composite norms run over."""
    out = []
    for g in range(fl.npatch):
        r = fl.patches[g]
        if int(r[PD_LEVEL]) < fl.rootIdx:
            continue
        mx, my = int(r[PD_MX]), int(r[PD_MY])
        co, qo = int(r[PD_COFF]), int(r[PD_QOFF])
        ii, jj = np.meshgrid(np.arange(mx), np.arange(my), indexing='ij')
        q = (qo + (ii + 1) + (jj + 1) * (mx + 2)).ravel(order='F')
        vis = fl.covered[co:co + mx * my] == 0
        out.append(q[vis])
    return np.concatenate(out) if out else np.zeros(0, dtype=np.int64)


def rel_errors(a, b, idx):
    """(relative L2, relative max) difference of a against b over idx."""
    d = a[idx] - b[idx]
    nb2 = float(np.linalg.norm(b[idx]))
    nbm = float(np.max(np.abs(b[idx]))) if idx.size else 0.0
    return (float(np.linalg.norm(d)) / max(nb2, 1e-300), float(np.max(np.abs(d))) / max(nbm, 1e-300) if idx.size else 0.0)
