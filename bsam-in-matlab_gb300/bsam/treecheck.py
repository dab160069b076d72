"""Structural invariants of a single-parent tree hierarchy
(``EllipticBSAMTree/src/ebtTreeCheck.m``).

Checked per level: no two patches overlap; every patch of a refined level
names one parent (1-based) whose box contains its 2-aligned footprint, with
``mbounds`` equal to that footprint in the parent's local cells; the
footprint plus a one-cell ring is covered by the coarser level; every
parent's ``children`` list and ``covered`` mask agree with the patches that
name it.  A violation raises ``ValueError('ebt_tree_check:<what>: ...')``.
"""
from __future__ import annotations

import numpy as np


def ebtTreeCheck(H):
    """Returns {'nlev', 'rootIdx', 'maxChildren', 'perLevel' (nlev x 2:
    patches, stored cells), 'maxDepth'}."""
    stats = {'nlev': H.nlev, 'rootIdx': H.rootIdx, 'maxChildren': 0,
             'perLevel': np.zeros((H.nlev, 2), dtype=np.int64)}
    for k in range(1, H.nlev + 1):
        lev = H.lev[k]
        stats['perLevel'][k - 1] = [lev.np, sum(f.size for f in lev.F)]
        occ = np.zeros((int(lev.n[0]), int(lev.n[1])), dtype=np.int32)
        for b in lev.box:
            occ[b[0] - 1:b[1], b[2] - 1:b[3]] += 1
        if (occ > 1).any():
            raise ValueError(f'ebt_tree_check:overlap: level {k} has overlapping patches.')
        if k == 1:
            continue
        levC = H.lev[k - 1]
        cover = np.zeros((int(levC.n[0]), int(levC.n[1])), dtype=bool)
        for qb in levC.box:
            cover[qb[0] - 1:qb[1], qb[2] - 1:qb[3]] = True
        count = np.zeros(levC.np, dtype=np.int64)
        chk = [np.zeros((int(qb[1] - qb[0] + 1), int(qb[3] - qb[2] + 1)), dtype=bool) for qb in levC.box]
        for p in range(lev.np):
            b = [int(v) for v in lev.box[p]]
            q = int(lev.parent[p])
            mb = [int(v) for v in lev.mbounds[p]]
            if q < 1 or q > levC.np:
                raise ValueError(f'ebt_tree_check:parent: level {k} patch {p + 1}: bad parent record.')
            qb = [int(v) for v in levC.box[q - 1]]
            pmx, pmy = qb[1] - qb[0] + 1, qb[3] - qb[2] + 1
            if mb[0] < 1 or mb[1] > pmx or mb[2] < 1 or mb[3] > pmy or mb[0] > mb[1] or mb[2] > mb[3]:
                raise ValueError(f'ebt_tree_check:containment: level {k} patch {p + 1}: mbounds outside parent {q}.')
            if b[0] % 2 != 1 or b[1] % 2 != 0 or b[2] % 2 != 1 or b[3] % 2 != 0:
                raise ValueError(f'ebt_tree_check:align: level {k} patch {p + 1}: box not 2-aligned.')
            fp = [(b[0] + 1) // 2, b[1] // 2, (b[2] + 1) // 2, b[3] // 2]
            if mb != [fp[0] - qb[0] + 1, fp[1] - qb[0] + 1, fp[2] - qb[2] + 1, fp[3] - qb[2] + 1]:
                raise ValueError(f'ebt_tree_check:mbounds: level {k} patch {p + 1}: mbounds inconsistent with '
                                 f'global box.')
            count[q - 1] += 1
            chk[q - 1][mb[0] - 1:mb[1], mb[2] - 1:mb[3]] = True
            i0, i1 = max(fp[0] - 1, 1), min(fp[1] + 1, int(levC.n[0]))
            j0, j1 = max(fp[2] - 1, 1), min(fp[3] + 1, int(levC.n[1]))
            if not cover[i0 - 1:i1, j0 - 1:j1].all():
                raise ValueError(f'ebt_tree_check:nesting: level {k} patch {p + 1}: ring cell not covered by '
                                 f'level {k - 1}.')
        for q in range(levC.np):
            kids = list(levC.children[q])
            if len(kids) != count[q] or any(int(lev.parent[c - 1]) != q + 1 for c in kids):
                raise ValueError(f'ebt_tree_check:children: level {k - 1} patch {q + 1}: children list '
                                 f'inconsistent.')
            if not np.array_equal(np.asarray(levC.covered[q], dtype=bool), chk[q]):
                raise ValueError(f'ebt_tree_check:covered: level {k - 1} patch {q + 1}: covered mask mismatch.')
            stats['maxChildren'] = max(stats['maxChildren'], len(kids))
    stats['maxDepth'] = H.nlev - H.rootIdx + 1
    return stats
