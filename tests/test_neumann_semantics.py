"""Reaction, gauge and source-projection semantics of the all-Neumann set-up
(EllipticBSAM/tests/testEbNeumannSemantics.m, tree copy
EllipticBSAMTree/tests/testEbtNeumannSemantics.m), on the oracle: a positive
reaction keeps the absolute constant error; the singular problem's error is
gauge-aligned for every SourceQuad; tiny but consistently scaled coefficients
are not classified as singular; the compatibility projection of a refined
Neumann problem shifts every visible source sample by one constant that
equals the raw defect, is idempotent, and the projected solve converges
(recorded finalRel = 1.599e-10 for both hierarchy forms).
"""
import copy

import numpy as np
import pytest

from bsam import ebOptions, ebProblem, ebSolve, ebtSolve, hierarchy as hier
from bsam.solve import ebSolveCycles, error_norms
from bsam_oracle import OracleBackend
from cases import printed_close

FINAL_REL = '1.599e-10'     # suite-output.txt lines 1 and 83


@pytest.mark.parametrize('tree', [False, True])
def test_neumann_semantics(tree):
    be = OracleBackend()
    H = hier.setup(ebProblem([0, 1, 0, 1], 1, 1, 0, ('neumann', 0), 0), ebOptions('BaseCells', [8, 8], 'Verbose', 0),
                   be, tree=tree)
    H.lev[1].Q[0][:] = 7
    e = error_norms(H)
    assert abs(e['linf'] - 7) < 1e-14 and e['meanShift'] == 0
    for nq in (1, 3):
        H = hier.setup(ebProblem([0, 1, 0, 1], 1, 0, 0, ('neumann', 0), 7),
                       ebOptions('BaseCells', [8, 8], 'SourceQuad', nq, 'Verbose', 0), be, tree=tree)
        e = error_norms(H)
        assert e['linf'] < 1e-14 and abs(e['meanShift'] + 7) < 1e-14
    solve = ebtSolve if tree else ebSolve
    sol = solve(ebProblem([0, 1, 0, 1], 1e-18, 1e-14, 1e-14, ('neumann', 0), 1), 'BaseCells', [8, 8], 'Verbose', 0,
                'RelTol', 1e-10, backend=be)
    assert not sol['H'].coarsest['singular'] and sol['err']['linf'] < 1e-11

    # u = x^4, -lap u = -12 x^2, outward g = 4 on the east side
    bc = {'west': ('neumann', 0), 'east': ('neumann', 4), 'south': ('neumann', 0), 'north': ('neumann', 0)}
    prob = ebProblem([0, 1, 0, 1], 1, 0, lambda x, y: -12 * x ** 2, bc, lambda x, y: x ** 4)
    H = hier.setup(prob, ebOptions('BaseCells', [16, 16], 'Verbose', 0), be, tree=tree)
    for box in ([5, 12, 5, 12], [12, 20, 12, 20]):
        H = hier.add_level(H, [[1] + box] if tree else [box], be)
    shifts, raw_sum = [], 0.0
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        for p in range(lev.np):
            b = lev.box[p]
            x, y = np.meshgrid((np.arange(b[0], b[1] + 1) - .5) * lev.h[0], (np.arange(b[2], b[3] + 1) - .5) * lev.h[1],
                               indexing='ij')
            raw = prob.f(x, y)
            vis = ~lev.covered[p]
            shifts.append((raw - lev.FTrue[p])[vis])
            raw_sum += float(np.sum(raw[vis])) * lev.h[0] * lev.h[1]
    shifts = np.concatenate(shifts)
    assert shifts.max() - shifts.min() < 1e-13
    assert abs(shifts.mean() - (raw_sum + 4)) < 1e-13
    H2 = copy.deepcopy(H)
    hier.compat_project(H2)
    assert abs(H2.compatibility['sourceShift'] - H.compatibility['sourceShift']) < 1e-13
    H = ebSolveCycles(H, be)
    rel = H.stats['stages'][-1]['finalRel']
    assert rel < 1e-8
    assert printed_close(rel, FINAL_REL), rel
