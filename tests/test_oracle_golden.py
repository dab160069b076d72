"""Pin the oracle (host set-up + C restatement of the solve path) to the
reference's recorded MATLAB outputs (tests/golden/reference_outputs.json,
extracted from the reference's verification/ folder by make_golden.py).

The reference's timings and numbers come from MATLAB R2026a; agreement is
to the printed precision of those records, except the starfish residual
history, which is recorded to 15 digits and is compared to the residual's
own round-off floor (|L u| terms near 1e6 leave ~1e-10 of absolute noise in
every max-norm residual).
"""
import json
import os

import numpy as np
import pytest

from bsam import ebSolve, ebtSolve
from bsam_oracle import OracleBackend
from cases import config1_problem, vardc_problem, gauss51_problem, box_in_box_tag, printed_close

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), 'golden', 'reference_outputs.json')))


@pytest.mark.parametrize('tree', [False, True])
def test_readme_config1_stage_lines(tree):
    """G3: README QC-ring / tree example, RelTol 1e-9 (readme-examples.txt:2-11)."""
    solve = ebtSolve if tree else ebSolve
    sol = solve(config1_problem(), 'BaseCells', 32, 'MaxLevels', 3, 'TagThreshold', 1e-2, 'Verbose', 0,
                backend=OracleBackend())
    gold = GOLD['readme_tree_stages' if tree else 'readme_ring_stages']
    stages = sol['stats']['stages']
    assert len(stages) == len(gold) == 3
    for st, g in zip(stages, gold):
        assert st['amrLevels'] == g['amrLevels']
        assert st['vcycles'] == g['vcycles']
        assert st['visibleCells'] == g['visibleCells']
        assert printed_close(st['finalRel'], g['rel']), (st['finalRel'], g['rel'])
        assert printed_close(st['avgFactor'], g['avgFactor']), (st['avgFactor'], g['avgFactor'])
    added = GOLD['readme_tree_added' if tree else 'readme_ring_added']
    for a, lv in zip(added, sol['levels'][1:]):
        assert lv['np'] == a['np'] and lv['cells'] == a['cells']
    if tree:
        H = sol['H']
        # ebtTreeCheck (readme-examples.txt:14-21): nlev 4, rootIdx 2, maxChildren 4
        assert H.nlev == 4 and H.rootIdx == 2
        assert max(len(c) for c in H.lev[3].children) == 4


def test_uniform_mms_T1():
    """G5: T1 uniform MMS with variable D, C (suite-output.txt:3-7)."""
    for g in GOLD['suite_T1_uniform_mms'][:3]:
        sol = ebSolve(vardc_problem(), 'BaseCells', g['m'], 'Verbose', 0, 'RelTol', 1e-11, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['vcycles'] == g['V']
        assert printed_close(sol['err']['linf'], g['err_inf']), (sol['err']['linf'], g['err_inf'])
        assert printed_close(sol['err']['l2'], g['err_l2']), (sol['err']['l2'], g['err_l2'])
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g['factor'])


@pytest.mark.parametrize('interp', ['qif', 'lif'])
def test_box_in_box_T3(interp):
    """G5: T3 fixed box-in-box hierarchies, m0 = 32 and 64, 2-4 levels
    (suite-output.txt:22-47): error, factor, V-cycles, mass defect < 1e-13."""
    rows = [g for g in GOLD['suite_T3_box_in_box'] if g['interp'] == interp and g['m0'] in (32, 64)]
    assert len(rows) == 6
    for g in rows:
        sol = ebSolve(gauss51_problem(), 'BaseCells', g['m0'], 'MaxLevels', g['L'], 'Indicator', 'fun',
                      'TagFunction', box_in_box_tag, 'TagBuffer', 0, 'GhostInterp', interp, 'Verbose', 0,
                      'RelTol', 1e-10, 'MaxVCycles', 40, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['vcycles'] == g['V'], (g, st['vcycles'])
        assert printed_close(sol['err']['linf'], g['err']), (sol['err']['linf'], g)
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g)
        assert sol['mass']['rel'] < 1e-13


@pytest.mark.slow
def test_starfish_golden():
    """G1 + G2: the starfish transmission problem of examples/demoStarfish.m
    (verification/starfish-full.json, starfish-full-residual.csv)."""
    from bsam.ddm import starfish_problem, starfish_tag
    prob, aux, g = starfish_problem()
    sol = ebSolve(prob, 'BaseCells', 64, 'MaxLevels', 5, 'Indicator', 'fun', 'TagFunction', starfish_tag(g),
                  'TagBuffer', 2, 'RelTol', 1e-10, 'MaxVCycles', 100, 'Verbose', 0, backend=OracleBackend())
    sj = GOLD['starfish']
    st = sol['stats']['stages'][-1]
    assert [lv['np'] for lv in sol['levels']] == sj['patchesPerLevel']
    assert [lv['cells'] for lv in sol['levels']] == sj['cellsPerLevel']
    assert st['visibleCells'] == sj['visibleCells']
    assert st['totalCells'] == sj['storedAmrCells']
    assert st['vcycles'] == sj['vcycles']
    assert st['finalRel'] <= 1e-10
    hist = np.asarray(st['resHist'])
    gold = np.asarray(GOLD['starfish_residual_history'])
    assert hist.shape == gold.shape
    # r_0 = max|F| over visible cells: source sampling + hierarchy, 1e-14
    assert abs(hist[0] - gold[0]) <= 1e-14 * gold[0]
    # every later residual to the round-off floor of the residual evaluation
    assert np.max(np.abs(hist - gold)) <= 1e-11 * gold[0], np.abs(hist - gold) / gold[0]
    # integrated equation balance (balanceDefect 4.87e-15): same order
    assert sol['mass']['rel'] < 1e-13
