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
    """G5: T1 uniform MMS with variable D, C, m = 32..256 (suite-output.txt:3-7)."""
    for g in GOLD['suite_T1_uniform_mms']:
        sol = ebSolve(vardc_problem(), 'BaseCells', g['m'], 'Verbose', 0, 'RelTol', 1e-11, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['vcycles'] == g['V']
        assert printed_close(sol['err']['linf'], g['err_inf']), (sol['err']['linf'], g['err_inf'])
        assert printed_close(sol['err']['l2'], g['err_l2']), (sol['err']['l2'], g['err_l2'])
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g['factor'])


@pytest.mark.parametrize('tree', [False, True])
@pytest.mark.parametrize('interp', ['qif', 'lif'])
@pytest.mark.parametrize('m0', [32, 64, 128, 256])
def test_box_in_box_T3(interp, m0, tree):
    """G5: T3 fixed box-in-box hierarchies, 2-4 levels, QC-ring and tree
    (suite-output.txt:17-44, 99-126): error, factor, V-cycles, mass defect
    < 1e-13."""
    key = 'suite_T3_box_in_box_tree' if tree else 'suite_T3_box_in_box'
    rows = [g for g in GOLD[key] if g['interp'] == interp and g['m0'] == m0]
    assert len(rows) == 3
    solve = ebtSolve if tree else ebSolve
    for g in rows:
        sol = solve(gauss51_problem(), 'BaseCells', g['m0'], 'MaxLevels', g['L'], 'Indicator', 'fun',
                    'TagFunction', box_in_box_tag, 'TagBuffer', 0, 'GhostInterp', interp, 'Verbose', 0,
                    'RelTol', 1e-10, 'MaxVCycles', 40, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['vcycles'] == g['V'], (g, st['vcycles'])
        assert printed_close(sol['err']['linf'], g['err']), (sol['err']['linf'], g)
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g)
        assert sol['mass']['rel'] < 1e-13


@pytest.mark.parametrize('tree', [False, True])
def test_h_independence_T6(tree):
    """T6 (runAllTests.m:148-155): the 2-level QIF V-cycle factor of T3 is
    h-independent, recorded to 3 significant digits for m0 = 32..256."""
    g = GOLD['suite_T6_h_independence_tree' if tree else 'suite_T6_h_independence']
    solve = ebtSolve if tree else ebSolve
    for m0, fac in zip(g['m0'], g['factors']):
        sol = solve(gauss51_problem(), 'BaseCells', m0, 'MaxLevels', 2, 'Indicator', 'fun',
                    'TagFunction', box_in_box_tag, 'TagBuffer', 0, 'GhostInterp', 'qif', 'Verbose', 0,
                    'RelTol', 1e-10, 'MaxVCycles', 40, backend=OracleBackend())
        assert printed_close(sol['stats']['stages'][-1]['avgFactor'], fac), (m0, fac)


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


@pytest.mark.slow
def test_starfish_history_gap_is_residual_roundoff():
    """The starfish residual history differs from the reference's recorded
    one by up to ~5e-12 r_0 (test_starfish_golden bounds it by 1e-11 r_0).
    That is the round-off floor of the residual maximum itself: moving every
    value of the converged solution by one or two units in the last place --
    the size of the difference that MATLAB's sparse LU of the coarsest
    operator and its libm leave between the two runs -- moves the residual
    maximum by the same order, while r_0 (which does not depend on the
    solution) matches to 1e-15."""
    import json
    import bench
    from bsam.flat import flatten
    from bsam_oracle import OracleHier
    H, opts = bench.starfish_hierarchy(OracleBackend())
    oh = OracleHier(flatten(H), opts)
    it, hist, rel, _ = oh.solve_cycles(opts.MaxVCycles + 2)
    gold = np.asarray(GOLD['starfish_residual_history'])
    r0 = hist[0]
    gap = np.abs(hist - gold) / r0
    assert gap[0] <= 1e-14 and 1e-13 < gap.max() <= 1e-11
    base = oh.residual()['linf']
    Q0 = oh.Q.copy()
    rng = np.random.Generator(np.random.PCG64(7))
    moved = []
    for _ in range(4):
        q = np.nextafter(Q0, rng.choice([-np.inf, np.inf], size=Q0.size))
        twice = rng.random(Q0.size) < 0.5
        q[twice] = np.nextafter(q[twice], np.where(q[twice] > Q0[twice], np.inf, -np.inf))
        oh.Q[:] = q
        moved.append(abs(oh.residual()['linf'] - base) / r0)
    oh.Q[:] = Q0
    # few-ulp solution differences move the residual max by ~1e-12 r_0: the
    # recorded history's gap is of that order, not a discrepancy of the path
    assert max(moved) >= 1e-13
    assert gap.max() <= 20 * max(moved), (gap.max(), moved)


def _solver(tree):
    return ebtSolve if tree else ebSolve


def _mass_order(value, printed):
    """A mass defect at round-off level: the same order of magnitude as the
    printed one (its digits are summation noise)."""
    return value <= 10 * float(printed) + 1e-15


@pytest.mark.parametrize('tree', [False, True])
def test_uniform_pure_neumann_T2(tree):
    """G5: T2 uniform singular pure-Neumann Poisson, m = 32..128
    (suite-output.txt T2 sections)."""
    from cases import pureneumann_problem
    rows = GOLD['suite_T2_pure_neumann' + ('_tree' if tree else '')][:3]
    for g in rows:
        sol = _solver(tree)(pureneumann_problem(), 'BaseCells', g['m'], 'Verbose', 0, 'RelTol', 1e-11,
                            backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['vcycles'] == g['V'], (g, st['vcycles'])
        assert printed_close(sol['err']['linf'], g['err_inf']), (sol['err']['linf'], g)
        assert printed_close(sol['err']['l2'], g['err_l2']), (sol['err']['l2'], g)
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g)


@pytest.mark.parametrize('tree', [False, True])
def test_lshape_T4(tree):
    """G5: T4 L-shaped refinement patch, m0 = 16, 32, 64: error, factor,
    number of level-2 patches (the reentrant corner needs two from m0 = 32)."""
    from cases import gauss52_problem, lshape_tag
    rows = GOLD['suite_T4_lshape' + ('_tree' if tree else '')][:3]
    for g in rows:
        sol = _solver(tree)(gauss52_problem(), 'BaseCells', g['m0'], 'MaxLevels', 2, 'Indicator', 'fun',
                            'TagFunction', lshape_tag, 'TagBuffer', 0, 'MinFillRatio', 0.9, 'Verbose', 0,
                            'RelTol', 1e-10, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert sol['levels'][1]['np'] == g['np2'], (g, sol['levels'][1]['np'])
        assert printed_close(sol['err']['linf'], g['err_inf']), (sol['err']['linf'], g)
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g)
        assert _mass_order(sol['mass']['rel'], g['mass']), (sol['mass']['rel'], g)


@pytest.mark.parametrize('tree', [False, True])
def test_fully_adaptive_T5(tree):
    """G5: T5 solution-driven adaptivity (undivided Laplacian, threshold
    1e-2 / 4^(L-1), buffer 2), MaxLevels 1..4: levels reached, errors,
    factor and the composite degrees of freedom."""
    from cases import threebumps_problem
    rows = GOLD['suite_T5_adaptive' + ('_tree' if tree else '')]
    for g in rows:
        sol = _solver(tree)(threebumps_problem(), 'BaseCells', 64, 'MaxLevels', g['MaxLevels'], 'Indicator', 'ulap',
                            'TagThreshold', lambda L: 1e-2 / 4 ** (L - 1), 'TagBuffer', 2, 'Verbose', 0,
                            'RelTol', 1e-10, 'MaxVCycles', 40, backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert len(sol['levels']) == g['got']
        assert sol['err']['dof'] == g['dof'], (sol['err']['dof'], g)
        assert printed_close(sol['err']['linf'], g['err_inf']), (sol['err']['linf'], g)
        assert printed_close(sol['err']['l2'], g['err_l2']), (sol['err']['l2'], g)
        assert printed_close(st['avgFactor'], g['factor']), (st['avgFactor'], g)


@pytest.mark.parametrize('tree', [False, True])
def test_mass_conservation_T7(tree):
    """G5: T7 discrete mass conservation: with the flux corrections the
    defect is round-off; without them it is the recorded O(1e-5..1e-4)."""
    rows = GOLD['suite_T7_mass' + ('_tree' if tree else '')]
    for g in rows:
        sol = _solver(tree)(gauss51_problem(), 'BaseCells', 64, 'MaxLevels', g['levels'], 'Indicator', 'fun',
                            'TagFunction', box_in_box_tag, 'TagBuffer', 0, 'MassCorrection', bool(g['corrections']),
                            'Verbose', 0, 'RelTol', 1e-11, 'MaxVCycles', 60, backend=OracleBackend())
        assert printed_close(sol['err']['linf'], g['err']), (sol['err']['linf'], g)
        if g['corrections']:
            assert sol['mass']['rel'] < 1e-14
        else:
            assert printed_close(sol['mass']['rel'], g['mass']), (sol['mass']['rel'], g)


@pytest.mark.parametrize('tree', [False, True])
def test_scattered_tagging_T8(tree):
    """G5: T8 24 random tag disks (rng 42): patch count, minimum width,
    factor, error, mass."""
    from cases import scattered_tag
    g = GOLD['suite_T8_scattered' + ('_tree' if tree else '')][0]
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        sol = _solver(tree)(vardc_problem(), 'BaseCells', 64, 'MaxLevels', 3, 'Indicator', 'fun',
                            'TagFunction', scattered_tag(), 'TagBuffer', 1, 'MinBoxWidth', 4, 'Verbose', 0,
                            'RelTol', 1e-10, 'MaxVCycles', 60, backend=OracleBackend())
    npat = sum(lv['np'] for lv in sol['levels'][1:])
    minw = min(int(min((lv['box'][:, 1] - lv['box'][:, 0] + 1).min(), (lv['box'][:, 3] - lv['box'][:, 2] + 1).min()))
               for lv in sol['levels'][1:])
    st = sol['stats']['stages'][-1]
    assert npat == g['patches'] and minw == g['minw'], (npat, minw, g)
    # the factor divides the last residual (~1e-13 of r_0, where the coarsest
    # solve's round-off -- MATLAB's sparse LU here a dense inverse -- shows):
    # to its printed digit, with that slack
    assert abs(st['avgFactor'] - float(g['factor'])) <= 1.5e-3, (st['avgFactor'], g)
    assert printed_close(sol['err']['linf'], g['err']), (sol['err']['linf'], g)
    assert _mass_order(sol['mass']['rel'], g['mass']), (sol['mass']['rel'], g)
