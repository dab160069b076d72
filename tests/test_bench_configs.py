"""GPU parity on the configurations the benchmark times.

Each case solves the benchmarked workload on the device and on the C oracle
(the CPU restatement of the reference's solve path) and compares them: bit
for bit on the FP64 path (residual history, V-cycle count, final relative
residual and every solution, coarse-shadow and force value), within the
precision form's stated 1e-9 relative L2 / max tolerance on the mixed path.

  * the diffuse-domain starfish of examples/demoStarfish.m:11-20 (543,384
    stored cells, 10 V-cycles), FP64 and mixed;
  * seeded instances of the batched random-coefficient workload, among them
    the slowest (51 V-cycles) and the largest, each through ebSolve's
    solution-driven pipeline (ebSolve.m:38-52) on both paths, then solved
    alone and as one batch;
  * the README heat example (ParabolicBSAM/src/ebpSolve.m:23-78, BDF2,
    50 steps with regrids every 5) at BaseCells 32 / 3 levels and 128 / 4;
  * the README elliptic example through the solution-driven pipeline, on
    the QC-ring hierarchy (ebSolve) and the single-parent tree (ebtSolve),
    to relative residual 1e-10.
"""
import warnings

import numpy as np
import pytest

from bsam.flat import flatten, visible_q_index, rel_errors, FIELD_Q
from bsam_oracle import OracleBackend, OracleHier
from cases import config1_problem, starfish_config2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-9


def dev():
    from bsam.device import DeviceBackend
    return DeviceBackend.get(0)


def _tables_equal(a, b):
    """Two flat hierarchies are the same upload: every array and count equal."""
    assert a.nlev == b.nlev and a.rootIdx == b.rootIdx and a.npatch == b.npatch
    for name, va in vars(a).items():
        vb = getattr(b, name)
        if isinstance(va, np.ndarray):
            np.testing.assert_array_equal(va, vb, err_msg=name)


def _solve_both(fl, opts):
    from bsam.device import DevHier, BSAM_FIELD_Q, BSAM_FIELD_QC, BSAM_FIELD_F
    oh = OracleHier(fl, opts)
    o = oh.solve_cycles(opts.MaxVCycles + 2)
    dh = DevHier(dev().ctx, fl, opts)
    d = dh.solve_cycles(opts.MaxVCycles + 2)
    state_d = (dh.get(BSAM_FIELD_Q, fl.Q.size), dh.get(BSAM_FIELD_QC, fl.QC.size), dh.get(BSAM_FIELD_F, fl.F.size))
    return o, (oh.Q, oh.QC, oh.F), d, state_d, dh


def _assert_same_solve(o, so, d, sd):
    assert o[0] == d[0], (o[0], d[0])                 # V-cycles
    np.testing.assert_array_equal(o[1], d[1])         # residual history
    assert o[2] == d[2]                               # final relative residual
    assert o[3] == d[3]                               # visible cells
    for a, b, name in zip(so, sd, ('Q', 'QC', 'F')):
        np.testing.assert_array_equal(a, b, err_msg=name)


@pytest.fixture(scope='module')
def starfish():
    """The starfish hierarchy built with the oracle's set-up steps and with
    the device's (the benchmark builds it on the device): identical uploads."""
    Ho, opts = starfish_config2(OracleBackend())
    Hd, _ = starfish_config2(dev())
    flo, fld = flatten(Ho), flatten(Hd)
    _tables_equal(flo, fld)
    return flo, opts


def test_config2_starfish_fp64_bitwise(starfish):
    fl, opts = starfish
    # the reference's recorded hierarchy (verification/starfish-full.json:
    # 543,384 stored cells at and above the root, cellsPerLevel)
    cells = [int(fl.levels[k, 5] - fl.levels[k, 4]) for k in range(fl.nlev)]
    assert cells[2:] == [4096, 11328, 33668, 114756, 379536] and sum(cells[2:]) == 543384, cells
    o, so, d, sd, _ = _solve_both(fl, opts)
    assert d[0] == 10 and len(d[1]) == 11 and d[2] <= 1e-10
    _assert_same_solve(o, so, d, sd)


def test_config2_starfish_mixed_within_tolerance(starfish):
    from bsam.device import DevHier, BSAM_FIELD_Q
    fl, opts = starfish
    oh = OracleHier(fl, opts)
    it_o, hist_o, rel_o, _ = oh.solve_cycles(opts.MaxVCycles + 2)
    om = opts.copy()
    om['Precision'] = 'mixed'
    dh = DevHier(dev().ctx, fl, om)
    it_m, hist_m, rel_m, _ = dh.solve_cycles(om.MaxVCycles + 2)
    assert rel_m <= 1e-10 and it_m <= it_o + 1, (it_m, it_o, rel_m)
    assert hist_m[0] == hist_o[0]
    l2, mx = rel_errors(dh.get(BSAM_FIELD_Q, fl.Q.size), oh.Q, visible_q_index(fl))
    assert l2 <= MIXED_TOL and mx <= MIXED_TOL, (l2, mx)


# seeds of the batched workload (instance i uses seed 1000 + i): the slowest
# (1090: 51 V-cycles), the next slowest (1214: 42), the deepest (1020: six
# levels), the largest (1066: 100,276 cells), a MaxLevels-2 instance on a
# 128^2 base (1171), and the first three of the benchmark's batch
CONFIG4_SEEDS = (1090, 1214, 1020, 1066, 1171, 1000, 1001, 1002)


def test_config4_instances_bitwise_solo_and_batch():
    from bsam.instances import random_elliptic, final_stage
    from bsam.batch import merge_flats, split_field
    from bsam.device import DevHier, BSAM_FIELD_Q
    parts, opts, solo = [], None, []
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        for s in CONFIG4_SEEDS:
            prob, o = random_elliptic(s)
            flo, Ho = final_stage(prob, o, OracleBackend())
            fld, _ = final_stage(prob, o, dev())          # the pipeline's earlier stages on the device
            _tables_equal(flo, fld)
            opts = opts or Ho.opts
            oo, so, dd, sd, _ = _solve_both(flo, Ho.opts)
            _assert_same_solve(oo, so, dd, sd)
            parts.append(flo)
            solo.append((dd, sd[0]))
    its = [r[0][0] for r in solo]
    assert max(its) == 51 and len({p.nlev for p in parts}) > 2, its
    b = merge_flats(parts)
    bh = DevHier(dev().ctx, b, opts)
    bh.solve_cycles(opts.MaxVCycles + 2)
    Q = bh.get(BSAM_FIELD_Q, b.Q.size)
    for i, (r, q) in enumerate(solo):
        rb = bh.batch_result(i, opts.MaxVCycles + 2)
        assert rb[0] == r[0], (i, rb[0], r[0])
        np.testing.assert_array_equal(rb[1], r[1])
        np.testing.assert_array_equal(split_field(b, FIELD_Q, Q, i), q)


@pytest.mark.parametrize('base,levels', [(32, 3), (128, 4)])
def test_config3_heat_full_run_bitwise(base, levels):
    """The whole 50-step BDF2 run (nine regrids), device pipeline vs oracle
    pipeline: per-step V-cycles and residuals, the final hierarchy's
    solution and BDF2 history bit for bit; composite mass per step to the
    reduction-order tolerance (the device sums in another order)."""
    from bsam.parabolic import ebpProblem, ebpSolve
    u0 = lambda x, y: 1 + 0.2 * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    prob = ebpProblem([0, 1, 0, 1], 1, 0, 0, ('neumann', 0), u0)
    kw = dict(Scheme='bdf2', Dt=0.002, TFinal=0.1, BaseCells=base, MaxLevels=levels, RegridEvery=5, StepVerbose=0)
    a = ebpSolve(prob, *sum(kw.items(), ()), backend=OracleBackend())
    b = ebpSolve(prob, *sum(kw.items(), ()), backend=dev())
    assert len(a['cycles']) == len(b['cycles']) == 50
    assert a['nregrids'] == b['nregrids'] == 9
    np.testing.assert_array_equal(a['cycles'], b['cycles'])
    np.testing.assert_array_equal(a['relres'], b['relres'])
    np.testing.assert_allclose(a['mass'], b['mass'], rtol=1e-13, atol=0)
    Ha, Hb = a['H'], b['H']
    assert Ha.nlev == Hb.nlev
    for k in range(1, Ha.nlev + 1):
        for qa, qb in zip(Ha.lev[k].Q, Hb.lev[k].Q):
            np.testing.assert_array_equal(qa[1:-1, 1:-1], qb[1:-1, 1:-1])
    for kp in Ha.par['Uo']:
        np.testing.assert_array_equal(Ha.par['Uo'][kp], Hb.par['Uo'][kp])
        np.testing.assert_array_equal(Ha.par['Uoo'][kp], Hb.par['Uoo'][kp])


@pytest.mark.parametrize('tree', [False, True])
def test_config1_solution_driven_pipeline_bitwise(tree):
    """BaseCells 32, MaxLevels 3, TagThreshold 1e-2, RelTol 1e-10: every
    stage (solve, tag on the solution, add a level) on both paths; the
    same boxes, stage histories and final field."""
    from bsam.solve import ebSolve, ebtSolve
    solve = ebtSolve if tree else ebSolve
    p = config1_problem()
    kw = ('BaseCells', 32, 'MaxLevels', 3, 'TagThreshold', 1e-2, 'RelTol', 1e-10, 'Verbose', 0)
    a = solve(p, *kw, backend=OracleBackend())
    b = solve(p, *kw, backend=dev())
    assert len(a['stats']['stages']) == len(b['stats']['stages']) == 3
    for sa, sb in zip(a['stats']['stages'], b['stats']['stages']):
        assert sa['vcycles'] == sb['vcycles']
        np.testing.assert_array_equal(sa['resHist'], sb['resHist'])
        assert sa['finalRel'] == sb['finalRel'] and sa['finalRel'] <= 1e-10
    for la, lb in zip(a['levels'], b['levels']):
        np.testing.assert_array_equal(la['box'], lb['box'])
    for k in range(1, a['H'].nlev + 1):
        for qa, qb in zip(a['H'].lev[k].Q, b['H'].lev[k].Q):
            np.testing.assert_array_equal(qa, qb)
