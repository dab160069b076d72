"""Mixed-precision form (Precision 'mixed'): FP32 FAS V-cycles on the
correction inside an FP64 defect-correction loop.

The FP64 oracle (C restatement of the reference) gives the reference
solution; the mixed solve must reach the same FP64 stop test (composite
relative residual 1e-10) and stay within 1e-9 relative L2 and max error of
the oracle's solution over the visible cells, the tolerance of the mixed
form.  A batch of mixed solves equals the same solves alone, bit for bit.
"""
import numpy as np
import pytest

from bsam import ebOptions
from bsam.flat import flatten, visible_q_index, rel_errors
from bsam.solve import build_hierarchy
from bsam_oracle import OracleBackend, OracleHier
from cases import config1_problem, vardc_problem, pureneumann_problem

pytestmark = pytest.mark.gpu

TOL = 1e-9

CIRCLE = lambda x, y: (x - 0.4) ** 2 + (y - 0.55) ** 2 < 0.04
BAND = lambda x, y: np.abs(x - y) < 0.15


def _opts(tag, precision, levels=3):
    return ebOptions('BaseCells', 32, 'MaxLevels', levels, 'Indicator', 'fun', 'TagFunction', tag, 'Verbose', 0,
                     'RelTol', 1e-10, 'Precision', precision)


def _solve_mixed_and_oracle(prob, tag, levels=3, mass=True, tree=False):
    o64 = _opts(tag, 'fp64', levels)
    o64['MassCorrection'] = mass
    H = build_hierarchy(prob, o64, OracleBackend(), tree=tree)
    fl = flatten(H)
    oh = OracleHier(fl, o64)
    it_o, hist_o, rel_o, _ = oh.solve_cycles(o64.MaxVCycles + 2)
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q
    om = o64.copy()
    om['Precision'] = 'mixed'
    dh = DevHier(DeviceBackend.get(0).ctx, fl, om)
    it_m, hist_m, rel_m, _ = dh.solve_cycles(om.MaxVCycles + 2)
    Qm = dh.get(BSAM_FIELD_Q, fl.Q.size)
    return fl, (it_o, hist_o, rel_o, oh.Q), (it_m, hist_m, rel_m, Qm)


@pytest.mark.parametrize('case', ['config1-circle', 'config1-band', 'vardc-band', 'vardc-band-nomass',
                                  'neumann-circle', 'vardc-band-tree', 'config1-circle-tree'])
def test_mixed_matches_fp64_oracle(case):
    prob = {'config1': config1_problem, 'vardc': vardc_problem, 'neumann': pureneumann_problem}[case.split('-')[0]]()
    tag = BAND if 'band' in case else CIRCLE
    levels = 2 if case.startswith('neumann') else 3
    fl, o, m = _solve_mixed_and_oracle(prob, tag, levels, mass='nomass' not in case, tree=case.endswith('-tree'))
    assert m[2] <= 1e-10, m[2]
    # the defect correction converges like the FP64 V-cycle
    assert m[0] <= o[0] + 2, (m[0], o[0])
    assert m[1][0] == o[1][0]          # same initial FP64 residual
    idx = visible_q_index(fl)
    qm, qo = m[3].copy(), o[3].copy()
    if fl.singular:
        # all-Neumann, C = 0: solutions are fixed up to a constant, which the
        # FP32 correction cycle and the FP64 V-cycle pin differently; compare
        # mean-free solutions (what ebSolve's MeanZero returns)
        qm[idx] -= qm[idx].mean()
        qo[idx] -= qo[idx].mean()
    l2, mx = rel_errors(qm, qo, idx)
    assert l2 <= TOL and mx <= TOL, (l2, mx)


def test_mixed_non_power_of_two_spacing():
    """[0,3] x [0,1.5]: the FP32 correction cycle divides by h^2 in FP32;
    the mixed solve still reaches the FP64 stop test within the tolerance."""
    from bsam import ebProblem
    D = lambda x, y: 1 + 0.2 * x * y
    f = lambda x, y: np.sin(2 * x) * np.cos(3 * y) + 0.5
    prob = ebProblem([0, 3, 0, 1.5], D, 1, f, ('dirichlet', 0))
    fl, o, m = _solve_mixed_and_oracle(prob, lambda x, y: np.abs(x - 2 * y) < 0.3)
    assert m[2] <= 1e-10 and m[0] <= o[0] + 2, (m[0], o[0], m[2])
    l2, mx = rel_errors(m[3], o[3], visible_q_index(fl))
    assert l2 <= TOL and mx <= TOL, (l2, mx)


@pytest.mark.parametrize('form', [None, '5'])
def test_mixed_batch_equals_solo(form, monkeypatch):
    """Instances with different level counts merged into one mixed batch
    give their solo results bit for bit (the consistency step's fills reach
    an instance's finest level below the batch's); form '5' forces the
    distributed-shared-memory smoother where a level fits it."""
    if form is not None:
        monkeypatch.setenv('BSAM_RELAX_N', form)
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q
    from bsam.batch import merge_flats, split_field
    from bsam.flat import FIELD_Q
    be = DeviceBackend.get(0)
    cases = [(config1_problem(), CIRCLE, 3), (vardc_problem(), BAND, 3), (config1_problem(), BAND, 2)]
    parts = []
    for prob, tag, lv in cases:
        parts.append(flatten(build_hierarchy(prob, _opts(tag, 'mixed', lv), OracleBackend())))
    om = _opts(CIRCLE, 'mixed')
    solo = []
    for p in parts:
        dh = DevHier(be.ctx, p, om)
        r = dh.solve_cycles(om.MaxVCycles + 2)
        solo.append((r, dh.get(BSAM_FIELD_Q, p.Q.size)))
    b = merge_flats(parts)
    bh = DevHier(be.ctx, b, om)
    bh.solve_cycles(om.MaxVCycles + 2)
    Q = bh.get(BSAM_FIELD_Q, b.Q.size)
    for i, (r, q) in enumerate(solo):
        rb = bh.batch_result(i, om.MaxVCycles + 2)
        assert rb[0] == r[0]
        np.testing.assert_array_equal(rb[1], r[1])
        np.testing.assert_array_equal(split_field(b, FIELD_Q, Q, i), q)
