"""The reference's parabolic suite (ParabolicBSAM/tests/runParabolicTests.m
P1-P4) and its regressions (runParabolicRegressions.m) through ebpSolve on
the oracle: every recorded line of suite-output.txt reproduced to its
printed digits (temporal Cauchy differences of BE / BDF2 / CN, the joint
h-Dt refinement with regrids, 200 heat steps with 39 conservative regrids,
the rotating-source tracking mesh, the large-step BE bound, the CN
time-dependent coefficient orders and composite mass).  GPU: the CUDA path
reproduces the oracle's P1b pipeline (time-dependent Dirichlet data,
regrids every two steps) bit for bit.
"""
import json
import os
import warnings

import numpy as np
import pytest

from bsam.parabolic import ebpProblem, ebpSolve, ebpOptions
from bsam_oracle import OracleBackend
from cases import printed_close

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), 'golden', 'reference_outputs.json')))['suite_parabolic']


def bump_problem():
    """Travelling Gaussian MMS, du/dt - lap u + u = f (runParabolicTests.m:22-29)."""
    sg, vx, vy = 0.06, 0.4, 0.3
    xc = lambda t: 0.30 + vx * t
    yc = lambda t: 0.35 + vy * t
    uex = lambda x, y, t: np.exp(-((x - xc(t)) ** 2 + (y - yc(t)) ** 2) / (2 * sg ** 2))
    ut = lambda x, y, t: uex(x, y, t) * ((x - xc(t)) * vx + (y - yc(t)) * vy) / sg ** 2
    lap = lambda x, y, t: uex(x, y, t) * (((x - xc(t)) ** 2 + (y - yc(t)) ** 2) / sg ** 4 - 2 / sg ** 2)
    ff = lambda x, y, t: ut(x, y, t) - lap(x, y, t) + uex(x, y, t)
    return ebpProblem([0, 1, 0, 1], 1, 1, ff, ('dirichlet', uex), lambda x, y: uex(x, y, 0), uex)


def heat2_problem():
    """Variable-D heat equation, Neumann, two bumps (runParabolicTests.m:88-91)."""
    D2 = lambda x, y: 1 + 0.5 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    u02 = lambda x, y: (0.5 + np.exp(-((x - 0.35) ** 2 + (y - 0.4) ** 2) / (2 * 0.03 ** 2))
                        + 0.7 * np.exp(-((x - 0.7) ** 2 + (y - 0.65) ** 2) / (2 * 0.04 ** 2)))
    return ebpProblem([0, 1, 0, 1], D2, 0, 0, ('neumann', 0), u02)


def p1b_solve(j, backend):
    """runParabolicTests.m:66-77."""
    thr = 5e-2 / 4 ** j
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return ebpSolve(bump_problem(), 'Scheme', 'bdf2', 'Dt', 0.05 / 2 ** j, 'TFinal', 0.4, 'RegridEvery', 2,
                        'StepVerbose', 0, 'BaseCells', [32 * 2 ** j] * 2, 'MaxLevels', 2, 'Indicator', 'ulap',
                        'TagThreshold', lambda L: thr / 4 ** (L - 1), 'TagBuffer', 3, 'RelTol', 1e-9,
                        backend=backend)


@pytest.mark.parametrize('scheme', ['be', 'bdf2', 'cn'])
def test_P1a_temporal_cauchy_differences(scheme):
    """Same-grid Dt-Cauchy differences on a uniform 128^2 mesh."""
    U = []
    for dt in 0.04 / 2 ** np.arange(4):
        s = ebpSolve(bump_problem(), 'Scheme', scheme, 'Dt', dt, 'TFinal', 0.4, 'RegridEvery', 0, 'StepVerbose', 0,
                     'BaseCells', [128, 128], 'MaxLevels', 1, 'RelTol', 1e-10, backend=OracleBackend())
        U.append(s['H'].lev[s['H'].nlev].Q[0][1:-1, 1:-1].copy())
    diffs = [float(np.max(np.abs(U[j] - U[j + 1]))) for j in range(3)]
    for d, g in zip(diffs, GOLD['P1a'][scheme]):
        assert printed_close(d, g), (scheme, diffs, GOLD['P1a'][scheme])


@pytest.mark.parametrize('j', range(3))
def test_P1b_joint_refinement_with_regrids(j):
    g = GOLD['P1b'][j]
    s = p1b_solve(j, OracleBackend())
    assert printed_close(s['err']['linf'], g['err_inf']), (s['err'], g)
    assert printed_close(float(np.mean(s['cycles'])), g['meanV'])
    assert s['nregrids'] == g['regrids']


def test_P2_heat_mass_across_regrids_and_P4_warm_start(capsys):
    s = ebpSolve(heat2_problem(), 'Scheme', 'bdf2', 'Dt', 2e-3, 'TFinal', 0.4, 'RegridEvery', 5, 'StepVerbose', 50,
                 'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'ulap',
                 'TagThreshold', lambda L: 1e-3 / 4 ** (L - 1), 'TagBuffer', 2, 'RelTol', 1e-9,
                 backend=OracleBackend())
    g = GOLD['P2']
    assert len(s['cycles']) == g['steps'] and s['nregrids'] == g['regrids']
    assert printed_close(float(np.mean(s['cycles'])), g['meanV'])
    assert printed_close(float(np.mean(s['cycles'])), GOLD['P4']['meanV'])
    drift = float(np.max(np.abs(s['mass'] - s['mass'][0])))
    assert printed_close(drift, g['drift']), (drift, g)
    assert printed_close(float(s['mass'][0]), g['mass'])
    assert len(s['levels']) == g['final_levels']
    for st in GOLD['P2_steps']:
        n = st['step']
        assert int(s['cycles'][n - 1]) == st['V']
        assert printed_close(float(s['relres'][n - 1]), st['rel'])
        assert printed_close(float(s['mass'][n]), st['mass'])
    # the step lines the driver printed are the recorded ones
    out = capsys.readouterr().out
    for st in GOLD['P2_steps']:
        assert f"step {st['step']:4d}/200" in out and f"mass={st['mass']}" in out


def test_P3_rotating_source_tracking():
    om, Rc, ss = 2 * np.pi, 0.22, 0.03
    cx = lambda t: 0.5 + Rc * np.cos(om * t)
    cy = lambda t: 0.5 + Rc * np.sin(om * t)
    src = lambda x, y, t: 25 * np.exp(-((x - cx(t)) ** 2 + (y - cy(t)) ** 2) / (2 * ss ** 2))
    p3 = ebpProblem([0, 1, 0, 1], 1, 0, src, ('dirichlet', 0), lambda x, y: 0 * x)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        s = ebpSolve(p3, 'Scheme', 'bdf2', 'Dt', 5e-3, 'TFinal', 1.0, 'RegridEvery', 4, 'StepVerbose', 0,
                     'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'ulap',
                     'TagThreshold', lambda L: 2e-3 / 4 ** (L - 1), 'TagBuffer', 3, 'RelTol', 1e-8,
                     backend=OracleBackend())
    g = GOLD['P3']
    H = s['H']
    lev = H.lev[H.nlev]
    covered = any(b[0] - 1 <= cx(1.0) / lev.h[0] <= b[1] and b[2] - 1 <= cy(1.0) / lev.h[1] <= b[3]
                  for b in lev.box)
    assert int(covered) == g['covered']
    assert sum(lv['cells'] for lv in s['levels']) == g['cells']
    assert s['nregrids'] == g['regrids']
    assert printed_close(float(np.mean(s['cycles'])), g['meanV'])


def test_P4_large_step_backward_euler_bounded():
    s = ebpSolve(heat2_problem(), 'Scheme', 'be', 'Dt', 0.1, 'TFinal', 0.5, 'RegridEvery', 0, 'StepVerbose', 0,
                 'BaseCells', [64, 64], 'MaxLevels', 1, 'RelTol', 1e-9, backend=OracleBackend())
    H = s['H']
    umax = max(float(np.max(np.abs(q))) for q in H.lev[H.nlev].Q)
    assert printed_close(umax, GOLD['P4']['umax_big_dt'])


def test_cn_time_dependent_reaction_order():
    """runParabolicRegressions.m:5-20: C(t) = 1 + t, spatially constant u."""
    p = ebpProblem([0, 1, 0, 1], 1, lambda x, y, t: 1 + t, lambda x, y, t: t * np.exp(-t), ('neumann', 0),
                   lambda x, y: np.ones(np.shape(x)), lambda x, y, t: np.exp(-t) * np.ones(np.shape(x)))
    e = []
    for dt in (0.1, 0.05, 0.025, 0.0125):
        s = ebpSolve(p, 'Scheme', 'cn', 'Dt', dt, 'TFinal', 0.4, 'BaseCells', [8, 8], 'MaxLevels', 1,
                     'CoarsestCells', 4, 'StepVerbose', 0, 'RegridEvery', 0, 'RelTol', 1e-12, backend=OracleBackend())
        e.append(float(np.max(np.abs(s['H'].lev[s['H'].nlev].Q[0][1:-1, 1:-1] - np.exp(-0.4)))))
    for v, g in zip(e, GOLD['CN_reaction_errors']):
        assert printed_close(v, g), (e, GOLD['CN_reaction_errors'])
    assert all(np.log2(np.array(e[:-1]) / np.array(e[1:])) > 1.8)


def test_cn_time_dependent_diffusion_and_boundary_order():
    """runParabolicRegressions.m:21-41: D(t) = 1 + t, time-dependent
    Dirichlet data, same-grid Cauchy differences."""
    u = lambda x, y, t: np.exp(-t) * (1 + x ** 2 + y ** 2)
    f = lambda x, y, t: -u(x, y, t) - 4 * (1 + t) * np.exp(-t)
    p = ebpProblem([0, 1, 0, 1], lambda x, y, t: 1 + t, 0, f, ('dirichlet', u), lambda x, y: u(x, y, 0), u)
    U = []
    for dt in (0.1, 0.05, 0.025, 0.0125):
        s = ebpSolve(p, 'Scheme', 'cn', 'Dt', dt, 'TFinal', 0.4, 'BaseCells', [16, 16], 'MaxLevels', 1,
                     'CoarsestCells', 4, 'StepVerbose', 0, 'RegridEvery', 0, 'RelTol', 1e-12, backend=OracleBackend())
        U.append(s['H'].lev[s['H'].nlev].Q[0][1:-1, 1:-1].copy())
    d = [float(np.max(np.abs(U[j] - U[j + 1]))) for j in range(3)]
    for v, g in zip(d, GOLD['CN_diffusion_cauchy']):
        assert printed_close(v, g), (d, GOLD['CN_diffusion_cauchy'])


@pytest.mark.parametrize('regrid', [0, 2])
def test_cn_composite_mass(regrid):
    """runParabolicRegressions.m:42-56: a fixed fine patch across a
    nonconstant profile; the composite mass telescopes."""
    p = ebpProblem([0, 1, 0, 1], lambda x, y: 1 + 0.2 * x, 0, 0, ('neumann', 0),
                   lambda x, y: 1 + 0.2 * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y))
    s = ebpSolve(p, 'Scheme', 'cn', 'Dt', 0.002, 'TFinal', 0.02, 'BaseCells', [16, 16], 'MaxLevels', 2,
                 'CoarsestCells', 4, 'Indicator', 'fun',
                 'TagFunction', lambda x, y: (x > 0.25) & (x < 0.625) & (y > 0.25) & (y < 0.75),
                 'TagBuffer', 1, 'StepVerbose', 0, 'RegridEvery', regrid, 'RelTol', 1e-11, backend=OracleBackend())
    g = next(c for c in GOLD['CN_mass'] if c['regrid'] == regrid)
    assert len(s['levels']) == 2
    drift = float(np.max(np.abs(s['mass'] - s['mass'][0])))
    assert drift < 2e-10                       # the reference's bound; the recorded 1.859e-13 is round-off
    assert printed_close(float(np.max(s['relres'])), g['rel'])


@pytest.mark.parametrize('bad', [0, -0.1, np.nan, np.inf])
def test_invalid_time_step_rejected(bad):
    with pytest.raises(ValueError, match='ebp_options:time'):
        ebpOptions('Dt', bad, 'TFinal', 1)


@pytest.mark.gpu
def test_P1b_device_matches_oracle_pipeline():
    from bsam.device import DeviceBackend
    a = p1b_solve(0, OracleBackend())
    b = p1b_solve(0, DeviceBackend.get(0))
    np.testing.assert_array_equal(a['cycles'], b['cycles'])
    np.testing.assert_array_equal(a['relres'], b['relres'])
    assert a['nregrids'] == b['nregrids']
    Ha, Hb = a['H'], b['H']
    assert Ha.nlev == Hb.nlev
    for k in range(Ha.rootIdx, Ha.nlev + 1):
        for qa, qb in zip(Ha.lev[k].Q, Hb.lev[k].Q):
            np.testing.assert_array_equal(qa, qb)
    assert a['err'] == b['err']


@pytest.mark.parametrize('name,bad', [('RegridEvery', -1), ('RegridEvery', 2.5), ('StepVerbose', np.inf),
                                      ('MaxVCyclesStep', 0), ('Callback', 3)])
def test_invalid_time_options_rejected(name, bad):
    """ebpOptions.m:47-54."""
    with pytest.raises(ValueError, match='ebp_options:'):
        ebpOptions('Dt', 0.1, 'TFinal', 1, name, bad)


def test_callback_called_after_every_step():
    seen = []
    s = ebpSolve(heat2_problem(), 'Scheme', 'be', 'Dt', 0.1, 'TFinal', 0.3, 'RegridEvery', 0, 'StepVerbose', 0,
                 'BaseCells', [32, 32], 'MaxLevels', 1, 'RelTol', 1e-9,
                 'Callback', lambda H, t, n: seen.append((round(t, 12), n)), backend=OracleBackend())
    assert seen == [(0.1, 1), (0.2, 2), (0.3, 3)]
    assert len(s['cycles']) == 3
