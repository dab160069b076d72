"""Parabolic driver (config 3): BDF2 heat diffusion with regrids.

Pinned to the reference's README heat example (verification/readme-
examples.txt:23-27: V, rel, levels, cells, mass at steps 10..50) on the
oracle; on the GPU the whole pipeline (set-up fills, regrid transfers, every
step's solve) must match the oracle pipeline bit for bit.
"""
import json
import os

import numpy as np
import pytest

from bsam.parabolic import ebpProblem, ebpSolve
from bsam_oracle import OracleBackend
from cases import printed_close

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), 'golden', 'reference_outputs.json')))


def heat_problem():
    u0 = lambda x, y: 1 + 0.2 * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    return ebpProblem([0, 1, 0, 1], 1, 0, 0, ('neumann', 0), u0)


def _step_lines(sol):
    out = {}
    for n in (10, 20, 30, 40, 50):
        out[n] = (int(sol['cycles'][n - 1]), float(sol['relres'][n - 1]), float(sol['mass'][n]))
    return out


def test_heat_readme_example_golden():
    sol = ebpSolve(heat_problem(), 'Scheme', 'bdf2', 'Dt', 0.002, 'TFinal', 0.1, 'BaseCells', 32,
                   'MaxLevels', 3, 'RegridEvery', 5, 'StepVerbose', 0, backend=OracleBackend())
    gold = {g['step']: g for g in GOLD['readme_heat_steps']}
    lines = _step_lines(sol)
    for n, g in gold.items():
        V, rel, mass = lines[n]
        assert V == g['V'], (n, V, g)
        assert printed_close(rel, g['rel']), (n, rel, g)
        assert printed_close(mass, g['mass']), (n, mass, g)
    # conservative scheme: total composite mass drift below the reference's
    # regression bound (ParabolicBSAM/tests/runParabolicRegressions.m: 2e-10)
    assert np.max(np.abs(sol['mass'] - sol['mass'][0])) < 2e-10
    assert sol['nregrids'] == 9


@pytest.mark.gpu
def test_heat_device_matches_oracle_pipeline():
    from bsam.device import DeviceBackend
    kw = dict(Scheme='bdf2', Dt=0.002, TFinal=0.024, BaseCells=32, MaxLevels=3, RegridEvery=5, StepVerbose=0)
    a = ebpSolve(heat_problem(), *sum(kw.items(), ()), backend=OracleBackend())
    b = ebpSolve(heat_problem(), *sum(kw.items(), ()), backend=DeviceBackend.get(0))
    np.testing.assert_array_equal(a['cycles'], b['cycles'])
    np.testing.assert_array_equal(a['relres'], b['relres'])
    Ha, Hb = a['H'], b['H']
    assert Ha.nlev == Hb.nlev
    for k in range(1, Ha.nlev + 1):
        for qa, qb in zip(Ha.lev[k].Q, Hb.lev[k].Q):
            np.testing.assert_array_equal(qa[1:-1, 1:-1], qb[1:-1, 1:-1])
    np.testing.assert_allclose(a['mass'], b['mass'], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_time_dependent_device_matches_oracle_pipeline():
    """Time-dependent D, C, f and boundary data: every step refreshes the
    coefficients (incremental upload) and samples f for the device right-hand
    side; the device pipeline (state resident between steps) still equals the
    oracle's bit for bit, through BE, BDF2 and two regrids."""
    from bsam.device import DeviceBackend
    D = lambda x, y, t: 1 + 0.3 * np.sin(np.pi * x) * np.cos(t)
    C = lambda x, y, t: 0.5 + 0 * x + 0.1 * t
    f = lambda x, y, t: np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.02) * (1 + t)
    g = lambda x, y, t: 0.1 * t + 0 * x
    u0 = lambda x, y: 1 + 0.2 * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    prob = ebpProblem([0, 1, 0, 1], D, C, f, ('dirichlet', g), u0)
    kw = dict(Scheme='bdf2', Dt=0.004, TFinal=0.048, BaseCells=32, MaxLevels=3, RegridEvery=5, StepVerbose=0)
    a = ebpSolve(prob, *sum(kw.items(), ()), backend=OracleBackend())
    b = ebpSolve(prob, *sum(kw.items(), ()), backend=DeviceBackend.get(0))
    assert a['nregrids'] == b['nregrids'] == 2
    np.testing.assert_array_equal(a['cycles'], b['cycles'])
    np.testing.assert_array_equal(a['relres'], b['relres'])
    # composite sums are reduced in another order on the device
    np.testing.assert_allclose(a['mass'], b['mass'], rtol=1e-13, atol=0)
    Ha, Hb = a['H'], b['H']
    for k in range(1, Ha.nlev + 1):
        for qa, qb in zip(Ha.lev[k].Q, Hb.lev[k].Q):
            np.testing.assert_array_equal(qa[1:-1, 1:-1], qb[1:-1, 1:-1])
    for kp in Ha.par['Uo']:
        np.testing.assert_array_equal(Ha.par['Uo'][kp], Hb.par['Uo'][kp])
        np.testing.assert_array_equal(Ha.par['Uoo'][kp], Hb.par['Uoo'][kp])


def _same_runs(a, b):
    np.testing.assert_array_equal(a['cycles'], b['cycles'])
    np.testing.assert_array_equal(a['relres'], b['relres'])
    np.testing.assert_array_equal(a['mass'], b['mass'])
    Ha, Hb = a['H'], b['H']
    assert Ha.nlev == Hb.nlev and a['nregrids'] == b['nregrids']
    for k in range(1, Ha.nlev + 1):
        for qa, qb in zip(Ha.lev[k].Q, Hb.lev[k].Q):
            np.testing.assert_array_equal(qa, qb)
    for kp in Ha.par['Uo']:
        np.testing.assert_array_equal(Ha.par['Uo'][kp], Hb.par['Uo'][kp])


def _skip_vs_rebuild(backend, base, ml, monkeypatch):
    import bsam.parabolic as par
    kw = dict(Scheme='bdf2', Dt=0.002, TFinal=0.1, BaseCells=base, MaxLevels=ml, RegridEvery=5, StepVerbose=0)
    hits = []
    keeps = par.regrid_keeps
    monkeypatch.setattr(par, 'regrid_keeps', lambda *x: hits.append(keeps(*x)) or hits[-1])
    a = ebpSolve(heat_problem(), *sum(kw.items(), ()), backend=backend)
    monkeypatch.setattr(par, 'regrid_keeps', lambda *x: False)
    b = ebpSolve(heat_problem(), *sum(kw.items(), ()), backend=backend)
    _same_runs(a, b)
    return hits


def test_regrid_skip_equals_rebuild(monkeypatch):
    """A regrid that would rebuild the same root-only hierarchy is skipped;
    the run equals the one that rebuilds at every regrid, bit for bit (the
    early regrids of this run still change the hierarchy and rebuild)."""
    hits = _skip_vs_rebuild(OracleBackend(), 32, 3, monkeypatch)
    assert any(hits) and not all(hits)


@pytest.mark.gpu
def test_regrid_skip_equals_rebuild_on_device(monkeypatch):
    from bsam.device import DeviceBackend
    hits = _skip_vs_rebuild(DeviceBackend.get(0), 128, 4, monkeypatch)
    assert all(hits)


def rotating_source_problem():
    """P3 of the reference's parabolic suite (ParabolicBSAM/tests/
    runParabolicTests.m: a Gaussian source circling the centre, Dirichlet 0,
    u0 = 0): the refinement follows the source, so every regrid rebuilds a
    three-level hierarchy in a new place."""
    om, Rc, ss = 2 * np.pi, 0.22, 0.03
    cx = lambda t: 0.5 + Rc * np.cos(om * t)
    cy = lambda t: 0.5 + Rc * np.sin(om * t)
    src = lambda x, y, t: 25 * np.exp(-((x - cx(t)) ** 2 + (y - cy(t)) ** 2) / (2 * ss ** 2))
    return ebpProblem([0, 1, 0, 1], 1, 0, src, ('dirichlet', 0), lambda x, y: 0 * x)


ROTATING_SOURCE_OPTS = ('Scheme', 'bdf2', 'Dt', 5e-3, 'TFinal', 0.2, 'RegridEvery', 4, 'StepVerbose', 0,
                        'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'ulap',
                        'TagThreshold', lambda L: 2e-3 / 4 ** (L - 1), 'TagBuffer', 3, 'RelTol', 1e-8)


@pytest.mark.gpu
def test_regrids_keep_history_on_device():
    """The rotating-source run's first 40 steps (nine regrids, each onto a
    moved three-level hierarchy): on the device the BDF2 history goes from
    the old hierarchy to the new one without passing through host memory
    (ebpRegrid.m:62-137 as kernels) -- one download of Uo / Uoo in the whole
    run, for the result.  Per-step V-cycles and residuals, the final field
    and history equal the oracle pipeline's bit for bit."""
    import warnings
    from bsam.device import DeviceBackend
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        a = ebpSolve(rotating_source_problem(), *ROTATING_SOURCE_OPTS, backend=OracleBackend())
        before = DeviceBackend.history_downloads
        b = ebpSolve(rotating_source_problem(), *ROTATING_SOURCE_OPTS, backend=DeviceBackend.get(0))
    assert DeviceBackend.history_downloads - before == 1
    assert a['nregrids'] == b['nregrids'] == 9
    assert len(b['levels']) == 3
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
