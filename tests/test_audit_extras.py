"""Property checks of EllipticBSAM/tests/auditExtras.m (A1-A8) and
testNeumannCompat.m, on the oracle.  The reference records no numbers for
these scripts; each check is its pass criterion restated:

A1 Berger-Rigoutsos boxes are free rectangles (skinny bands, parent-cell
   aligned) and the solve on them converges.
A2 a QC-ring fine patch straddling two parent patches (multi-parent) solves
   without degradation.
A3 anisotropic cells on a rectangular domain keep second order.
A4 mixed Dirichlet/Neumann sides keep second order.
A5 'rte' tagging reduces the error.
A6 Omega and InitialGuess variants converge.
A7 six adaptive levels keep the V-cycle factor and reduce the error.
A8 ebSample agrees with the exact solution to the grid's accuracy.
Neumann compatibility: 3-level singular pure-Neumann, SourceQuad 1, ring
   and tree: the compatibility projection keeps factor <= 0.15, the final
   residual <= 1e-9 and second order.
"""
import warnings

import numpy as np
import pytest

from bsam import ebProblem, ebSolve, ebtSolve, ebSample, ebtSample
from bsam_oracle import OracleBackend
from cases import threebumps_problem, gauss52_problem, vardc_problem


def _rates(errs):
    errs = np.asarray(errs)
    return np.log2(errs[:-1] / errs[1:])


def test_A1_free_rectangles():
    uex = lambda X, Y: np.sin(np.pi * X) * np.cos(np.pi * Y)
    prob = ebProblem([0, 1, 0, 1], 1, 1, lambda X, Y: (2 * np.pi ** 2 + 1) * uex(X, Y), ('dirichlet', uex), uex)
    band = lambda X, Y, L: (((np.abs(Y - 0.70) < 0.035) & (X > 0.06) & (X < 0.94)) | (np.abs(Y - X) < 0.05))
    sol = ebSolve(prob, 'BaseCells', [64, 64], 'MaxLevels', 2, 'Indicator', 'fun', 'TagFunction', band,
                  'TagBuffer', 0, 'Verbose', 0, 'RelTol', 1e-9, backend=OracleBackend())
    bx = sol['levels'][1]['box']
    w, h = bx[:, 1] - bx[:, 0] + 1, bx[:, 3] - bx[:, 2] + 1
    assert np.all(bx[:, 0] % 2 == 1) and np.all(bx[:, 1] % 2 == 0)
    assert np.all(bx[:, 2] % 2 == 1) and np.all(bx[:, 3] % 2 == 0)
    assert np.max(np.maximum(w / h, h / w)) >= 4
    assert sol['stats']['stages'][-1]['finalRel'] <= 1e-8


def test_A2_ring_patch_straddling_two_parents():
    two = lambda X, Y: (((X >= 0.25) & (X < 0.5) & (Y >= 0.25) & (Y < 0.75))
                        | ((X >= 0.5) & (X < 0.75) & (Y >= 0.40) & (Y < 0.60)))
    strad = lambda X, Y: (np.abs(X - 0.5) < 0.04) & (np.abs(Y - 0.5) < 0.03)
    sol = ebSolve(gauss52_problem(), 'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'fun',
                  'TagFunction', lambda X, Y, L: (L == 1) * two(X, Y) + (L == 2) * strad(X, Y), 'TagBuffer', 0,
                  'MinFillRatio', 0.95, 'Verbose', 0, 'RelTol', 1e-11, 'MaxVCycles', 40, backend=OracleBackend())
    H = sol['H']
    assert max(len(P) for P in H.lev[H.nlev].parents) >= 2
    st = sol['stats']['stages'][-1]
    assert st['finalRel'] <= 5e-10 and sol['mass']['rel'] <= 1e-11 and st['avgFactor'] <= 0.2


def test_A3_anisotropic_cells_rectangular_domain():
    uex = lambda X, Y: np.sin(np.pi * X) * np.cos(np.pi * Y)
    D = lambda X, Y: 1 + 0.5 * X
    f = lambda X, Y: (-0.5 * np.pi * np.cos(np.pi * X) * np.cos(np.pi * Y)
                      + 2 * np.pi ** 2 * (1 + 0.5 * X) * np.sin(np.pi * X) * np.cos(np.pi * Y) + uex(X, Y))
    prob = ebProblem([0, 2, 0, 1], D, lambda X, Y: 1 + 0 * X, f, ('dirichlet', uex), uex)
    centre = lambda X, Y, L: (X - 1) ** 2 + (Y - 0.5) ** 2 < 0.2 ** 2
    errs = []
    for base in ([64, 16], [128, 32], [256, 64]):
        sol = ebSolve(prob, 'BaseCells', base, 'MaxLevels', 2, 'Indicator', 'fun', 'TagFunction', centre,
                      'Verbose', 0, 'RelTol', 1e-10, backend=OracleBackend())
        errs.append(sol['err']['linf'])
    assert np.all(_rates(errs) >= 1.8), errs


def mixed_bc_problem():
    """A4 (auditExtras.m): D = 1 + xy/2, C = 1 + x + y; Dirichlet west and
    south, Neumann east and north."""
    uex = lambda X, Y: np.exp(X) * np.sin(np.pi * Y) + 0.5 * X ** 2
    D = lambda X, Y: 1 + 0.5 * X * Y
    C = lambda X, Y: 1 + X + Y
    f = lambda X, Y: (-(0.5 * Y * (np.exp(X) * np.sin(np.pi * Y) + X)
                        + (1 + 0.5 * X * Y) * (np.exp(X) * np.sin(np.pi * Y) + 1)
                        + 0.5 * X * (np.pi * np.exp(X) * np.cos(np.pi * Y))
                        + (1 + 0.5 * X * Y) * (-np.pi ** 2 * np.exp(X) * np.sin(np.pi * Y)))
                      + C(X, Y) * uex(X, Y))
    bc = {'west': ('dirichlet', uex), 'east': ('neumann', lambda X, Y: np.exp(X) * np.sin(np.pi * Y) + X),
          'south': ('dirichlet', uex), 'north': ('neumann', lambda X, Y: np.pi * np.exp(X) * np.cos(np.pi * Y))}
    return ebProblem([0, 1, 0, 1], D, C, f, bc, uex)


def corner_tag(X, Y, L):
    return (X - 0.75) ** 2 + (Y - 0.75) ** 2 < 0.15 ** 2


def test_A4_mixed_dirichlet_neumann_sides():
    errs = []
    for m in (32, 64, 128, 256):
        sol = ebSolve(mixed_bc_problem(), 'BaseCells', [m, m], 'MaxLevels', 2, 'Indicator', 'fun',
                      'TagFunction', corner_tag, 'Verbose', 0, 'RelTol', 1e-10, backend=OracleBackend())
        errs.append(sol['err']['linf'])
    assert np.all(_rates(errs) >= 1.8), errs


def test_A5_rte_indicator_reduces_error():
    errs = []
    for nlv in (1, 2, 3):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            sol = ebSolve(threebumps_problem(), 'BaseCells', [64, 64], 'MaxLevels', nlv, 'Indicator', 'rte',
                          'TagThreshold', lambda L: 2e-3 / 4 ** (L - 1), 'TagBuffer', 2, 'Verbose', 0,
                          'RelTol', 1e-9, 'MaxVCycles', 40, backend=OracleBackend())
        errs.append(sol['err']['linf'])
    assert errs[2] <= 0.35 * errs[0], errs


@pytest.mark.parametrize('omega', [0.85, 1.0, 1.15])
def test_A6_omega_and_initial_guess(omega):
    sol = ebSolve(vardc_problem(), 'BaseCells', [64, 64], 'Omega', omega, 'Verbose', 0, 'RelTol', 1e-10,
                  'InitialGuess', lambda X, Y: np.cos(3 * X) * Y, backend=OracleBackend())
    assert sol['stats']['stages'][-1]['finalRel'] <= 1e-9


def test_A7_six_adaptive_levels():
    errs = []
    for nlv in (4, 5, 6):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            sol = ebSolve(threebumps_problem(), 'BaseCells', [32, 32], 'MaxLevels', nlv, 'Indicator', 'ulap',
                          'TagThreshold', lambda L: 4e-2 / 4 ** (L - 1), 'TagBuffer', 2, 'Verbose', 0,
                          'RelTol', 1e-9, 'MaxVCycles', 60, backend=OracleBackend())
        assert sol['stats']['stages'][-1]['avgFactor'] <= 0.2
        errs.append(sol['err']['linf'])
    assert len(sol['levels']) == 6
    assert errs[-1] <= 0.15 * errs[0], errs


@pytest.mark.parametrize('tree', [False, True])
def test_A8_sample_accuracy(tree):
    prob = vardc_problem()
    solve, sample = (ebtSolve, ebtSample) if tree else (ebSolve, ebSample)
    sol = solve(prob, 'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'ulap',
                'TagThreshold', lambda L: 1e-2 / 4 ** (L - 1), 'Verbose', 0, 'RelTol', 1e-10, backend=OracleBackend())
    rs = np.random.RandomState(7)                # MATLAB rng(7) + rand: MT19937, 53-bit doubles
    xq = np.concatenate([rs.random_sample(2000), [0, 1, 0, 1, 0.5, 0.5, 0, 1]])
    yq = np.concatenate([rs.random_sample(2000), [0, 0, 1, 1, 0, 1, 0.5, 0.5]])
    v = sample(sol['H'], xq, yq)
    assert np.max(np.abs(v - prob.exact(xq, yq))) <= 50 * sol['err']['linf']
    # a point exactly at a cell centre returns that cell's value
    H = sol['H']
    lev = H.lev[H.rootIdx]
    h = lev.h
    xc, yc = (np.array([10]) - 0.5) * h[0], (np.array([20]) - 0.5) * h[1]
    if not H.lev[H.rootIdx].covered[0][9, 19]:
        assert sample(H, xc, yc)[0] == lev.Q[0][10, 20]
    with pytest.raises(ValueError, match='_sample:cover'):
        sample(H, np.array([1.5]), np.array([0.5]))


@pytest.mark.parametrize('tree', [False, True])
def test_neumann_compatibility_three_levels(tree):
    uex = lambda X, Y: np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    prob = ebProblem([0, 1, 0, 1], 1, 0, lambda X, Y: 8 * np.pi ** 2 * uex(X, Y), ('neumann', 0), uex)
    tag = lambda X, Y, L: ((L == 1) * (np.maximum(np.abs(X - 0.5), np.abs(Y - 0.5)) < 0.30)
                           + (L == 2) * (np.maximum(np.abs(X - 0.5), np.abs(Y - 0.5)) < 0.15))
    solve = ebtSolve if tree else ebSolve
    errs = []
    for m in (32, 64, 128):
        sol = solve(prob, 'BaseCells', [m, m], 'MaxLevels', 3, 'Indicator', 'fun', 'TagFunction', tag,
                    'TagBuffer', 0, 'Verbose', 0, 'RelTol', 1e-10, 'MaxVCycles', 40, 'SourceQuad', 1,
                    backend=OracleBackend())
        st = sol['stats']['stages'][-1]
        assert st['avgFactor'] <= 0.15 and st['finalRel'] <= 1e-9, st
        errs.append(sol['err']['linf'])
    assert np.all(_rates(errs) >= 1.8), errs


def _audit_case(name, backend):
    if name == 'A2':
        two = lambda X, Y: (((X >= 0.25) & (X < 0.5) & (Y >= 0.25) & (Y < 0.75))
                            | ((X >= 0.5) & (X < 0.75) & (Y >= 0.40) & (Y < 0.60)))
        strad = lambda X, Y: (np.abs(X - 0.5) < 0.04) & (np.abs(Y - 0.5) < 0.03)
        return ebSolve(gauss52_problem(), 'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'fun',
                       'TagFunction', lambda X, Y, L: (L == 1) * two(X, Y) + (L == 2) * strad(X, Y),
                       'TagBuffer', 0, 'MinFillRatio', 0.95, 'Verbose', 0, 'RelTol', 1e-11, 'MaxVCycles', 40,
                       backend=backend)
    if name == 'A3':
        uex = lambda X, Y: np.sin(np.pi * X) * np.cos(np.pi * Y)
        f = lambda X, Y: (-0.5 * np.pi * np.cos(np.pi * X) * np.cos(np.pi * Y)
                          + 2 * np.pi ** 2 * (1 + 0.5 * X) * np.sin(np.pi * X) * np.cos(np.pi * Y) + uex(X, Y))
        prob = ebProblem([0, 2, 0, 1], lambda X, Y: 1 + 0.5 * X, 1, f, ('dirichlet', uex), uex)
        return ebSolve(prob, 'BaseCells', [128, 32], 'MaxLevels', 2, 'Indicator', 'fun',
                       'TagFunction', lambda X, Y, L: (X - 1) ** 2 + (Y - 0.5) ** 2 < 0.2 ** 2, 'Verbose', 0,
                       'RelTol', 1e-10, backend=backend)
    if name == 'A4':
        return ebSolve(mixed_bc_problem(), 'BaseCells', [128, 128], 'MaxLevels', 2, 'Indicator', 'fun',
                       'TagFunction', corner_tag, 'Verbose', 0, 'RelTol', 1e-10, backend=backend)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return ebSolve(threebumps_problem(), 'BaseCells', [32, 32], 'MaxLevels', 6, 'Indicator', 'ulap',
                       'TagThreshold', lambda L: 4e-2 / 4 ** (L - 1), 'TagBuffer', 2, 'Verbose', 0,
                       'RelTol', 1e-9, 'MaxVCycles', 60, backend=backend)


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['A2', 'A3', 'A4', 'A7'])
def test_audit_hierarchies_device_bitwise(name):
    """Multi-parent ring patches, anisotropic cells on a rectangle, mixed
    Dirichlet/Neumann sides and six adaptive levels: the CUDA path's
    residual histories and composite field equal the oracle's bit for bit."""
    from bsam.device import DeviceBackend
    o = _audit_case(name, OracleBackend())
    d = _audit_case(name, DeviceBackend.get(0))
    assert len(o['stats']['stages']) == len(d['stats']['stages'])
    for so, sd in zip(o['stats']['stages'], d['stats']['stages']):
        np.testing.assert_array_equal(so['resHist'], sd['resHist'])
    Ho, Hd = o['H'], d['H']
    assert Ho.nlev == Hd.nlev
    for k in range(Ho.rootIdx, Ho.nlev + 1):
        for qa, qb in zip(Ho.lev[k].Q, Hd.lev[k].Q):
            np.testing.assert_array_equal(qa, qb)
    assert o['err'] == d['err']
