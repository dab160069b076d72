"""Known-answer tests of the solve path on the C oracle, after the
reference's unit tests (EllipticBSAM/tests/unitKernels.m:12-89)."""
import numpy as np
import pytest

from bsam import ebOptions, ebProblem, ebSolve, hierarchy as hier
from bsam.flat import flatten, scatter_field, FIELD_Q, FIELD_QC
from bsam_oracle import OracleBackend, OracleHier
from cases import vardc_problem


def _two_level(box, interp='qif', base=16):
    prob = ebProblem([0, 1, 0, 1], 1, 1, 0, ('dirichlet', 0))
    opts = ebOptions('BaseCells', base, 'MaxLevels', 2, 'GhostInterp', interp, 'Verbose', 0)
    H = hier.setup(prob, opts, OracleBackend())
    H = hier.add_level(H, np.array([box]), OracleBackend())
    return H


def _centres(lev, p, pad):
    b = lev.box[p]
    i = np.arange(b[0] - pad, b[1] + pad + 1)
    j = np.arange(b[2] - pad, b[3] + pad + 1)
    xc = (i - 0.5) * lev.h[0]
    yc = (j - 0.5) * lev.h[1]
    return np.meshgrid(xc, yc, indexing='ij')


@pytest.mark.parametrize('interp,u', [
    ('qif', lambda x, y: 1.5 + 0.3 * x - 0.7 * y + 0.25 * x ** 2 - 0.4 * x * y + 0.6 * y ** 2),
    ('lif', lambda x, y: 1.5 + 0.3 * x - 0.7 * y)])
def test_ghost_interp_reproduces_polynomials(interp, u):
    """unitKernels.m:15-35: QIF reproduces quadratics, LIF linears, on every
    coarse-fine ghost cell including CF corners (poisoned ghosts = 99)."""
    H = _two_level([5, 10, 4, 11], interp)
    X, Y = _centres(H.lev[1], 0, 1)
    H.lev[1].Q[0][...] = u(X, Y)
    Xf, Yf = _centres(H.lev[2], 0, 1)
    exact = u(Xf, Yf)
    Q = exact.copy()
    Q[0, :] = Q[-1, :] = Q[:, 0] = Q[:, -1] = 99
    H.lev[2].Q[0][...] = Q
    fl = flatten(H)
    oh = OracleHier(fl, H.opts)
    oh.op('fill_ghosts', 2)
    scatter_field(H, fl, FIELD_Q, oh.Q)
    got = H.lev[2].Q[0]
    mask = np.zeros(got.shape, bool)
    mask[[0, -1], :] = True
    mask[:, [0, -1]] = True
    assert np.max(np.abs(got[mask] - exact[mask])) <= 1e-12


def test_restrict_prolong_affine():
    """unitKernels.m:68-78: restrict(prolong(W)) == W for affine W."""
    H = _two_level([3, 8, 5, 12])
    aff = lambda x, y: 0.3 + 0.2 * x - 0.45 * y
    X, Y = _centres(H.lev[1], 0, 1)
    H.lev[1].Q[0][...] = aff(X, Y)
    fl = flatten(H)
    oh = OracleHier(fl, H.opts)
    oh.op('correct', 2, 0)       # Q_2 interior = prolong(W)
    oh.op('restrict', 2)         # QC interior = restrict2(Q_2)
    scatter_field(H, fl, FIELD_QC, oh.QC)
    lev = H.lev[2]
    b = lev.box[0]
    Il, Ih, Jl, Jh = (b[0] + 1) // 2, b[1] // 2, (b[2] + 1) // 2, b[3] // 2
    Xc, Yc = np.meshgrid((np.arange(Il, Ih + 1) - 0.5) * H.lev[1].h[0],
                         (np.arange(Jl, Jh + 1) - 0.5) * H.lev[1].h[1], indexing='ij')
    assert np.max(np.abs(lev.QC[0][1:-1, 1:-1] - aff(Xc, Yc))) <= 1e-13


def test_uniform_vcycle_matches_direct():
    """unitKernels.m:80-89: uniform 64^2, RelTol 1e-11: rel <= 1e-11, err <= 5e-3."""
    sol = ebSolve(vardc_problem(), 'BaseCells', 64, 'MaxLevels', 1, 'Verbose', 0, 'RelTol', 1e-11,
                  backend=OracleBackend())
    st = sol['stats']['stages'][0]
    assert st['finalRel'] <= 1e-11
    assert sol['err']['linf'] <= 5e-3


def test_operator_second_order():
    """unitKernels.m:37-66: truncation error of op2d decays at rate >= 1.8."""
    uex = lambda x, y: np.sin(np.pi * x) * np.cos(np.pi * y)
    D = lambda x, y: 1 + 0.5 * np.sin(2 * np.pi * x) * np.cos(np.pi * y)
    C = lambda x, y: 1 + x * y
    from cases import vardc_problem as vp
    f = vp().f
    errs = []
    for n in (32, 64, 128):
        h = 1.0 / n
        XF, YC = np.meshgrid(np.arange(0, n + 1) * h, (np.arange(1, n + 1) - 0.5) * h, indexing='ij')
        XC, YF = np.meshgrid((np.arange(1, n + 1) - 0.5) * h, np.arange(0, n + 1) * h, indexing='ij')
        X, Y = np.meshgrid((np.arange(0, n + 2) - 0.5) * h, (np.arange(0, n + 2) - 0.5) * h, indexing='ij')
        Lu = hier.op2d(uex(X, Y), D(XF, YC), D(XC, YF), C(X[1:-1, 1:-1], Y[1:-1, 1:-1]), h, h)
        errs.append(np.max(np.abs(Lu - f(X[1:-1, 1:-1], Y[1:-1, 1:-1]))))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates >= 1.8)
