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


@pytest.mark.parametrize('tree', [False, True])
def test_uniform_vcycle_matches_direct(tree):
    """unitKernels.m:80-89 (tree copy unitTreeKernels.m): uniform 64^2, RelTol
    1e-11: rel <= 1e-11, err <= 5e-3."""
    from bsam import ebtSolve
    sol = (ebtSolve if tree else ebSolve)(vardc_problem(), 'BaseCells', 64, 'MaxLevels', 1, 'Verbose', 0,
                                          'RelTol', 1e-11, backend=OracleBackend())
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


def _rand_points_1127():
    """rng(1127); X = 4*rand(300,1)-2; Y = 4*rand(300,1)-2 (MATLAB's MT19937,
    reproduced by numpy's legacy generator with the same seeding)."""
    r = np.random.RandomState(1127).random_sample(600)
    return 4 * r[:300] - 2, 4 * r[300:] - 2


def _inpolygon(X, Y, v):
    """Crossing-number point-in-polygon test (points on the boundary count
    as inside, as in MATLAB's inpolygon)."""
    x0, y0, x1, y1 = v[:-1, 0], v[:-1, 1], v[1:, 0], v[1:, 1]
    inside = np.zeros(X.shape, dtype=bool)
    for i in range(X.size):
        cond = (y0 > Y[i]) != (y1 > Y[i])
        xc = x0[cond] + (Y[i] - y0[cond]) * (x1[cond] - x0[cond]) / (y1[cond] - y0[cond])
        inside[i] = np.count_nonzero(X[i] < xc) % 2 == 1
    return inside


def test_starfish_distance_brute_force():
    """testStarfish.m:5-16: the tree-pruned signed distance against a brute
    force over every segment, its sign against point-in-polygon, vertices on
    the curve."""
    from bsam.ddm import ddStarfishGeometry
    g = ddStarfishGeometry()
    X, Y = _rand_points_1127()
    v = g.vertices
    brute = np.full(X.shape, np.inf)
    for k in range(v.shape[0] - 1):
        a = v[k]
        e = v[k + 1] - a
        t = np.maximum(0, np.minimum(1, ((X - a[0]) * e[0] + (Y - a[1]) * e[1]) / np.sum(e ** 2)))
        brute = np.minimum(brute, np.hypot(X - a[0] - t * e[0], Y - a[1] - t * e[1]))
    d = g.signedDistance(X, Y)
    assert np.max(np.abs(np.abs(d) - brute)) < 5e-14
    assert np.all((d >= 0) == _inpolygon(X, Y, v))
    assert g.signedDistance(np.array([0.0]), np.array([0.0]))[0] > 0
    assert g.signedDistance(np.array([2.0]), np.array([2.0]))[0] < 0
    assert np.max(np.abs(g.signedDistance(v[:, 0], v[:, 1]))) < 1e-13


def _constant_solution(backend, device_geometry=None):
    from bsam.ddm import StarGeometry, ddTransmissionProblem
    from bsam import ebSolve
    g = StarGeometry(3000, 0.9, 1.2, 0.7, 5.0, 0.0, device=device_geometry)
    data = {'alpha': 3, 'beta': 2, 'gamma': 1, 'kappa': 0.01, 'q': 2, 'h': 4, 'g': -0.02,
            'exact': lambda x, y: 2 + np.zeros(np.shape(x))}
    p, aux = ddTransmissionProblem(g, 0.05, [-2, 2, -2, 2], data)
    X, Y = _rand_points_1127()
    assert np.max(np.abs(p.f(X, Y) - 2 * p.C(X, Y))) < 1e-13
    return ebSolve(p, 'BaseCells', 32, 'MaxLevels', 3, 'Indicator', 'fun',
                   'TagFunction', lambda x, y: np.abs(g.signedDistance(x, y)) < 0.2, 'RelTol', 1e-11,
                   'Verbose', 0, backend=backend)


def test_transmission_constant_solution():
    """testStarfish.m:17-30: u = 2 with q = gamma u, h = beta u,
    g = -kappa u is exact; the interface source sign makes or breaks it
    (reference: Linf 4.263e-14, residual 3.183e-12)."""
    s = _constant_solution(OracleBackend())
    assert s['err']['linf'] < 1e-9 and s['stats']['stages'][-1]['finalRel'] < 1e-11


@pytest.mark.gpu
def test_transmission_constant_solution_device():
    """The same known answer on the device path, with the geometry's segment
    minimum on the device too."""
    from bsam.device import DeviceBackend
    be = DeviceBackend.get(0)
    s = _constant_solution(be, be.ctx)
    assert s['err']['linf'] < 1e-9 and s['stats']['stages'][-1]['finalRel'] < 1e-11
