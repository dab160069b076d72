"""GPU parity: the CUDA solve path against the C oracle on the same hierarchy.

Both receive the identical flat tables; the device must reproduce the
oracle's residual history and final field bit for bit (FP64 path).
"""
import numpy as np
import pytest

from bsam import ebOptions, hierarchy as hier
from bsam.solve import build_hierarchy, ebSolve, ebtSolve
from bsam.flat import flatten
from bsam_oracle import OracleBackend, OracleHier
from cases import config1_problem, vardc_problem, pureneumann_problem

pytestmark = pytest.mark.gpu


def dev():
    from bsam.device import DeviceBackend
    return DeviceBackend.get(0)


def _both(prob, opts, tree=False):
    """Build one hierarchy (oracle set-up), then solve it on both paths."""
    H = build_hierarchy(prob, opts, OracleBackend(), tree=tree)
    fl = flatten(H)
    oh = OracleHier(fl, opts)
    it_o, hist_o, rel_o, vis_o = oh.solve_cycles(opts.MaxVCycles + 2)
    from bsam.device import DevHier
    dh = DevHier(dev().ctx, fl, opts)
    it_d, hist_d, rel_d, vis_d = dh.solve_cycles(opts.MaxVCycles + 2)
    Qd = dh.get(0, fl.Q.size)
    return (it_o, hist_o, rel_o, vis_o, oh.Q), (it_d, hist_d, rel_d, vis_d, Qd)


def _assert_bitwise(o, d):
    assert o[0] == d[0]
    assert o[3] == d[3]
    np.testing.assert_array_equal(o[1], d[1])
    assert o[2] == d[2]
    np.testing.assert_array_equal(o[4], d[4])


@pytest.mark.parametrize('tree', [False, True])
def test_config1_fixed_hierarchy_bitwise(tree):
    opts = ebOptions('BaseCells', 32, 'MaxLevels', 3, 'TagThreshold', 1e-2, 'Indicator', 'fun',
                     'TagFunction', lambda x, y: (x - 0.4) ** 2 + (y - 0.55) ** 2 < 0.04, 'Verbose', 0,
                     'RelTol', 1e-10)
    o, d = _both(config1_problem(), opts, tree)
    _assert_bitwise(o, d)


@pytest.mark.parametrize('interp', ['qif', 'lif'])
@pytest.mark.parametrize('mass', [True, False])
def test_options_bitwise(interp, mass):
    opts = ebOptions('BaseCells', 32, 'MaxLevels', 3, 'Indicator', 'fun',
                     'TagFunction', lambda x, y: np.abs(x - y) < 0.15, 'Verbose', 0, 'RelTol', 1e-10,
                     'GhostInterp', interp, 'MassCorrection', mass)
    o, d = _both(vardc_problem(), opts)
    _assert_bitwise(o, d)


def test_singular_neumann_bitwise():
    opts = ebOptions('BaseCells', 32, 'MaxLevels', 2, 'Indicator', 'fun',
                     'TagFunction', lambda x, y: (x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.05, 'Verbose', 0,
                     'RelTol', 1e-10)
    o, d = _both(pureneumann_problem(), opts)
    _assert_bitwise(o, d)


def test_config1_solution_driven_matches_oracle_pipeline():
    """Full ebSolve (solve, tag, add level, solve) on the device vs the
    oracle pipeline: same hierarchies, bitwise equal stage histories."""
    p = config1_problem()
    a = ebSolve(p, 'BaseCells', 32, 'MaxLevels', 3, 'TagThreshold', 1e-2, 'Verbose', 0, backend=OracleBackend())
    b = ebSolve(p, 'BaseCells', 32, 'MaxLevels', 3, 'TagThreshold', 1e-2, 'Verbose', 0, backend=dev())
    for sa, sb in zip(a['stats']['stages'], b['stats']['stages']):
        assert sa['vcycles'] == sb['vcycles']
        np.testing.assert_array_equal(sa['resHist'], sb['resHist'])
    for la, lb in zip(a['levels'], b['levels']):
        np.testing.assert_array_equal(la['box'], lb['box'])
    for k in range(1, a['H'].nlev + 1):
        for qa, qb in zip(a['H'].lev[k].Q, b['H'].lev[k].Q):
            np.testing.assert_array_equal(qa, qb)


@pytest.mark.gpu
@pytest.mark.parametrize('indicator', ['ulap', 'rte'])
@pytest.mark.parametrize('tree', [False, True])
def test_device_tag_mask_equals_host(indicator, tree):
    """Tagging on the device (indicator, buffer, cover erosion) gives the
    host restatement's mask bit for bit on a solved hierarchy."""
    from bsam.tagcluster import tag_cluster
    opts = ebOptions('BaseCells', 32, 'MaxLevels', 3, 'Indicator', indicator, 'TagThreshold', 1e-3, 'Verbose', 0,
                     'TagBuffer', 2, 'RelTol', 1e-10)
    be = dev()
    from bsam.solve import ebSolveCycles
    p = vardc_problem()
    H = hier.setup(p, opts, be, tree=tree)
    H = ebSolveCycles(H, be)
    for _ in range(2):
        host = tag_cluster(H)
        devb = tag_cluster(H, be)
        np.testing.assert_array_equal(host, devb)
        assert host.shape[0] > 0
        H = hier.add_level(H, host, be)
        H = ebSolveCycles(H, be)


@pytest.mark.parametrize('tree', [False, True])
def test_non_power_of_two_spacing_bitwise(tree):
    """A [0,3] x [0,1.5] domain: no cell size is a power of two, so every
    kernel divides by h^2 as the reference does (the exact-reciprocal
    products of power-of-two levels do not apply); solved on both paths."""
    from bsam import ebProblem
    D = lambda x, y: 1 + 0.2 * x * y
    f = lambda x, y: np.sin(2 * x) * np.cos(3 * y) + 0.5
    prob = ebProblem([0, 3, 0, 1.5], D, 1, f, ('dirichlet', 0))
    opts = ebOptions('BaseCells', 32, 'MaxLevels', 3, 'Indicator', 'fun',
                     'TagFunction', lambda x, y: np.abs(x - 2 * y) < 0.3, 'Verbose', 0, 'RelTol', 1e-10)
    H = build_hierarchy(prob, opts, OracleBackend(), tree=tree)
    fl = flatten(H)
    for hx, hy in np.asarray(fl.hs).reshape(-1, 2):
        assert np.frexp(hx * hx)[0] != 0.5 or np.frexp(hy * hy)[0] != 0.5
    o, d = _both(prob, opts, tree)
    _assert_bitwise(o, d)
