"""Adversarial interface geometries (EllipticBSAM/tests/stressInterfaces.m
S1-S9, EllipticBSAMTree/tests/stressTreeInterfaces.m S1-S10).

CPU (oracle): each case's pass criterion restated -- Linf rates above 1.75
over m = 32, 64, 128, V-cycle factor <= 0.2, relative mass defect <= 5e-10
-- for comb interfaces, corner-only adjacency, reentrant tag shapes, hanging
nodes on Dirichlet / Neumann / mixed sides, minimum-width patches,
hand-built checkerboards / spirals / corridors / edge kisses / surrounded
patches, a 5-level cross point, the conservation discriminators (the defect
scales with RelTol; corrections off break it) and singular Neumann with
SourceQuad 3; the tree form of every layout passes ebtTreeCheck and agrees
with the ring form on identical meshes (S10).  GPU: every layout, ring and
tree, solved on the CUDA path equals the oracle bit for bit (residual
history and composite field).
"""
import warnings

import numpy as np
import pytest

from bsam import ebOptions, ebProblem, ebSolve, ebtSolve, hierarchy as hier
from bsam.solve import ebSolveCycles, error_norms
from bsam.treecheck import ebtTreeCheck
from bsam_oracle import OracleBackend
from cases import vardc_problem

MS = (32, 64, 128)
RATE_BAR, FAC_BAR, MASS_BAR = 1.75, 0.2, 5e-10


# ------------------------------------------------------------------ problems
def _pm():
    uex = lambda x, y: np.exp(x) * np.sin(np.pi * y) + 0.5 * x ** 2
    D = lambda x, y: 1 + 0.5 * x * y
    C = lambda x, y: 1 + x + y
    f = lambda x, y: (-(0.5 * y * (np.exp(x) * np.sin(np.pi * y) + x)
                        + (1 + 0.5 * x * y) * (np.exp(x) * np.sin(np.pi * y) + 1)
                        + 0.5 * x * (np.pi * np.exp(x) * np.cos(np.pi * y))
                        + (1 + 0.5 * x * y) * (-np.pi ** 2 * np.exp(x) * np.sin(np.pi * y)))
                      + C(x, y) * uex(x, y))
    g = {'W': lambda x, y: -(np.exp(x) * np.sin(np.pi * y) + x), 'E': lambda x, y: np.exp(x) * np.sin(np.pi * y) + x,
         'S': lambda x, y: -(np.pi * np.exp(x) * np.cos(np.pi * y)), 'N': lambda x, y: np.pi * np.exp(x) * np.cos(np.pi * y)}
    return uex, D, C, f, g


def problem(name):
    """The suite's problems (stressInterfaces.m:52-102)."""
    if name == 'V':
        return vardc_problem()
    if name in ('MD', 'MN', 'MX'):
        uex, D, C, f, g = _pm()
        if name == 'MD':
            bc = ('dirichlet', uex)
        elif name == 'MN':
            bc = {'west': ('neumann', g['W']), 'south': ('neumann', g['S']), 'east': ('dirichlet', uex),
                  'north': ('dirichlet', uex)}
        else:
            bc = {'west': ('dirichlet', uex), 'south': ('neumann', g['S']), 'east': ('neumann', g['E']),
                  'north': ('dirichlet', uex)}
        return ebProblem([0, 1, 0, 1], D, C, f, bc, uex)
    if name == 'A':
        uex = lambda x, y: np.sin(np.pi * x) * np.cos(np.pi * y)
        f = lambda x, y: (-0.5 * np.pi * np.cos(np.pi * x) * np.cos(np.pi * y)
                          + 2 * np.pi ** 2 * (1 + 0.5 * x) * np.sin(np.pi * x) * np.cos(np.pi * y) + uex(x, y))
        return ebProblem([0, 2, 0, 1], lambda x, y: 1 + 0.5 * x, 1, f, ('dirichlet', uex), uex)
    if name == 'N':
        D = lambda x, y: 1 + 0.5 * np.sin(2 * np.pi * x) * np.cos(np.pi * y)
        Dx = lambda x, y: np.pi * np.cos(2 * np.pi * x) * np.cos(np.pi * y)
        Dy = lambda x, y: -0.5 * np.pi * np.sin(2 * np.pi * x) * np.sin(np.pi * y)
        uex = lambda x, y: np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
        ux = lambda x, y: -2 * np.pi * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
        uy = lambda x, y: -2 * np.pi * np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y)
        f = lambda x, y: -(Dx(x, y) * ux(x, y) + Dy(x, y) * uy(x, y) + D(x, y) * (-8 * np.pi ** 2 * uex(x, y)))
        return ebProblem([0, 1, 0, 1], D, 0, f, ('neumann', 0), uex)
    raise KeyError(name)


# ------------------------------------------------------------ tag functions
def comb(X, Y):
    return (((X > 4 / 32) & (X < 16 / 32) & (Y > 4 / 32) & (Y < 28 / 32))
            | ((X > 16 / 32) & (X < 20 / 32) & (((Y > 4 / 32) & (Y < 7 / 32)) | ((Y > 10 / 32) & (Y < 13 / 32))
                                                | ((Y > 16 / 32) & (Y < 19 / 32)) | ((Y > 22 / 32) & (Y < 25 / 32)))))


def comb_bdy(X, Y):
    return (X < 4 / 32) & (32 * Y > 2) & (32 * Y < 28) & (np.mod(np.floor((32 * Y - 2) / 2), 2) == 0)


def comb_aniso(X, Y):
    return (((X > 0.5) & (X < 1.0) & (Y > 1 / 8) & (Y < 7 / 8))
            | ((X >= 1.0) & (X < 1.25) & (((Y > 1 / 8) & (Y < 2 / 8)) | ((Y > 3 / 8) & (Y < 4 / 8))
                                          | ((Y > 5 / 8) & (Y < 6 / 8)))))


def _u16(X, Y, x1, x2, y1, y2):
    return (X >= x1 / 16) & (X <= x2 / 16) & (Y >= y1 / 16) & (Y <= y2 / 16)


def zigzag(X, Y):
    d = np.floor(8 * X - 8 * Y)
    return (d >= -1) & (d <= 0) & (X > 2 / 16) & (X < 14 / 16) & (Y > 2 / 16) & (Y < 14 / 16)


def annulus(X, Y):
    r = np.maximum(np.abs(X - 0.5), np.abs(Y - 0.5))
    return (r >= 3 / 16) & (r <= 6 / 16)


# (name, tag, MinFillRatio, GhostInterp, minimum patch count)
TAG_CASES = {
    'COMB-qif': (lambda X, Y, L: comb(X, Y), 0.95, 'qif', 4),
    'COMB-lif': (lambda X, Y, L: comb(X, Y), 0.95, 'lif', 4),
    'COMBB': (lambda X, Y, L: comb_bdy(X, Y), 0.85, 'qif', 5),
    'USHAPE': (lambda X, Y, L: _u16(X, Y, 4, 12, 4, 6) | _u16(X, Y, 4, 6, 6, 12) | _u16(X, Y, 10, 12, 6, 12), 0.95,
               'qif', 2),
    'TSHAPE': (lambda X, Y, L: _u16(X, Y, 4, 12, 8, 10) | _u16(X, Y, 7, 9, 2, 8), 0.95, 'qif', 2),
    'PLUS': (lambda X, Y, L: _u16(X, Y, 3, 13, 7, 9) | _u16(X, Y, 7, 9, 3, 13), 0.95, 'qif', 2),
    'ZIGZAG': (lambda X, Y, L: zigzag(X, Y), 0.85, 'qif', 2),
    'ANNULUS': (lambda X, Y, L: annulus(X, Y), 0.85, 'qif', 2),
}
TAG_PROBLEM = {'COMBB-NN': 'MN'}


# ------------------------------------------------------- hand-built layouts
def _chain():
    return np.array([[7 + 2 * i, 8 + 2 * i, 7 + 2 * i, 8 + 2 * i] for i in range(1, 8)])


def _checker(n, off):
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
    keep = (ii + jj) % 2 == 0
    i, j = ii.T[keep.T], jj.T[keep.T]          # column-major order, as ndgrid(:) lists them
    return np.stack([4 * i + off, 4 * i + off + 3, 4 * j + off, 4 * j + off + 3], axis=1)


def _deepcross():
    out = []
    for lv in range(2, 6):
        n = 32 * 2 ** (lv - 2)
        c0 = n // 2
        out.append(np.array([[c0 - 7, c0, c0 - 7, c0], [c0 + 1, c0 + 8, c0 - 7, c0],
                             [c0 - 7, c0, c0 + 1, c0 + 8], [c0 + 1, c0 + 8, c0 + 1, c0 + 8]]))
    return out


SPIRAL = [[1, 32, 1, 4], [29, 32, 5, 32], [1, 28, 29, 32], [1, 4, 5, 28], [5, 28, 5, 8], [25, 28, 9, 28],
          [5, 24, 25, 28], [5, 8, 9, 24], [9, 24, 9, 12], [21, 24, 13, 24], [9, 20, 21, 24], [9, 12, 13, 20],
          [13, 20, 13, 16]]
CORRIDORS = [[5, 26, 5, 6], [27, 28, 5, 26], [7, 28, 27, 28], [5, 6, 7, 28], [9, 22, 9, 10], [23, 24, 9, 22],
             [11, 24, 23, 24], [9, 10, 11, 22]]
SURROUND = [[9, 12, 9, 12], [13, 20, 9, 12], [21, 24, 9, 12], [9, 12, 13, 20], [13, 20, 13, 20], [21, 24, 13, 20],
            [9, 12, 21, 24], [13, 20, 21, 24], [21, 24, 21, 24]]

# name -> (problem, [per-level boxes in the base-32 index space of the then-finest level])
BOX_CASES = {
    'CORNER2': ('V', [[[9, 16, 9, 16], [17, 24, 17, 24]]]),
    'CORNER2AD': ('V', [[[17, 24, 9, 16], [9, 16, 17, 24]]]),
    'CORNERA': ('V', [[[5, 16, 5, 16], [17, 28, 17, 24]]]),
    'CORNER4': ('V', [[[9, 16, 9, 16], [17, 24, 9, 16], [9, 16, 17, 24], [17, 24, 17, 24]]]),
    'HANGQ-D': ('MD', [[[1, 16, 1, 16]]]),
    'HANGQ-NN': ('MN', [[[1, 16, 1, 16]]]),
    'HANGQ-MX': ('MX', [[[1, 16, 1, 16]]]),
    'NOTCH-MX': ('MX', [[[9, 24, 1, 8]]]),
    'STRIP-MX': ('MX', [[[1, 16, 1, 32]]]),
    'HANGQ3-MX': ('MX', [[[1, 16, 1, 16]], [[1, 16, 1, 16]]]),
    'SANDWICH': ('V', [[[5, 28, 15, 16], [5, 28, 17, 26], [5, 28, 27, 28]]]),
    'DOMINOES': ('V', [[[9, 10, 9, 24], [11, 12, 9, 24], [13, 14, 9, 24], [15, 16, 9, 24]]]),
    'CHAIN': ('V', [_chain()]),
    'RINGTOUCH': ('V', [[[1, 4, 13, 16], [1, 4, 9, 12], [1, 4, 17, 20], [5, 8, 13, 16]]]),
    'SKINNY3': ('V', [[[9, 24, 9, 24]], [[25, 26, 19, 42]]]),
    'CHECKER': ('V', [_checker(8, 1)]),
    'CHECKER3': ('V', [[[5, 28, 5, 28]], _checker(10, 13)]),
    'SPIRAL': ('V', [SPIRAL]),
    'CORRIDORS': ('V', [CORRIDORS]),
    'EDGEKISS': ('V', [[[5, 16, 5, 28], [17, 28, 5, 28]], [[25, 32, 17, 40]]]),
    'EDGEKISS2': ('V', [[[5, 16, 5, 28], [17, 28, 5, 28]], [[25, 32, 17, 40], [33, 40, 29, 52]]]),
    'SURROUND': ('V', [SURROUND]),
    'DEEPCROSS5': ('V', _deepcross()),
}


def scale_boxes(b, s):
    b = np.asarray(b, dtype=np.int64)
    return np.stack([(b[:, 0] - 1) * s + 1, b[:, 1] * s, (b[:, 2] - 1) * s + 1, b[:, 3] * s], axis=1)


def build_boxes(prob, m, levels, rtol, maxv, backend, tree=False, **opts):
    """ebSetup + ebAddLevel per box list + ebSolveCycles (stressInterfaces.m
    buildBoxes); the tree form resolves each box's single parent by
    containment and checks every tree invariant before the solve
    (stressTreeInterfaces.m buildBoxesT)."""
    o = ebOptions('BaseCells', [m, m], 'Verbose', 0, 'RelTol', rtol, 'MaxVCycles', maxv, **opts)
    H = hier.setup(prob, o, backend, tree=tree)
    for bx in levels:
        bx = np.asarray(bx, dtype=np.int64)
        for a in range(len(bx)):
            for b in range(a + 1, len(bx)):
                assert not (bx[a, 0] <= bx[b, 1] and bx[a, 1] >= bx[b, 0] and bx[a, 2] <= bx[b, 3]
                            and bx[a, 3] >= bx[b, 2]), 'stress:overlap'
        if tree:
            levC = H.lev[H.nlev]
            par = [next(q + 1 for q, qb in enumerate(levC.box)
                        if qb[0] <= b[0] and b[1] <= qb[1] and qb[2] <= b[2] and b[3] <= qb[3]) for b in bx]
            bx = np.column_stack([par, bx])
        H = hier.add_level(H, bx, backend)
    if tree:
        ebtTreeCheck(H)
    return ebSolveCycles(H, backend)


def box_case(name, m, backend, rtol=1e-10, maxv=60, tree=False):
    pname, levels = BOX_CASES[name]
    s = m // 32
    return build_boxes(problem(pname), m, [scale_boxes(b, s) for b in levels], rtol, maxv, backend, tree=tree)


def tag_case(name, m, backend, prob=None, rtol=1e-10, maxv=60, tree=False, **extra):
    tag, fill, ghost, _ = TAG_CASES[name]
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return (ebtSolve if tree else ebSolve)(prob or problem('V'), 'BaseCells', [m, m], 'MaxLevels', 2, 'Indicator', 'fun',
                       'TagFunction', tag, 'TagBuffer', 0, 'MinBoxWidth', 2, 'MinFillRatio', fill,
                       'GhostInterp', ghost, 'Verbose', 0, 'RelTol', rtol, 'MaxVCycles', maxv, backend=backend,
                       **extra)


def _check_sweep(errs, facs, mass):
    r = np.log2(np.asarray(errs[:-1]) / np.asarray(errs[1:]))
    assert np.all(r > RATE_BAR), (errs, r)
    assert max(facs) <= FAC_BAR, facs
    assert max(abs(v) for v in mass) <= MASS_BAR, mass


# ------------------------------------------------------------------ CPU tests
@pytest.mark.parametrize('tree', [False, True])
@pytest.mark.parametrize('name', list(TAG_CASES) + ['COMBB-NN'])
def test_tag_driven_interfaces(name, tree):
    """S1 comb interfaces (QIF, LIF, boundary comb, Neumann-side comb) and
    S3 reentrant shapes, ring and tree; ANNULUS keeps its coarse hole at
    every size; every tree hierarchy passes ebtTreeCheck."""
    be = OracleBackend()
    base = 'COMBB' if name == 'COMBB-NN' else name
    prob = problem(TAG_PROBLEM.get(name, 'V'))
    errs, facs, mass = [], [], []
    for m in MS:
        sol = tag_case(base, m, be, prob=prob, tree=tree)
        if tree:
            ebtTreeCheck(sol['H'])
        errs.append(sol['err']['linf'])
        facs.append(sol['stats']['stages'][-1]['avgFactor'])
        mass.append(sol['mass']['rel'])
        assert sol['levels'][1]['np'] >= TAG_CASES[base][3]
        if base == 'ANNULUS':
            lev = sol['H'].lev[sol['H'].nlev]
            c = [v // 2 for v in lev.n]
            assert not any(b[0] <= c[0] <= b[1] and b[2] <= c[1] <= b[3] for b in lev.box)
    _check_sweep(errs, facs, mass)


def test_comb_anisotropic_cells():
    """S1 COMB-ANISO: 2:1 cells; the factor bar is 0.25 there."""
    be = OracleBackend()
    errs, facs, mass = [], [], []
    for base in ([64, 16], [128, 32], [256, 64]):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            sol = ebSolve(problem('A'), 'BaseCells', base, 'MaxLevels', 2, 'Indicator', 'fun',
                          'TagFunction', lambda X, Y, L: comb_aniso(X, Y), 'TagBuffer', 0, 'MinBoxWidth', 2,
                          'MinFillRatio', 0.95, 'Verbose', 0, 'RelTol', 1e-10, 'MaxVCycles', 60, backend=be)
        errs.append(sol['err']['linf'])
        facs.append(sol['stats']['stages'][-1]['avgFactor'])
        mass.append(sol['mass']['rel'])
    r = np.log2(np.asarray(errs[:-1]) / np.asarray(errs[1:]))
    assert np.all(r >= RATE_BAR) and max(facs) <= 0.25 and max(abs(v) for v in mass) <= MASS_BAR


@pytest.mark.parametrize('tree', [False, True])
@pytest.mark.parametrize('name', list(BOX_CASES))
def test_hand_built_layouts(name, tree):
    """S2 corner-only adjacency, S4 hanging nodes at the boundary, S5
    minimum-width patches, S6 adversarial layouts, S7 the 5-level cross,
    ring and tree."""
    be = OracleBackend()
    errs, facs, mass = [], [], []
    for m in MS:
        H = box_case(name, m, be, tree=tree)
        errs.append(error_norms(H)['linf'])
        facs.append(H.stats['stages'][-1]['avgFactor'])
        mass.append(be.mass_check(H)['rel'])
    _check_sweep(errs, facs, mass)


@pytest.mark.parametrize('name,tree', [('EDGEKISS', False), ('EDGEKISS2', False), ('CHECKER', True),
                                       ('CHECKER3', True), ('EDGEKISS', True), ('EDGEKISS2', True)])
def test_fill_down_face_copies_identical(name, tree):
    """S6: both stored copies of a face shared by abutting same-level patches
    carry the same coefficient after the fill-down."""
    H = box_case(name, 32, OracleBackend(), rtol=1e-9, maxv=2, tree=tree)
    dup = 0.0
    for k in range(1, H.nlev + 1):
        lev = H.lev[k]
        for a in range(lev.np):
            ab = lev.box[a]
            for b in range(lev.np):
                if a == b:
                    continue
                bb = lev.box[b]
                if ab[1] + 1 == bb[0]:
                    j0, j1 = max(ab[2], bb[2]), min(ab[3], bb[3])
                    if j0 <= j1:
                        va = lev.DeW[a][ab[1] - ab[0] + 1, j0 - ab[2]:j1 - ab[2] + 1]
                        vb = lev.DeW[b][0, j0 - bb[2]:j1 - bb[2] + 1]
                        dup = max(dup, float(np.max(np.abs(va - vb))))
                if ab[3] + 1 == bb[2]:
                    i0, i1 = max(ab[0], bb[0]), min(ab[1], bb[1])
                    if i0 <= i1:
                        va = lev.DnS[a][i0 - ab[0]:i1 - ab[0] + 1, ab[3] - ab[2] + 1]
                        vb = lev.DnS[b][i0 - bb[0]:i1 - bb[0] + 1, 0]
                        dup = max(dup, float(np.max(np.abs(va - vb))))
    assert dup <= 1e-14


@pytest.mark.parametrize('depth', [3, 4, 5])
def test_deep_cross_point(depth):
    be = OracleBackend()
    H = build_boxes(problem('V'), 32, BOX_CASES['DEEPCROSS5'][1][:depth - 1], 1e-10, 60, be)
    assert H.stats['stages'][-1]['avgFactor'] <= FAC_BAR
    assert abs(be.mass_check(H)['rel']) <= MASS_BAR


@pytest.mark.parametrize('name', ['COMB', 'ANNULUS', 'EDGEKISS2', 'RINGTOUCH', 'CHECKER3', 'DEEPCROSS5'])
def test_mass_defect_scales_with_tolerance(name):
    """S8a: no tolerance-independent defect floor."""
    be = OracleBackend()
    md = []
    for tol in (1e-10, 1e-12):
        if name in ('COMB', 'ANNULUS'):
            sol = tag_case('COMB-qif' if name == 'COMB' else 'ANNULUS', 64, be, rtol=tol, maxv=90)
            md.append(abs(sol['mass']['rel']))
        else:
            pname, levels = BOX_CASES[name]
            H = build_boxes(problem(pname), 64, [scale_boxes(b, 2) for b in levels], tol, 90, be)
            md.append(abs(be.mass_check(H)['rel']))
    assert md[0] <= MASS_BAR and md[1] <= 1e-12, md


def test_corrections_off_break_conservation():
    """S8b: with the flux corrections off the comb's defect grows by orders
    of magnitude."""
    be = OracleBackend()
    on = tag_case('COMB-qif', 64, be, rtol=1e-11, maxv=90, MassCorrection=True)['mass']['rel']
    off = tag_case('COMB-qif', 64, be, rtol=1e-11, maxv=90, MassCorrection=False)['mass']['rel']
    assert abs(off) > 1e3 * max(abs(on), 1e-16), (on, off)


def test_singular_neumann_exotic_meshes():
    """S9: annulus and checkerboard meshes, singular Neumann, SourceQuad 3."""
    be = OracleBackend()
    errs, facs, mass = [], [], []
    for m in MS:
        sol = tag_case('ANNULUS', m, be, prob=problem('N'), SourceQuad=3)
        errs.append(sol['err']['linf'])
        facs.append(sol['stats']['stages'][-1]['avgFactor'])
        mass.append(sol['mass']['rel'])
    r = np.log2(np.asarray(errs[:-1]) / np.asarray(errs[1:]))
    assert np.all(r >= RATE_BAR) and max(facs) <= FAC_BAR and max(abs(v) for v in mass) <= 1e-10
    errs, facs = [], []
    for m in MS[:2]:
        o = ebOptions('BaseCells', [m, m], 'SourceQuad', 3, 'Verbose', 0, 'RelTol', 1e-10, 'MaxVCycles', 60)
        H = hier.setup(problem('N'), o, be)
        H = hier.add_level(H, scale_boxes(_checker(8, 1), m // 32), be)
        H = ebSolveCycles(H, be)
        mz, _ = be.composite_mean(H)
        for k in range(1, H.nlev + 1):
            for p in range(H.lev[k].np):
                H.lev[k].Q[p] = H.lev[k].Q[p] - mz
        errs.append(error_norms(H)['linf'])
        facs.append(H.stats['stages'][-1]['avgFactor'])
    assert np.log2(errs[0] / errs[1]) >= RATE_BAR and max(facs) <= FAC_BAR


S10 = [('CORNER4', 32), ('CORNER4', 64), ('CHAIN', 32), ('RINGTOUCH', 32), ('SKINNY3', 32), ('CHECKER', 32),
       ('CHECKER', 64), ('CHECKER3', 32), ('SPIRAL', 32), ('CORRIDORS', 32), ('EDGEKISS2', 32), ('EDGEKISS2', 64),
       ('DEEPCROSS5', 32), ('DEEPCROSS5', 64), ('HANGQ3-V', 32)]


@pytest.mark.parametrize('name,m', S10)
def test_ring_and_tree_agree_on_identical_meshes(name, m):
    """S10 (stressTreeInterfaces.m:317-345): the ring and tree solvers on the
    same hand-built mesh agree to 1e-11 with equal V-cycle counts."""
    be = OracleBackend()
    levels = BOX_CASES['HANGQ3-MX'][1] if name == 'HANGQ3-V' else BOX_CASES[name][1]
    lv = [scale_boxes(b, m // 32) for b in levels]
    Hr = build_boxes(problem('V'), m, lv, 1e-10, 60, be)
    Ht = build_boxes(problem('V'), m, lv, 1e-10, 60, be, tree=True)
    assert Hr.stats['stages'][-1]['vcycles'] == Ht.stats['stages'][-1]['vcycles']
    d = 0.0
    for k in range(Hr.rootIdx, Hr.nlev + 1):
        for qa, qb in zip(Hr.lev[k].Q, Ht.lev[k].Q):
            d = max(d, float(np.max(np.abs(qa[1:-1, 1:-1] - qb[1:-1, 1:-1]))))
    assert d <= 1e-11, d


# ------------------------------------------------------------------ GPU tests
def _assert_same(Ho, Hd):
    for so, sd in zip(Ho.stats['stages'], Hd.stats['stages']):
        np.testing.assert_array_equal(so['resHist'], sd['resHist'])
    assert Ho.nlev == Hd.nlev
    for k in range(Ho.rootIdx, Ho.nlev + 1):
        for qa, qb in zip(Ho.lev[k].Q, Hd.lev[k].Q):
            np.testing.assert_array_equal(qa, qb)


@pytest.mark.gpu
@pytest.mark.parametrize('tree', [False, True])
@pytest.mark.parametrize('name', list(BOX_CASES))
def test_hand_built_layouts_device_bitwise(name, tree):
    from bsam.device import DeviceBackend
    _assert_same(box_case(name, 64, OracleBackend(), tree=tree), box_case(name, 64, DeviceBackend.get(0), tree=tree))


@pytest.mark.gpu
@pytest.mark.parametrize('tree', [False, True])
@pytest.mark.parametrize('name', list(TAG_CASES) + ['COMBB-NN'])
def test_tag_driven_interfaces_device_bitwise(name, tree):
    from bsam.device import DeviceBackend
    base = 'COMBB' if name == 'COMBB-NN' else name
    prob = problem(TAG_PROBLEM.get(name, 'V'))
    o = tag_case(base, 64, OracleBackend(), prob=prob, tree=tree)
    d = tag_case(base, 64, DeviceBackend.get(0), prob=prob, tree=tree)
    _assert_same(o['H'], d['H'])
