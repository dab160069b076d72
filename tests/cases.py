"""Problem definitions shared by the tests (the reference's own cases)."""
import numpy as np

from bsam import ebProblem


def config1_problem(tree=False):
    """The reference's README elliptic example (its top-level README.md: -Laplace(u) + u = f, Dirichlet 0)."""
    u = lambda x, y: np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
    f = lambda x, y: (1 + 8 * np.pi ** 2) * u(x, y)
    return ebProblem([0, 1, 0, 1], 1, 1, f, ('dirichlet', 0), u)


def vardc_problem():
    """mmsCases('vardc') (EllipticBSAM/tests/mmsCases.m:4-16)."""
    uex = lambda x, y: np.sin(np.pi * x) * np.cos(np.pi * y)
    D = lambda x, y: 1 + 0.5 * np.sin(2 * np.pi * x) * np.cos(np.pi * y)
    C = lambda x, y: 1 + x * y
    Dx = lambda x, y: np.pi * np.cos(2 * np.pi * x) * np.cos(np.pi * y)
    Dy = lambda x, y: -0.5 * np.pi * np.sin(2 * np.pi * x) * np.sin(np.pi * y)
    ux = lambda x, y: np.pi * np.cos(np.pi * x) * np.cos(np.pi * y)
    uy = lambda x, y: -np.pi * np.sin(np.pi * x) * np.sin(np.pi * y)
    lap = lambda x, y: -2 * np.pi ** 2 * uex(x, y)
    f = lambda x, y: -(Dx(x, y) * ux(x, y) + Dy(x, y) * uy(x, y) + D(x, y) * lap(x, y)) + C(x, y) * uex(x, y)
    return ebProblem([0, 1, 0, 1], D, C, f, ('dirichlet', uex), uex)


def pureneumann_problem():
    """mmsCases('pureneumann') (EllipticBSAM/tests/mmsCases.m:18-22)."""
    uex = lambda x, y: np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    f = lambda x, y: 8 * np.pi ** 2 * uex(x, y)
    return ebProblem([0, 1, 0, 1], 1, 0, f, ('neumann', 0), uex)


def gauss51_problem():
    """mmsCases('gauss51') (EllipticBSAM/tests/mmsCases.m:24-32): u - lap u = f,
    homogeneous Neumann on (-0.25, 0.25)^2."""
    from bsam import hostlib
    sg = 0.25
    gp = lambda t: -np.pi * np.sin(4 * np.pi * t) / sg ** 2
    gpp = lambda t: -4 * np.pi ** 2 * np.cos(4 * np.pi * t) / sg ** 2
    uex = lambda x, y: hostlib.exp(-(np.sin(2 * np.pi * x) ** 2 + np.sin(2 * np.pi * y) ** 2) / (2 * sg ** 2))
    f = lambda x, y: uex(x, y) * (1 - (gpp(x) + gp(x) ** 2 + gpp(y) + gp(y) ** 2))
    return ebProblem([-0.25, 0.25, -0.25, 0.25], 1, 1, f, ('neumann', 0), uex)


def box_in_box_tag(X, Y, L):
    """T3 tag function (EllipticBSAM/tests/runAllTests.m:53-56)."""
    return ((L == 1) * (np.maximum(np.abs(X), np.abs(Y)) < 0.1875)
            + (L == 2) * (np.maximum(np.abs(X), np.abs(Y)) < 0.125)
            + (L == 3) * (np.maximum(np.abs(X), np.abs(Y)) < 0.0625))


def printed_close(value, printed):
    """True when `value` rounds to the printed decimal string `printed`
    (half a unit in its last digit, plus a little slack)."""
    s = printed.strip()
    if 'e' in s.lower():
        mant, ex = s.lower().split('e')
        dec = len(mant.split('.')[1]) if '.' in mant else 0
        ulp = 10.0 ** (int(ex) - dec)
    else:
        dec = len(s.split('.')[1]) if '.' in s else 0
        ulp = 10.0 ** (-dec)
    return abs(value - float(s)) <= 0.5 * ulp * (1 + 1e-9) + 1e-300


def gauss52_problem():
    """mmsCases('gauss52') (EllipticBSAM/tests/mmsCases.m:34-39, makeGauss52
    :62-82): three periodic Gaussians on [0,1]^2, u - lap u = f, Dirichlet."""
    sg = 0.25
    xi, yi, Ai = (0.4375, 0.4375, 0.5625), (0.5625, 0.4375, 0.4375), (1.0, -1.0, 1.0)

    def uex(x, y):
        v = 0
        for i in range(3):
            v = v + Ai[i] * np.exp(-(np.sin(x - xi[i]) ** 2 + np.sin(y - yi[i]) ** 2) / (2 * sg ** 2))
        return v

    def f(x, y):
        v = 0
        for i in range(3):
            gi = np.exp(-(np.sin(x - xi[i]) ** 2 + np.sin(y - yi[i]) ** 2) / (2 * sg ** 2))
            gpx = -np.sin(2 * (x - xi[i])) / (2 * sg ** 2)
            gppx = -np.cos(2 * (x - xi[i])) / sg ** 2
            gpy = -np.sin(2 * (y - yi[i])) / (2 * sg ** 2)
            gppy = -np.cos(2 * (y - yi[i])) / sg ** 2
            v = v + Ai[i] * gi * (1 - (gppx + gpx ** 2 + gppy + gpy ** 2))
        return v
    return ebProblem([0, 1, 0, 1], 1, 1, f, ('dirichlet', uex), uex)


def threebumps_problem():
    """mmsCases('threebumps') (EllipticBSAM/tests/mmsCases.m:41-53)."""
    s = 0.02
    xi, yi, Ai = (0.30, 0.66, 0.49), (0.34, 0.42, 0.72), (1.0, 0.8, -0.9)
    g = lambda x, y, a, b: np.exp(-((x - a) ** 2 + (y - b) ** 2) / (2 * s ** 2))
    lg = lambda x, y, a, b: g(x, y, a, b) * (((x - a) ** 2 + (y - b) ** 2) / s ** 4 - 2 / s ** 2)
    uex = lambda x, y: (Ai[0] * g(x, y, xi[0], yi[0]) + Ai[1] * g(x, y, xi[1], yi[1])) + Ai[2] * g(x, y, xi[2], yi[2])
    lap = lambda x, y: (Ai[0] * lg(x, y, xi[0], yi[0]) + Ai[1] * lg(x, y, xi[1], yi[1])) + Ai[2] * lg(x, y, xi[2], yi[2])
    f = lambda x, y: uex(x, y) - lap(x, y)
    return ebProblem([0, 1, 0, 1], 1, 1, f, ('dirichlet', uex), uex)


def lshape_tag(X, Y, L):
    """T4 tag (EllipticBSAM/tests/runAllTests.m:89-90)."""
    return (((X >= 0.375) & (X <= 0.625) & (Y >= 0.375) & (Y <= 0.5)) |
            ((X >= 0.375) & (X <= 0.5) & (Y >= 0.5) & (Y <= 0.625)))


def scattered_tag():
    """T8 tag (runAllTests.m:207-212): 24 disks of radius 0.02 at rand(24,2)
    after rng(42) -- MATLAB's default generator is MT19937 seeded like
    numpy's legacy RandomState, with the same 53-bit doubles; rand fills the
    24x2 matrix column by column."""
    r = np.random.RandomState(42).random_sample(48)
    px, py = r[:24], r[24:]

    def tag(X, Y, L):
        Xv, Yv = np.asarray(X).reshape(-1, 1, order='F'), np.asarray(Y).reshape(-1, 1, order='F')
        hit = np.any((Xv - px[None, :]) ** 2 + (Yv - py[None, :]) ** 2 < 0.0004, axis=1)
        return hit.reshape(np.shape(X), order='F')
    return tag


def starfish_config2(backend):
    """The diffuse-domain starfish of examples/demoStarfish.m:11-20 (64^2 base
    refined through 5 levels, tag |d| < max(3 eps, 3*4/(64 2^(L-1))), buffer 2,
    RelTol 1e-10, MaxVCycles 100): the hierarchy of the benchmarked solve,
    built on `backend`, and its options."""
    import warnings
    from bsam import ebOptions
    from bsam.ddm import starfish_problem, starfish_tag
    from bsam.solve import build_hierarchy
    prob, aux, g = starfish_problem()
    opts = ebOptions('BaseCells', 64, 'MaxLevels', 5, 'Indicator', 'fun', 'TagFunction', starfish_tag(g),
                     'TagBuffer', 2, 'RelTol', 1e-10, 'MaxVCycles', 100, 'Verbose', 0)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        H = build_hierarchy(prob, opts, backend)
    return H, opts
