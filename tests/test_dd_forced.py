"""Forced diffuse-domain studies without a manufactured solution
(DiffuseDomainBSAM/tests/runDdForced.m), run at the reference's full sizes
through the CUDA path: pentagon, f = 1 + x/2.

F1a h-Cauchy self-convergence at eps = 0.2 (Dirichlet penalty, effective
    N = 256 .. 2048): the bulk rate (psi < -2.5 eps) reaches 1.7, the
    whole-interior rate 1.0, every mass defect <= 2e-9.
F1b eps-Cauchy at fixed h (effective 1024, eps = 0.4 .. 0.05): rates >= 1.2
    inside Omega_1 and >= 1.4 on the eroded bulk.
F2  the Dirichlet penalty's normal-derivative kink at Gamma sharpens like
    eps (uniform 1024^2, eps = 0.2, 0.1, 0.05).
F3  the Neumann flux form keeps du/dx continuous across Gamma: its jump
    over +-2 eps is far below the Dirichlet form's.
These are the script's pass criteria (it records no numbers).  F1a and F1b
also run on the oracle (a few seconds each); F2 and F3 solve 1024^2 uniform
grids and run on the device only.
"""
import warnings

import numpy as np
import pytest

from bsam.ddsolve import ddGeometry, ddSolve, ddToUniform

BOX = [-2.5, 2.5, -2.5, 2.5]
N0 = 256
GEOM = ddGeometry('pentagon', 1.2)
FFUN = lambda x, y: 1 + 0.5 * x
DATA_D = {'f': FFUN, 'g': 0, 'C': 0}


def _backend(kind='device'):
    if kind == 'oracle':
        from bsam_oracle import OracleBackend
        return OracleBackend()
    from bsam.device import DeviceBackend
    return DeviceBackend.get(0)


BACKENDS = [pytest.param('oracle'), pytest.param('device', marks=pytest.mark.gpu)]


def _grid():
    c = BOX[0] + (np.arange(1, N0 + 1) - 0.5) * (BOX[1] - BOX[0]) / N0
    X0, Y0 = np.meshgrid(c, c, indexing='ij')
    return X0, Y0, ((BOX[1] - BOX[0]) / N0) ** 2


def _solve(ep, bctype, data, *opts, kind='device'):
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return ddSolve(GEOM, ep, BOX, bctype, data, *opts, 'Verbose', 0, 'RelTol', 1e-9, 'MaxVCycles', 40,
                       backend=_backend(kind))


@pytest.mark.parametrize('kind', BACKENDS)
def test_F1a_h_cauchy(kind):
    X0, Y0, da0 = _grid()
    ep = 0.2
    inside = GEOM.psi(X0, Y0) < 0
    bulk = GEOM.psi(X0, Y0) < -2.5 * ep
    U = []
    for N in (256, 512, 1024, 2048):
        sol = _solve(ep, 'dirichlet', DATA_D, 'BaseCells', N // 8, 'MaxLevels', 4, 'TagWidth', 2.5, 'TagBuffer', 2,
                     'Mu', 1, kind=kind)
        assert sol['mass']['rel'] <= 2e-9
        U.append(ddToUniform(sol['H'], N0)[0])
    dh = [np.sqrt(np.sum((U[i] - U[i + 1])[inside] ** 2) * da0) for i in range(3)]
    dhb = [np.sqrt(np.sum((U[i] - U[i + 1])[bulk] ** 2) * da0) for i in range(3)]
    assert np.log2(dhb[-2] / dhb[-1]) >= 1.7, dhb
    assert np.log2(dh[-2] / dh[-1]) >= 1.0, dh


@pytest.mark.parametrize('kind', BACKENDS)
def test_F1b_eps_cauchy(kind):
    X0, Y0, da0 = _grid()
    epsl = (0.4, 0.2, 0.1, 0.05)
    inside = GEOM.psi(X0, Y0) < 0
    eroded = GEOM.psi(X0, Y0) < -2 * max(epsl)
    U = [ddToUniform(_solve(ep, 'dirichlet', DATA_D, 'BaseCells', 128, 'MaxLevels', 4, 'TagWidth', 2.5,
                            'TagBuffer', 2, 'Mu', 1, kind=kind)['H'], N0)[0] for ep in epsl]
    de = np.array([np.sqrt(np.sum((U[j] - U[j + 1])[inside] ** 2) * da0) for j in range(3)])
    dee = np.array([np.sqrt(np.sum((U[j] - U[j + 1])[eroded] ** 2) * da0) for j in range(3)])
    assert np.all(np.log2(de[:-1] / de[1:]) >= 1.2), de
    assert np.all(np.log2(dee[:-1] / dee[1:]) >= 1.4), dee


def _profiles(bctype, data):
    """u and du/dx along the cell row nearest y = 0 of a uniform 1024^2 solve."""
    Nu = 1024
    h = (BOX[1] - BOX[0]) / Nu
    xs = BOX[0] + (np.arange(1, Nu + 1) - 0.5) * h
    j0 = int(round((0 - BOX[2]) / h + 0.5))
    out = {}
    for ep in (0.2, 0.1, 0.05):
        sol = _solve(ep, bctype, data, 'BaseCells', Nu, 'MaxLevels', 1)
        u = sol['H'].lev[sol['H'].nlev].Q[0][1:-1, j0]
        du = np.full(u.shape, np.nan)
        du[1:-1] = (u[2:] - u[:-2]) / (2 * h)
        out[ep] = du
    return xs, h, out


XG = 1.2 * np.cos(np.pi / 5) / np.cos(np.pi / 10)      # where the pentagon's right edge meets y = 0


@pytest.mark.gpu
def test_F2_dirichlet_kink_sharpens_like_eps():
    xs, h, dprof = _profiles('dirichlet', DATA_D)
    width = []
    for ep, du in dprof.items():
        win = (xs > XG - 3.5 * ep) & (xs < XG + 3.5 * ep)
        dw = du[win]
        lout = np.interp(XG + 2.5 * ep, xs, du)
        slope_in = float(np.min(dw))
        ddu = (dw[2:] - dw[:-2]) / (2 * h)
        width.append((lout - slope_in) / np.max(ddu))
    width = np.array(width)
    eps = np.array(list(dprof))
    assert np.all(np.isfinite(width)) and np.all(np.diff(width) < 0), width
    assert width[-1] / width[0] <= 0.55 and np.all(width <= 1.5 * eps), width


@pytest.mark.gpu
def test_F3_neumann_flux_form_derivative_continuous():
    _, _, dD = _profiles('dirichlet', DATA_D)
    xs, _, dN = _profiles('neumann', {'f': FFUN, 'g': 0.3, 'C': 1})
    for ep in dN:
        jn = abs(np.interp(XG + 2 * ep, xs, dN[ep]) - np.interp(XG - 2 * ep, xs, dN[ep]))
        jd = abs(np.interp(XG + 2 * ep, xs, dD[ep]) - np.interp(XG - 2 * ep, xs, dD[ep]))
        assert jn < 0.5 * jd, (ep, jn, jd)
