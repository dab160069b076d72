"""Diffuse-domain geometry sweep (DiffuseDomainBSAM/tests/runDdGeometries.m)
on the oracle: each ddGeometry kind in a real adaptive solve.

G1 Neumann form (u = r^2/4 with g = grad u . n_psi) on the circle, ellipse,
   pentagon, flower3, peanut and the 5-lobe star, eps = 0.2 and 0.1 at
   fixed eps/h: conservation (relative mass defect <= 1e-11), V-cycle factor
   <= 0.35, every refined patch touching the tag band, and the L2 error
   decaying at the per-geometry rate the reference asserts.
G2 Dirichlet penalty on the pentagon: the L2 error decreases monotonically
   in eps.
The reference records no numbers for this script; these are its pass
criteria.
"""
import warnings

import numpy as np
import pytest

from bsam.ddsolve import ddGeometry, ddSolve
from bsam_oracle import OracleBackend

BOX = [-2.5, 2.5, -2.5, 2.5]
UEX = lambda x, y: (x ** 2 + y ** 2) / 4
FEX = lambda x, y: (x ** 2 + y ** 2) / 4 - 1

GEOMS = {                                    # kind args, minimum L2 decay rate
    'circle': (('circle', 1.0), 0.8),
    'ellipse': (('ellipse', 1.4, 0.8), 0.8),
    'pentagon': (('pentagon', 1.2), 0.4),
    'flower3': (('flower3',), 0.8),
    'peanut': (('peanut',), 0.8),
    'star5': (('star', 0.5), 0.8),
}


def neumann_g(geom):
    def g(X, Y):
        gx, gy = geom.gpsi(X, Y)
        return (X * gx + Y * gy) / (2 * np.maximum(geom.gpsimag(X, Y), 1e-12))
    return g


def localized(H, geom, ep):
    """Every refined patch touches |psi| < 2.5 eps, with the cell-size slack
    converted to psi units by the local |grad psi| (runDdGeometries.m:144-161)."""
    for k in range(H.rootIdx + 1, H.nlev + 1):
        lev = H.lev[k]
        for b in lev.box:
            xc = BOX[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0]
            yc = BOX[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1]
            XC, YC = np.meshgrid(xc, yc, indexing='ij')
            gm = float(np.max(geom.gpsimag(XC.ravel(order='F'), YC.ravel(order='F'))))
            if np.min(np.abs(geom.psi(XC.ravel(order='F'), YC.ravel(order='F')))) > 2.5 * ep + 8 * (2 * max(lev.h)) * gm:
                return False
    return True


@pytest.mark.parametrize('name', list(GEOMS))
def test_G1_neumann_across_geometries(name):
    args, min_rate = GEOMS[name]
    geom = ddGeometry(*args)
    data = {'f': FEX, 'g': neumann_g(geom), 'C': 1, 'D': 1, 'exact': UEX}
    l2 = []
    for ep, N in ((0.2, 256), (0.1, 512)):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            sol = ddSolve(geom, ep, BOX, 'neumann', data, 'BaseCells', N // 8, 'MaxLevels', 4, 'TagWidth', 2.5,
                          'TagBuffer', 2, 'Verbose', 0, 'RelTol', 1e-10, 'MaxVCycles', 30, backend=OracleBackend())
        assert abs(sol['mass']['rel']) <= 1e-11, sol['mass']
        assert sol['stats']['stages'][-1]['avgFactor'] <= 0.35
        assert localized(sol['H'], geom, ep)
        l2.append(sol['errInside']['l2'])
    assert np.log2(l2[0] / l2[1]) >= min_rate, l2


def test_G2_pentagon_dirichlet_penalty_monotone():
    geom = ddGeometry('pentagon', 1.2)
    data = {'f': FEX, 'g': UEX, 'C': 1, 'D': 1, 'exact': UEX}
    l2 = []
    for ep, N in ((0.4, 128), (0.2, 256), (0.1, 512)):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            sol = ddSolve(geom, ep, BOX, 'dirichlet', data, 'BaseCells', N // 8, 'MaxLevels', 4, 'TagWidth', 2.5,
                          'TagBuffer', 2, 'Mu', 1, 'Verbose', 0, 'RelTol', 1e-10, 'MaxVCycles', 40,
                          backend=OracleBackend())
        l2.append(sol['errInside']['l2'])
    assert np.all(np.diff(l2) < 0), l2
