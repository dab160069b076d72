"""The allocation-free residual entry point agrees with the resident-hierarchy
residual (bsam_comp_residual) on the same state.

bsam_patch_residual_noalloc is for callers that cannot call cudaMalloc: it
works on device arrays the caller already owns (here: torch tensors standing
in for a host framework's memory pool) and keeps its reduction scratch in a
static device array.  This file runs last so that a failure here leaves the
rest of the suite already run; it passes alone and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _uniform_state():
    """A uniform 128^2 vardc problem after two V-cycles on the device."""
    from bsam import ebOptions
    from bsam.solve import build_hierarchy
    from bsam.flat import flatten, PD_MX, PD_MY, PD_QOFF, PD_COFF, PD_DEWOFF, PD_DNSOFF, LD_P0
    from bsam.device import DeviceBackend, DevHier
    from cases import vardc_problem
    opts = ebOptions('BaseCells', 128, 'MaxLevels', 1, 'Verbose', 0, 'RelTol', 1e-11)
    backend = DeviceBackend.get(0)
    H = build_hierarchy(vardc_problem(), opts, backend)
    fl = flatten(H)
    dh = DevHier(backend.ctx, fl, opts)
    dh.vcycle()
    dh.vcycle()
    ref = dh.residual()
    Q = dh.get(0, fl.Q.size)
    r = fl.patches[fl.levels[H.rootIdx - 1, LD_P0]]
    mx, my = int(r[PD_MX]), int(r[PD_MY])
    q0, c0, e0, n0 = int(r[PD_QOFF]), int(r[PD_COFF]), int(r[PD_DEWOFF]), int(r[PD_DNSOFF])
    arrays = {
        'Q': Q[q0:q0 + (mx + 2) * (my + 2)],
        'FTrue': fl.FTrue[c0:c0 + mx * my],
        'DeW': fl.DeW[e0:e0 + (mx + 1) * my],
        'DnS': fl.DnS[n0:n0 + mx * (my + 1)],
        'CC': fl.CC[c0:c0 + mx * my],
        'covered': fl.covered[c0:c0 + mx * my],
    }
    return ref, arrays, mx, my, H.lev[H.rootIdx].h


def test_noalloc_residual_matches_resident_residual_twice():
    import torch
    from bsam.device import lib, check
    ref, arrays, mx, my, h = _uniform_state()
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to('cuda:0') for k, v in arrays.items()}
    out = torch.zeros(5, dtype=torch.float64, device='cuda:0')
    fn = lib().bsam_patch_residual_noalloc
    fn.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    want = np.array([ref['linf'], ref['l2'], ref['fnorm'], ref['rel'], ref['ncell']])
    for _ in range(2):   # two calls in a row share (and must re-clear) the static scratch
        out.zero_()
        check(fn(dev['Q'].data_ptr(), dev['FTrue'].data_ptr(), dev['DeW'].data_ptr(), dev['DnS'].data_ptr(),
                 dev['CC'].data_ptr(), dev['covered'].data_ptr(), mx, my, h[0], h[1], out.data_ptr(), None))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[0] == want[0] and got[2] == want[2] and got[3] == want[3] and got[4] == want[4], (got, want)
        assert abs(got[1] - want[1]) <= 1e-12 * want[1], (got, want)


def _fn():
    from bsam.device import lib
    fn = lib().bsam_patch_residual_noalloc
    fn.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    return fn


def _plain_residual(a, mx, my, hx, hy):
    """numpy restatement of the plain residual the entry point computes:
    r = FTrue - op2d(Q) (ebKernels.m:13-25, same operation order; a true
    division by h^2 unless h^2 is a power of two, where the exact reciprocal
    gives the same bits), norms over the cells whose covered byte is 0,
    max-norms ignoring NaN (0 when nothing is left)."""
    Qp = a['Q'].reshape(my + 2, mx + 2)
    q, qe, qw, qn, qs = Qp[1:-1, 1:-1], Qp[1:-1, 2:], Qp[1:-1, :-2], Qp[2:, 1:-1], Qp[:-2, 1:-1]
    DeW = a['DeW'].reshape(my, mx + 1)
    DnS = a['DnS'].reshape(my + 1, mx)
    feE = DeW[:, 1:] * (qe - q)
    feW = DeW[:, :-1] * (q - qw)
    fnN = DnS[1:, :] * (qn - q)
    fnS = DnS[:-1, :] * (q - qs)
    hx2, hy2 = hx * hx, hy * hy
    op = ((-(feE - feW)) / hx2 - (fnN - fnS) / hy2) + a['CC'].reshape(my, mx) * q
    r = (a['FTrue'].reshape(my, mx) - op).ravel()
    vis = a['covered'] == 0
    rv, fv = np.abs(r[vis]), np.abs(a['FTrue'][vis])
    nanmax = lambda v: float(np.max(v[~np.isnan(v)])) if np.any(~np.isnan(v)) else 0.0
    linf, fnorm = nanmax(rv), nanmax(fv)
    l2 = float(np.sqrt(np.sum(rv * rv) * hx * hy))
    fn = max(fnorm, 2.2250738585072014e-308)
    return np.array([linf, l2, fnorm, linf / fn, float(vis.sum())])


def _random_patch(mx, my, seed, cover_frac):
    g = np.random.default_rng(seed)
    return {'Q': g.standard_normal((mx + 2) * (my + 2)), 'FTrue': g.standard_normal(mx * my) * 10,
            'DeW': g.uniform(0.1, 10, (mx + 1) * my), 'DnS': g.uniform(0.1, 10, mx * (my + 1)),
            'CC': g.uniform(0, 1, mx * my), 'covered': (g.uniform(0, 1, mx * my) < cover_frac).astype(np.uint8)}


def _call(a, mx, my, hx, hy):
    import torch
    from bsam.device import check
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to('cuda:0') for k, v in a.items()}
    out = torch.full((5,), -1.0, dtype=torch.float64, device='cuda:0')
    check(_fn()(dev['Q'].data_ptr(), dev['FTrue'].data_ptr(), dev['DeW'].data_ptr(), dev['DnS'].data_ptr(),
                dev['CC'].data_ptr(), dev['covered'].data_ptr(), mx, my, hx, hy, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _agree(got, want):
    # max-norms are order-free: bitwise; the L2 sum is reduced in another order
    assert got[0] == want[0] and got[2] == want[2] and got[3] == want[3] and got[4] == want[4], (got, want)
    assert abs(got[1] - want[1]) <= 1e-12 * want[1], (got, want)


@pytest.mark.parametrize('mx,my,hx,hy,cover', [
    (96, 40, 0.1, 0.3, 0.3),          # h^2 not a power of two: true divisions
    (130, 70, 1 / 64, 1 / 32, 0.5),   # power-of-two h^2, half the cells covered by a finer level
])
def test_noalloc_plain_residual_with_covered_mask(mx, my, hx, hy, cover):
    a = _random_patch(mx, my, 7 + mx, cover)
    want = _plain_residual(a, mx, my, hx, hy)
    for _ in range(2):
        _agree(_call(a, mx, my, hx, hy), want)


def test_noalloc_at_the_size_limit():
    """Exactly BSAM_NOALLOC_MAX_BLOCKS * 256 = 4,194,304 cells (2048^2): the
    largest patch the static scratch admits, every block partial used."""
    mx = my = 2048
    a = _random_patch(mx, my, 11, 0.1)
    _agree(_call(a, mx, my, 1 / 2048, 1 / 2048), _plain_residual(a, mx, my, 1 / 2048, 1 / 2048))


def test_noalloc_max_norms_ignore_nan():
    """NaN values (ordinary input data) drop out of linf and fnorm as in
    MATLAB's max; the L2 sum carries them."""
    mx, my = 64, 48
    a = _random_patch(mx, my, 5, 0.0)
    a['FTrue'][:512] = np.nan             # two whole 256-cell blocks of NaN
    a['Q'][(mx + 2) * 20 + 30] = np.nan   # and one solution value
    want = _plain_residual(a, mx, my, 1 / 64, 1 / 64)
    got = _call(a, mx, my, 1 / 64, 1 / 64)
    assert np.isfinite(want[0]) and np.isfinite(want[2])
    assert got[0] == want[0] and got[2] == want[2] and got[3] == want[3] and got[4] == want[4], (got, want)
    assert np.isnan(got[1]) and np.isnan(want[1])


def test_noalloc_rejects_oversized_patch():
    from bsam.device import lib
    fn = lib().bsam_patch_residual_noalloc
    fn.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    rc = fn(dummy, dummy, dummy, dummy, dummy, None, 4096, 4096, 1.0, 1.0, dummy, None)
    assert rc == 1
    assert b'no-allocation limit' in lib().bsam_last_error()
