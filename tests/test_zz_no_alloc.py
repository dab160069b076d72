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


def test_noalloc_rejects_oversized_patch():
    from bsam.device import lib
    fn = lib().bsam_patch_residual_noalloc
    fn.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    rc = fn(dummy, dummy, dummy, dummy, dummy, None, 4096, 4096, 1.0, 1.0, dummy, None)
    assert rc == 1
    assert b'no-allocation limit' in lib().bsam_last_error()
