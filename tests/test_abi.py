"""The C-ABI library builds, loads and exports every entry point declared in
include/bsam_dev.h; on a machine without a GB300 the context call fails
with BSAM_ERR_NODEV instead of falling back to anything."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, 'include', 'bsam_dev.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'^\s*(?:int|const char \*)\s*(bsam_\w+)\s*\(', src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared()
    for must in ('bsam_ctx_create', 'bsam_hier_upload', 'bsam_solve_cycles', 'bsam_fill_ghosts',
                 'bsam_comp_residual', 'bsam_mass_check', 'bsam_last_error'):
        assert must in names


def test_library_exports_every_declared_symbol():
    from bsam.build import build_dev
    lib = ctypes.CDLL(build_dev())
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_host_library_exports():
    from bsam.build import build_host
    lib = ctypes.CDLL(build_host())
    for n in ('bsam_vexp', 'bsam_vtanh', 'bsam_vcosh', 'bsam_starfish_new', 'bsam_starfish_distance'):
        assert hasattr(lib, n)


def test_no_device_is_an_error_not_a_fallback():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip('a GPU is present')
    except ImportError:
        pass
    from bsam.device import Context, DeviceError
    with pytest.raises(DeviceError) as ei:
        Context(0)
    assert ei.value.code == 5 and ei.value.ident == 'bsam:device:nodev'
