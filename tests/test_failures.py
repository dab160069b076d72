"""Failure behaviour, injected on the host only (nothing here faults, traps
or hangs a GPU): malformed upload tables are rejected with bsam:device:arg
before anything is copied; a MaxVCycles stall, a NaN in the source and a
checkpoint/resume behave exactly as on the oracle / an uninterrupted run.
"""
import numpy as np
import pytest

from bsam import ebOptions
from bsam.flat import flatten, PD_QOFF, PD_RING0, LD_P0, LD_P1
from bsam.solve import build_hierarchy
from bsam_oracle import OracleBackend, OracleHier
from cases import config1_problem, vardc_problem

pytestmark = pytest.mark.gpu

BAND = lambda x, y: np.abs(x - y) < 0.15


def _flat(**kw):
    o = dict(BaseCells=32, MaxLevels=3, Indicator='fun', TagFunction=BAND, Verbose=0, RelTol=1e-10)
    o.update(kw)
    opts = ebOptions(*sum(o.items(), ()))
    return flatten(build_hierarchy(vardc_problem(), opts, OracleBackend())), opts


def _upload(fl, opts):
    from bsam.device import DeviceBackend, DevHier
    return DevHier(DeviceBackend.get(0).ctx, fl, opts)


@pytest.mark.parametrize('corruption', ['q_offset', 'ring_index', 'level_tiling', 'coarsest_size', 'batch_instance',
                                        'batch_order'])
def test_malformed_tables_are_rejected(corruption):
    from bsam.device import DeviceError
    from bsam.batch import merge_flats
    fl, opts = _flat()
    if corruption == 'q_offset':
        fl.patches = fl.patches.copy()
        fl.patches[-1, PD_QOFF] = fl.Q.size          # past the end of Q
    elif corruption == 'ring_index':
        fl.ring = fl.ring.copy()
        fl.ring[0, 1] = fl.QC.size + 5
    elif corruption == 'level_tiling':
        fl.levels = fl.levels.copy()
        fl.levels[0, LD_P1] += 1                     # levels overlap
    elif corruption == 'coarsest_size':
        fl.bcRhs = fl.bcRhs[:-1]
    elif corruption == 'batch_instance':
        fl = merge_flats([fl, _flat()[0]])
        fl.patch_inst = fl.patch_inst.copy()
        fl.patch_inst[-1] = 7                        # no such instance
    else:
        fl = merge_flats([fl, _flat()[0]])
        fl.patch_inst = fl.patch_inst.copy()
        p0 = int(fl.levels[fl.nlev - 1, LD_P0])
        fl.patch_inst[p0] = 1                        # finest level: instance 1 before instance 0
    with pytest.raises(DeviceError) as ei:
        _upload(fl, opts)
    assert 'bsam:device:arg' in str(ei.value) or ei.value.args[0] == 1


def test_maxvcycles_stall_matches_oracle():
    fl, opts = _flat(RelTol=1e-15, MaxVCycles=3)
    oh = OracleHier(fl, opts)
    it_o, hist_o, rel_o, _ = oh.solve_cycles(10)
    it_d, hist_d, rel_d, _ = _upload(fl, opts).solve_cycles(10)
    assert it_o == it_d == 3 and rel_d > 1e-15
    np.testing.assert_array_equal(hist_o, hist_d)


def test_nan_in_source_matches_oracle():
    """A NaN in the source propagates as on the oracle (the max-norms skip it
    like the reference's max); both stop after the same V-cycles."""
    fl, opts = _flat(MaxVCycles=6)
    fl.FTrue = fl.FTrue.copy()
    fl.F = fl.F.copy()
    c = fl.FTrue.size // 3
    fl.FTrue[c] = np.nan
    fl.F[c] = np.nan
    oh = OracleHier(fl, opts)
    it_o, hist_o, rel_o, _ = oh.solve_cycles(10)
    it_d, hist_d, rel_d, _ = _upload(fl, opts).solve_cycles(10)
    assert it_o == it_d
    np.testing.assert_array_equal(hist_o, hist_d)


def test_checkpoint_resume_equals_uninterrupted():
    """Two solves of 3 V-cycles on one upload equal 3 V-cycles, a host
    checkpoint, a fresh upload resumed from it, and 3 more."""
    from bsam.device import BSAM_FIELD_Q
    fl, opts = _flat(RelTol=1e-15, MaxVCycles=3)
    a = _upload(fl, opts)
    a.solve_cycles(10)
    ra = a.solve_cycles(10)
    b1 = _upload(fl, opts)
    b1.solve_cycles(10)
    cp = b1.checkpoint()
    del b1
    b2 = _upload(fl, opts)
    b2.resume(cp)
    rb = b2.solve_cycles(10)
    assert ra[0] == rb[0]
    np.testing.assert_array_equal(ra[1], rb[1])
    np.testing.assert_array_equal(a.get(BSAM_FIELD_Q, fl.Q.size), b2.get(BSAM_FIELD_Q, fl.Q.size))


def test_trace_file(tmp_path, monkeypatch):
    import json
    import bsam.device as dv
    path = tmp_path / 'trace.jsonl'
    monkeypatch.setattr(dv, '_trace_path', str(path))
    fl, opts = _flat()
    it, hist, rel, vis = _upload(fl, opts).solve_cycles(70)
    rec = [json.loads(l) for l in open(path)]
    assert rec[-1]['event'] == 'solve_cycles' and rec[-1]['vcycles'] == it
    assert rec[-1]['resHist'] == list(hist) and rec[-1]['finalRel'] == rel


def test_context_destroyed_before_its_hierarchy():
    """A hierarchy keeps its context alive: the context's handle may be
    destroyed first (as at interpreter shutdown, where finaliser order is
    arbitrary), and the hierarchy still solves and frees cleanly."""
    from bsam.device import Context, DevHier, lib
    fl, opts = _flat()
    ctx = Context(0)
    dh = DevHier(ctx, fl, opts)
    ref = _upload(fl, opts).solve_cycles(opts.MaxVCycles + 2)
    lib().bsam_ctx_destroy(ctx.h)
    ctx.h = None                        # its finaliser then has nothing to free
    it, hist, rel, vis = dh.solve_cycles(opts.MaxVCycles + 2)
    assert it == ref[0] and rel == ref[2]
    np.testing.assert_array_equal(hist, ref[1])
    del dh
