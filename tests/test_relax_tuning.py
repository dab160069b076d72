"""Smoother autotuner: the launch form of each level's relaxation -- 1, 2 or
4 colour cells updated per thread with one launch per colour pass,
persistent blocks (form 3), or every pass and the closing fill in one launch
of a single thread-block cluster, reading the solution from L2 (form 0) or
holding the level's solution in the cluster's distributed shared memory
(form 5, on levels whose Q range fits it) -- is picked per level and
precision at the first solve of a hierarchy, by timing the candidates on the
live state.  The choice may
differ run to run, so it must never change a result bit: each forced form
(BSAM_RELAX_N, on every level) and the tuned one give the same V-cycle
count, residual history and solution, in the FP64 cycle
(ebRelaxLevel.m:28-38 per sweep) and the FP32 correction cycle.
"""
import numpy as np
import pytest

from bsam import ebOptions
from bsam.flat import flatten
from bsam.solve import build_hierarchy
from bsam_oracle import OracleBackend
from cases import vardc_problem

pytestmark = pytest.mark.gpu

WIDE_BAND = lambda x, y: np.abs(x - y) < 0.4


def _flat(precision):
    o = ebOptions('BaseCells', 128, 'MaxLevels', 3, 'Indicator', 'fun', 'TagFunction', WIDE_BAND, 'Verbose', 0,
                  'RelTol', 1e-10, 'Precision', precision)
    return flatten(build_hierarchy(vardc_problem(), o, OracleBackend())), o


def _solve(fl, o):
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q
    dh = DevHier(DeviceBackend.get(0).ctx, fl, o)
    it, hist, rel, _ = dh.solve_cycles(o.MaxVCycles + 2)
    return dh, it, hist, dh.get(BSAM_FIELD_Q, fl.Q.size)


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_every_coarsening_gives_the_same_bits(precision, monkeypatch):
    fl, o = _flat(precision)
    monkeypatch.delenv('BSAM_RELAX_N', raising=False)
    dh, it, hist, Q = _solve(fl, o)
    p = 1 if precision == 'mixed' else 0
    tuned = dh.relax_tuning(p)
    assert set(tuned.tolist()) <= {0, 1, 2, 3, 4, 5} and tuned[0] == 1
    assert np.all(dh.relax_tuning(1 - p) == -1)     # that cycle never ran
    for kn in (0, 1, 2, 3, 4, 5):
        monkeypatch.setenv('BSAM_RELAX_N', str(kn))
        dk, itk, histk, Qk = _solve(fl, o)
        forms = dk.relax_tuning(p)[1:]
        if kn == 5:     # where a level fits: here the coarser ones
            assert set(forms.tolist()) <= {1, 5} and forms[0] == 5, forms
        else:
            assert np.all(forms == kn)
        assert itk == it
        np.testing.assert_array_equal(histk, hist)
        np.testing.assert_array_equal(Qk, Q)


def test_fp64_rate_is_measured():
    """The FP64 issue-rate probe (the FP64 roofline's denominator) returns a
    plausible figure: above 50 Gop/s, below the FP32 rate of any GPU."""
    from bsam.device import DeviceBackend, fp64_rate
    g = fp64_rate(DeviceBackend.get(0).ctx)
    assert 50 < g < 1e5, g
