"""Batches of independent hierarchies (bsam.batch, bsam_batch_* of the C-ABI).

CPU: the merged upload tables are a relabelling of every instance's own
tables (round trip, index tables mapped back entry by entry, spacing check).
GPU: each instance of a batch ends bit for bit where its solve alone ends
(solution, coarse shadows, force, residual history, V-cycle count), with
instances that stop at different V-cycles and on different stop tests.
"""
import numpy as np
import pytest

from bsam import ebOptions
from bsam.batch import merge_flats, split_field, join_field
from bsam.flat import flatten, FIELD_Q, FIELD_QC, FIELD_F, PD_LEVEL, PD_SAME0, PD_SAME1, PD_RING0, PD_RING1
from bsam.solve import build_hierarchy
from bsam_oracle import OracleBackend
from cases import config1_problem, vardc_problem, pureneumann_problem, gauss51_problem


def _opts(**kw):
    base = dict(BaseCells=32, MaxLevels=3, Indicator='fun', Verbose=0, RelTol=1e-10,
                TagFunction=lambda x, y: (x - 0.4) ** 2 + (y - 0.55) ** 2 < 0.04)
    base.update(kw)
    args = []
    for k, v in base.items():
        args += [k, v]
    return ebOptions(*args)


def _instances():
    """Five hierarchies on the unit square with a 16x16 coarsest grid:
    different problems, depths, roots (BaseCells 32 and 64), ring and tree
    builds, and a singular all-Neumann case."""
    cases = [
        (config1_problem(), _opts(), False),
        (vardc_problem(), _opts(TagFunction=lambda x, y: np.abs(x - y) < 0.15), False),
        (config1_problem(), _opts(BaseCells=64, MaxLevels=2,
                                  TagFunction=lambda x, y: (x - 0.7) ** 2 + (y - 0.3) ** 2 < 0.02), False),
        (pureneumann_problem(), _opts(MaxLevels=2,
                                      TagFunction=lambda x, y: (x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.05), False),
        (config1_problem(), _opts(TagFunction=lambda x, y: (x - 0.3) ** 2 + (y - 0.6) ** 2 < 0.03), True),
    ]
    Hs = [build_hierarchy(p, o, OracleBackend(), tree=t) for (p, o, t) in cases]
    return Hs


@pytest.fixture(scope='module')
def parts():
    return [flatten(H) for H in _instances()]


def test_merge_round_trip(parts):
    b = merge_flats(parts)
    assert b.ninst == len(parts)
    assert b.patch_inst[:len(parts)].tolist() == list(range(len(parts)))
    assert b.inst_root.tolist() == [p.rootIdx for p in parts]
    for i, p in enumerate(parts):
        np.testing.assert_array_equal(split_field(b, FIELD_Q, b.Q, i), p.Q)
        np.testing.assert_array_equal(split_field(b, FIELD_QC, b.QC, i), p.QC)
        np.testing.assert_array_equal(split_field(b, FIELD_F, b.FTrue, i), p.FTrue)
        np.testing.assert_array_equal(split_field(b, FIELD_F, b.covered, i), p.covered)
    np.testing.assert_array_equal(join_field(b, FIELD_Q, [p.Q for p in parts]), b.Q)
    # level-major order: every merged level is a run of instances
    lv = b.patches[:, PD_LEVEL]
    assert np.all(np.diff(lv) >= 0)
    for k in range(1, b.nlev + 1):
        assert np.all(np.diff(b.patch_inst[lv == k]) >= 0)
    # the coarsest blocks are the instances' own, in instance order
    np.testing.assert_array_equal(b.Ainv, np.concatenate([np.asarray(p.Ainv).ravel() for p in parts]))


def test_merge_maps_tables_entry_by_entry(parts):
    b = merge_flats(parts)
    inv_q = np.full(b.Q.size, -1)
    inv_qc = np.full(b.QC.size, -1)
    owner_q = np.full(b.Q.size, -1)
    for i, m in enumerate(b.maps):
        inv_q[m['q']] = np.arange(m['q'].size)
        owner_q[m['q']] = i
        inv_qc[m['qc']] = np.arange(m['qc'].size)
    assert np.all(inv_q >= 0) and np.all(inv_qc >= 0)
    # walk the merged patches in order and compare their table slices
    seen = [0] * len(parts)
    for g in range(b.npatch):
        i = int(b.patch_inst[g])
        p = parts[i]
        # the instance's patches appear in its own level-major order
        lvl = int(b.patches[g, PD_LEVEL])
        own = [q for q in range(p.npatch) if int(p.patches[q, PD_LEVEL]) == lvl]
        q = own[sum(1 for gg in range(g) if b.patch_inst[gg] == i and b.patches[gg, PD_LEVEL] == lvl)]
        seen[i] += 1
        r, r0 = b.patches[g], p.patches[q]
        ms = b.same[r[PD_SAME0]:r[PD_SAME1]]
        np.testing.assert_array_equal(inv_q[ms], p.same[r0[PD_SAME0]:r0[PD_SAME1]])
        assert np.all(owner_q[ms] == i)
        if lvl > 1:
            mr = b.ring[r[PD_RING0]:r[PD_RING1]]
            np.testing.assert_array_equal(inv_q[mr[:, 0]], p.ring[r0[PD_RING0]:r0[PD_RING1], 0])
            np.testing.assert_array_equal(inv_qc[mr[:, 1]], p.ring[r0[PD_RING0]:r0[PD_RING1], 1])
    assert seen == [p.npatch for p in parts]


def test_merge_rejects_different_spacing(parts):
    H = build_hierarchy(gauss51_problem(), _opts(MaxLevels=2, TagFunction=lambda x, y: x ** 2 + y ** 2 < 0.01),
                        OracleBackend())
    with pytest.raises(ValueError, match='bsam_batch:spacing'):
        merge_flats([parts[0], flatten(H)])


@pytest.mark.gpu
@pytest.mark.parametrize('form', [None, '0', '2', '3', '5'])
def test_batch_equals_solo_bitwise(parts, form, monkeypatch):
    """form: the smoother's launch form forced on the batch (None: tuned; '0'
    one cluster launch per relaxation; '2' two colour cells per thread; '3'
    persistent blocks; '5' one cluster launch with the level's solution in
    distributed shared memory, where it fits), so frozen instances are
    skipped through the per-chunk flags in every form."""
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q, BSAM_FIELD_QC, BSAM_FIELD_F
    ctx = DeviceBackend.get(0).ctx
    Hs = _instances()
    opts = Hs[0].opts
    # different stop tests: one instance capped at 3 V-cycles, one at a looser tolerance
    stops = [(opts.MaxVCycles, opts.RelTol)] * len(parts)
    stops[1] = (3, opts.RelTol)
    stops[3] = (opts.MaxVCycles, 1e-6)
    solo = []
    for i, p in enumerate(parts):
        dh = DevHier(ctx, p, opts)
        dh.set_stop(0, *stops[i])
        it, hist, rel, vis = dh.solve_cycles(opts.MaxVCycles + 2)
        solo.append((it, hist, rel, vis, dh.get(BSAM_FIELD_Q, p.Q.size), dh.get(BSAM_FIELD_QC, p.QC.size),
                     dh.get(BSAM_FIELD_F, p.F.size)))
    b = merge_flats(parts)
    if form is not None:
        monkeypatch.setenv('BSAM_RELAX_N', form)
    bh = DevHier(ctx, b, opts)
    for i, s in enumerate(stops):
        bh.set_stop(i, *s)
    bh.solve_cycles(opts.MaxVCycles + 2)
    Q = bh.get(BSAM_FIELD_Q, b.Q.size)
    QC = bh.get(BSAM_FIELD_QC, b.QC.size)
    F = bh.get(BSAM_FIELD_F, b.F.size)
    its = []
    for i, s in enumerate(solo):
        it, hist, rel, vis = bh.batch_result(i, opts.MaxVCycles + 2)
        its.append(it)
        assert it == s[0], (i, it, s[0])
        np.testing.assert_array_equal(hist, s[1])
        assert rel == s[2] and vis == s[3]
        np.testing.assert_array_equal(split_field(b, FIELD_Q, Q, i), s[4])
        np.testing.assert_array_equal(split_field(b, FIELD_QC, QC, i), s[5])
        np.testing.assert_array_equal(split_field(b, FIELD_F, F, i), s[6])
    assert its[1] == 3 and len(set(its)) > 1
    # a second solve of the same batch starts from the solved state, as a
    # second ebSolveCycles call would
    it0, _, _, _ = bh.solve_cycles(opts.MaxVCycles + 2)
    assert it0 <= its[0]


@pytest.mark.gpu
def test_batch_of_one_equals_solo(parts):
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q
    ctx = DeviceBackend.get(0).ctx
    opts = _instances()[0].opts
    p = parts[0]
    a = DevHier(ctx, p, opts)
    ra = a.solve_cycles(opts.MaxVCycles + 2)
    b = merge_flats([p])
    bh = DevHier(ctx, b, opts)
    rb = bh.solve_cycles(opts.MaxVCycles + 2)
    assert ra[0] == rb[0]
    np.testing.assert_array_equal(ra[1], rb[1])
    np.testing.assert_array_equal(a.get(BSAM_FIELD_Q, p.Q.size), split_field(b, FIELD_Q, bh.get(BSAM_FIELD_Q, b.Q.size), 0))


@pytest.mark.gpu
def test_random_instances_batch_equals_solo():
    """Seeded instances of the batched-instances workload (uneven depths,
    roots 2-4, several patches per level): batch == solo bit for bit."""
    import warnings
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q
    from bsam.instances import random_elliptic, final_stage
    be = DeviceBackend.get(0)
    parts, opts = [], None
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        for s in range(1000, 1012):
            prob, o = random_elliptic(s)
            fl, H = final_stage(prob, o, be)
            parts.append(fl)
            opts = opts or H.opts
    assert len({p.nlev for p in parts}) > 1 and len({p.rootIdx for p in parts}) > 1
    solo = []
    for p in parts:
        dh = DevHier(be.ctx, p, opts)
        r = dh.solve_cycles(opts.MaxVCycles + 2)
        solo.append((r, dh.get(BSAM_FIELD_Q, p.Q.size)))
    b = merge_flats(parts)
    bh = DevHier(be.ctx, b, opts)
    bh.solve_cycles(opts.MaxVCycles + 2)
    Q = bh.get(BSAM_FIELD_Q, b.Q.size)
    for i, (r, q) in enumerate(solo):
        rb = bh.batch_result(i, opts.MaxVCycles + 2)
        assert rb[0] == r[0], (i, rb[0], r[0])
        np.testing.assert_array_equal(rb[1], r[1])
        np.testing.assert_array_equal(split_field(b, FIELD_Q, Q, i), q)
