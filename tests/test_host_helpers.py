"""Host set-up helpers (CPU): the vectorised box filter that replaces the
all-pairs patch-box loops returns every box an inclusive rectangle test can
hit, in order; the memoised coarsest inverse returns the very same bits as a
fresh inverse."""
import threading

import numpy as np
import pytest

from bsam.hierarchy import near_boxes, rect_isect, dense_inverse


def test_near_boxes_superset_in_order():
    rng = np.random.default_rng(5)
    boxes = []
    for _ in range(300):
        i0, j0 = rng.integers(1, 200, 2)
        boxes.append([i0, i0 + rng.integers(0, 20), j0, j0 + rng.integers(0, 20)])
    boxes = np.array(boxes, dtype=np.int64)
    for _ in range(200):
        i0, j0 = rng.integers(1, 200, 2)
        r = [int(i0), int(i0 + rng.integers(0, 30)), int(j0), int(j0 + rng.integers(0, 30))]
        cand = near_boxes(boxes, r)
        assert cand == sorted(cand)
        # the cell test and both face tests of the coefficient and window loops
        for q in range(len(boxes)):
            qb = [int(v) for v in boxes[q]]
            hits = (rect_isect(r, qb) is not None or
                    rect_isect([r[0], r[1] + 1, r[2], r[3]], [qb[0], qb[1] + 1, qb[2], qb[3]]) is not None or
                    rect_isect([r[0], r[1], r[2], r[3] + 1], [qb[0], qb[1], qb[2], qb[3] + 1]) is not None)
            if hits:
                assert q in cand
        exact = near_boxes(boxes, r, pad=0)
        assert exact == [q for q in range(len(boxes)) if rect_isect(r, [int(v) for v in boxes[q]]) is not None]


def test_dense_inverse_memo_is_bitwise_and_threadsafe():
    rng = np.random.default_rng(1)
    mats = [np.eye(40) * 4 + rng.standard_normal((40, 40)) * 0.1 for _ in range(3)]
    fresh = [np.linalg.inv(a) for a in mats]
    out = {}

    def work(t):
        out[t] = [dense_inverse(mats[(t + i) % 3]) for i in range(12)]

    th = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    for t, res in out.items():
        for i, r in enumerate(res):
            np.testing.assert_array_equal(r, fresh[(t + i) % 3])
    # a returned inverse is a copy: changing it leaves the cache intact
    a = dense_inverse(mats[0])
    a[0, 0] = 1e9
    np.testing.assert_array_equal(dense_inverse(mats[0]), fresh[0])


def test_deepcopy_of_a_hierarchy_leaves_its_device_copy_behind():
    """A deep copy must not duplicate the resident device handle (both copies
    would free it); it drops it and re-uploads when next solved."""
    import copy
    from bsam import ebOptions, ebProblem, hierarchy as hier
    from bsam.device import DevHier, Context
    from bsam_oracle import OracleBackend
    H = hier.setup(ebProblem([0, 1, 0, 1], 1, 1, 1, ('dirichlet', 0)), ebOptions('BaseCells', 16, 'Verbose', 0),
                   OracleBackend())
    class NoDevHier(DevHier):                  # stands in for an uploaded copy: no handle, no device
        def __del__(self):
            pass

    class NoContext(Context):
        def __del__(self):
            pass

    fake = NoDevHier.__new__(NoDevHier)
    H._dev = (H.version, fake)
    H.host_stale = True
    G = copy.deepcopy(H)
    assert G._dev is None and H._dev[1] is fake
    assert G.host_stale is True                # using the copy still requires a host sync of the original
    np.testing.assert_array_equal(G.lev[1].Q[0], H.lev[1].Q[0])
    assert G.lev[1].Q[0] is not H.lev[1].Q[0]
    with pytest.raises(TypeError, match='bsam_device:copy'):
        copy.deepcopy(fake)
    ctx = NoContext.__new__(NoContext)
    with pytest.raises(TypeError, match='bsam_device:copy'):
        copy.copy(ctx)


@pytest.mark.parametrize('tree', [False, True])
def test_error_norms_without_exact_solution(tree):
    """ebErrorNorms.m:14-16 / ebtErrorNorms: no exact solution is an error."""
    from bsam import ebOptions, ebProblem, hierarchy as hier
    from bsam.solve import error_norms
    from bsam_oracle import OracleBackend
    H = hier.setup(ebProblem([0, 1, 0, 1], 1, 1, 1, ('dirichlet', 0)), ebOptions('BaseCells', 16, 'Verbose', 0),
                   OracleBackend(), tree=tree)
    with pytest.raises(ValueError, match=('ebt' if tree else 'eb') + '_error_norms:noexact'):
        error_norms(H)
    assert error_norms(H, lambda x, y: 0 * x)['linf'] == 0.0


@pytest.mark.parametrize('tree', [False, True])
def test_error_identifiers_follow_the_hierarchy_form(tree):
    """The tree copies raise ``ebt_*`` identifiers (ebtProblem.m, ebtOptions.m,
    ebtMakeLevel.m, ebtTagCluster.m), the QC-ring code ``eb_*``."""
    from bsam import ebOptions, ebtOptions, ebProblem, ebtProblem, ebSolve, ebtSolve, hierarchy as hier
    from bsam.tagcluster import tag_cluster
    from bsam_oracle import OracleBackend
    pre = 'ebt_' if tree else 'eb_'
    mkprob, mkopts, solve = (ebtProblem, ebtOptions, ebtSolve) if tree else (ebProblem, ebOptions, ebSolve)
    with pytest.raises(ValueError, match=pre + 'problem:domain'):
        mkprob([1, 0, 0, 1], 1, 1, 1, ('dirichlet', 0))
    with pytest.raises(ValueError, match=pre + 'options:ghost'):
        mkopts('GhostInterp', 'cubic')
    prob = mkprob([0, 1, 0, 1], 1, 1, 1, ('dirichlet', 0))
    with pytest.raises(ValueError, match=pre + 'options:ghost'):
        solve(prob, 'GhostInterp', 'cubic', 'Verbose', 0, backend=OracleBackend())
    with pytest.raises(ValueError, match=pre + 'make_level:D'):
        hier.setup(mkprob([0, 1, 0, 1], lambda x, y: 0 * x, 1, 1, ('dirichlet', 0)),
                   mkopts('BaseCells', 16, 'Verbose', 0), OracleBackend(), tree=tree)
    with pytest.raises(ValueError, match=pre + 'make_level:eval'):
        hier.setup(mkprob([0, 1, 0, 1], 1, lambda x, y: x[:1], 1, ('dirichlet', 0)),
                   mkopts('BaseCells', 16, 'Verbose', 0), OracleBackend(), tree=tree)
    H = hier.setup(prob, mkopts('BaseCells', 16, 'MaxLevels', 2, 'Indicator', 'fun', 'Verbose', 0), OracleBackend(),
                   tree=tree)
    with pytest.raises(ValueError, match=pre + 'tag_cluster:tagfun'):
        tag_cluster(H, OracleBackend())
    H.opts.Indicator = 'gradient'
    with pytest.raises(ValueError, match=pre + 'tag_cluster:ind'):
        tag_cluster(H, OracleBackend())
