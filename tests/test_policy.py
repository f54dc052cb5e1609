"""IndexBuilder::search's L policies (weavess_gb300.policy) against the
reference's loop, with a search that answers from a fixed accuracy table: the
widths visited and L_min."""
import numpy as np

from weavess_gb300 import policy as P


def fake_search(curve, gt):
    """A search whose accuracy at width L is curve(L): the first
    round(acc * K) result ids of every query are hits."""
    def fn(L):
        acc = curve(L)
        hits = int(round(acc * 10))
        res = np.full((gt.shape[0], 10), 10**6, np.uint32)
        res[:, :hits] = gt[:, :hits]
        res[:, hits:] = 10**6 + np.arange(10 - hits)
        return res, L * 7, L
    return fn


def test_accuracy_formula_counts_ground_rows_beyond_the_queries():
    gt = np.arange(40, dtype=np.uint32).reshape(4, 10)
    res = gt[:2].copy()
    res[0, 3] = 999
    # 1 miss over 4 ground-truth rows x 10
    assert P.reference_accuracy(res, gt) == np.float32(1) - np.float32(np.float32(1) / np.float32(40))


def test_set_recall_walk():
    gt = np.arange(1000, dtype=np.uint32).reshape(100, 10)
    # accuracy rises with L and reaches 0.99 (all 10 hits) from L = 70 on
    steps, L_min = P.set_recall(fake_search(lambda L: 1.0 if L >= 70 else min(0.9, L / 100), gt), gt)
    Ls = [s["L"] for s in steps]
    # the reference's walk: 10 -> +(1000 * (0.99 - 0.1)) = 900 (step 890) -> overshoot, then halve back
    assert Ls[0] == 10 and Ls[1] == 900
    assert L_min == min(L for L in Ls if L >= 70)
    assert all(s["dist_count"] == s["L"] * 7 for s in steps)
    # every width is visited once
    assert len(set(Ls)) == len(Ls)


def test_ascend_widths():
    gt = np.arange(100, dtype=np.uint32).reshape(10, 10)
    steps = P.ascend(fake_search(lambda L: 0.5, gt), gt)
    assert [s["L"] for s in steps] == [13, 21, 34, 55, 89, 144, 233, 377, 610, 987]


def test_assign_rejects_small_width():
    import pytest
    gt = np.zeros((2, 10), np.uint32)
    with pytest.raises(ValueError):
        P.assign(fake_search(lambda L: 1.0, gt), 5, gt)
