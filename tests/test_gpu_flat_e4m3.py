"""Flat fast form with an E4M3 (FP8) shortlist (tcgen05 kind::f8f6f4, per-row
scales, FP32 accumulation) and the exact FP32 rerank of k * 4 rows: the
returned distances are the exact FP32 ones of the returned rows, and the
rerank wins the recall back against the exact scan."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _recall(gt, lab):
    return np.mean([len(set(a) & set(b)) / len(a) for a, b in zip(gt, lab)])


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d", [96, 128, 200])
def test_e4m3_shortlist_recall_and_exact_distances(mv, metric, d):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(30000, d=d, n_centers=64, seed=51, nq=200)
    ix = mv.IndexFlat(d, metric)
    ix.add(base)
    ed, el = ix.search(q, 10, plain_scan=True)  # exact FP32 scan
    fd, fl = ix.search(q, 10, form=mv.FORM_FAST, rerank=40, e4m3=True)
    assert _recall(el, fl) >= 0.95
    # every returned distance is the exact FP32 distance of its row: equal to
    # the exact scan's wherever the same row is returned at the same rank
    same = fl == el
    assert same.mean() > 0.9 and np.array_equal(fd[same], ed[same])
    # a deep shortlist returns the exact answer
    dd, dl = ix.search(q, 10, form=mv.FORM_FAST, rerank=400, e4m3=True)
    assert _recall(el, dl) >= 0.995


def test_e4m3_needs_rerank(mv):
    ix = mv.IndexFlat(32, 0)
    ix.add(np.random.default_rng(0).standard_normal((5000, 32)).astype(np.float32))
    with pytest.raises(mv.MojoVecGPUError):
        ix.search(np.zeros((2, 32), np.float32), 5, form=mv.FORM_FAST, e4m3=True)
