"""Fast form of the flat scan: BF16 tcgen05 GEMM with the per-row heap
epilogue, segment merge, exact FP32 rerank.

On integer rows in [0, 255] with d <= 128 every BF16 product and FP32
partial sum is an exact integer, so the fast form must return exactly the
plain form's ids and distances (with and without rerank, including the
smaller-id tie rule). On real-valued rows the rerank restores recall and the
distances of the ids both forms return agree within 1e-5 relative.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(4242)


def _pair(mv, base, metric):
    ix = mv.IndexFlat(base.shape[1], metric)
    ix.add(base)
    return ix


def _assert_same(a, b):
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], b[0])


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("k,rerank", [(10, 40), (10, 0), (1, 4), (100, 400), (32, 128)])
def test_fast_equals_plain_on_integer_rows(mv, metric, k, rerank):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(20000, d=128, n_centers=50, nq=300, seed=11)
    ix = _pair(mv, base, metric)
    plain = ix.search(q, k)
    fast = ix.search(q, k, form=mv.FORM_FAST, rerank=rerank)
    _assert_same(fast, plain)


@pytest.mark.parametrize("d", [8, 96, 200, 256])
@pytest.mark.parametrize("nb,nq", [(1, 1), (129, 7), (5003, 130)])
def test_fast_equals_plain_shapes(mv, d, nb, nq):
    base = RNG.integers(0, 16, size=(nb, d)).astype(np.float32)
    q = RNG.integers(0, 16, size=(nq, d)).astype(np.float32)
    for metric in (0, 1):
        ix = _pair(mv, base, metric)
        _assert_same(ix.search(q, 10, form=mv.FORM_FAST, rerank=40), ix.search(q, 10))


def test_fast_filter_and_padding(mv):
    base = RNG.integers(0, 200, size=(3000, 64)).astype(np.float32)
    q = RNG.integers(0, 200, size=(50, 64)).astype(np.float32)
    ix = _pair(mv, base, 0)
    flt = (RNG.random(3000) < 0.3).astype(np.uint8)
    _assert_same(ix.search(q, 10, filter=flt, form=mv.FORM_FAST, rerank=40),
                 ix.search(q, 10, filter=flt))
    # more results asked than rows: 0.0 / -1 (index_flat.mojo:232-238)
    small = _pair(mv, base[:5], 0)
    d, l = small.search(q[:3], 8, form=mv.FORM_FAST, rerank=32)
    assert (l[:, 5:] == -1).all() and (d[:, 5:] == 0.0).all()
    _assert_same((d, l), small.search(q[:3], 8))


def test_fast_overflowing_segment_falls_back_exactly(mv):
    """1000 rows close to the query sit in one column segment, so a segment
    keeping 64 keys drops shortlist keys for k = 100: the query is detected
    and recomputed with the exact scan."""
    d = 64
    near = RNG.integers(0, 3, size=(1000, d)).astype(np.float32)
    far = RNG.integers(100, 200, size=(200000, d)).astype(np.float32)
    base = np.concatenate([near, far])
    q = np.zeros((4, d), np.float32)
    ix = _pair(mv, base, 0)
    _assert_same(ix.search(q, 100, form=mv.FORM_FAST, rerank=400), ix.search(q, 100))


def test_fast_real_valued_recall(mv):
    base = RNG.standard_normal((50000, 128)).astype(np.float32)
    q = RNG.standard_normal((500, 128)).astype(np.float32)
    for metric in (0, 1):
        ix = _pair(mv, base, metric)
        dp, lp = ix.search(q, 10)
        df, lf = ix.search(q, 10, form=mv.FORM_FAST, rerank=40)
        recall = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(lf, lp)])
        assert recall >= 0.99, (metric, recall)
        for i in range(len(q)):
            common = set(lf[i]) & set(lp[i])
            for c in common:
                a = df[i][list(lf[i]).index(c)]
                b = dp[i][list(lp[i]).index(c)]
                assert abs(a - b) <= 1e-5 * max(1.0, abs(b)), (metric, i, a, b)


def test_fast_is_deterministic(mv):
    base = RNG.standard_normal((30000, 96)).astype(np.float32)
    q = RNG.standard_normal((257, 96)).astype(np.float32)
    ix = _pair(mv, base, 0)
    a = ix.search(q, 10, form=mv.FORM_FAST, rerank=40)
    b = ix.search(q, 10, form=mv.FORM_FAST, rerank=40)
    _assert_same(a, b)
