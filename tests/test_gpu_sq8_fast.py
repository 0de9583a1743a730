"""SQ8 scan on the tensor cores (mv_sq8_search_ex, form FAST).

SQ8 codes are small integers, exact in BF16, and below the stated
dimensions every dot product is an exact FP32 integer, so the fast form must
return exactly the integer scan's ids and distances (index_flat_sq8.mojo
semantics, smaller id first on equal distances), with and without the FP32
rerank, with filters and with more results than rows. Rows drawn from a
handful of values make many equal distances and exercise the per-query
rescan that guards ties at the shortlist boundary.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(8080)


def _idx(mv, base, metric):
    ix = mv.IndexFlatSQ8(base.shape[1], metric)
    ix.add(base)
    return ix


def _same(a, b):
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], b[0])


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("k,factor", [(10, 0), (10, 2), (1, 0), (100, 2), (40, 0)])
def test_sq8_fast_equals_plain_sift_like(mv, metric, k, factor):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(30000, d=128, n_centers=60, nq=200, seed=21)
    ix = _idx(mv, base, metric)
    _same(ix.search(q, k, form=mv.FORM_FAST, rerank_factor=factor),
          ix.search(q, k, form=mv.FORM_PLAIN, rerank_factor=factor))


@pytest.mark.parametrize("d", [16, 96, 200, 256])
def test_sq8_fast_equals_plain_real_valued(mv, d):
    base = RNG.standard_normal((8000, d)).astype(np.float32)
    q = RNG.standard_normal((130, d)).astype(np.float32)
    for metric in (0, 1):  # L2 above d = 129 takes the integer scan
        ix = _idx(mv, base, metric)
        for factor in (0, 2):
            _same(ix.search(q, 10, form=mv.FORM_FAST, rerank_factor=factor),
                  ix.search(q, 10, form=mv.FORM_PLAIN, rerank_factor=factor))


def test_sq8_fast_ties_filter_and_padding(mv):
    base = RNG.integers(0, 3, size=(20000, 32)).astype(np.float32)  # many equal distances
    q = RNG.integers(0, 3, size=(64, 32)).astype(np.float32)
    for metric in (0, 1):
        ix = _idx(mv, base, metric)
        _same(ix.search(q, 10, form=mv.FORM_FAST), ix.search(q, 10, form=mv.FORM_PLAIN))
        flt = (RNG.random(20000) < 0.5).astype(np.uint8)
        _same(ix.search(q, 10, filter=flt, form=mv.FORM_FAST),
              ix.search(q, 10, filter=flt, form=mv.FORM_PLAIN))
    small = _idx(mv, base[:7], 0)
    d, l = small.search(q[:5], 12, form=mv.FORM_FAST)
    assert (l[:, 7:] == -1).all() and (d[:, 7:] == 0.0).all()
    _same((d, l), small.search(q[:5], 12, form=mv.FORM_PLAIN))
