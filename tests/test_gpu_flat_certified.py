"""Plain Flat search through the certified tensor-core path (k_flat_certify):
the BF16 shortlist, the reference FP32 distances of its rows and the error
bound must give exactly the reference's top-k (index/index_flat.mojo:
260-325, canonical (distance, id) order) whatever the data. Checked
bit-exactly against the oracle on integer SIFT-like rows (BF16-exact),
real-valued rows, both metrics, k from 1 to 100 (the last one with the
segment-overflow path), a filter mask, and rows with many exact ties at the
k-boundary, which only the exact scan can settle."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all(a == b))


def _stats(mv):
    st = mv.Context.default().certify_stats()
    return st["flat_queries"], st["flat_fallback"]


def _check(mv, orc, base, q, k, metric, filt=None):
    ix = mv.IndexFlat(base.shape[1], metric)
    ix.add(base)
    q0, f0 = _stats(mv)
    gd, gl = ix.search(q, k, filter=filt)
    q1, f1 = _stats(mv)
    rd, rl = orc.flat_search(base, q, k, metric=metric, filter=filt)
    assert np.array_equal(gl, rl)
    assert _same(gd, rd)
    return q1 - q0, f1 - f0


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("k", [1, 10, 100])
def test_sift_like_exact_and_settled(mv, orc, metric, k):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(30000, d=128, n_centers=64, seed=41, nq=200)
    n, fb = _check(mv, orc, base, q, k, metric)
    assert n == len(q)
    if metric == 0:
        assert fb <= 0.05 * len(q), fb  # integer rows are exact in BF16: the bound is tight


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d", [32, 96, 200])
def test_real_valued_exact(mv, orc, metric, d):
    from mojovec_gb300 import synth

    base, q = synth.cos_mixture(20000, d=d, n_centers=256, seed=42, nq=150)
    n, _ = _check(mv, orc, base, q, 10, metric)
    assert n == len(q)


def test_filter_exact(mv, orc):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(20000, d=64, n_centers=32, seed=43, nq=100)
    filt = (np.random.default_rng(44).random(len(base)) < 0.4).astype(np.uint8)
    _check(mv, orc, base, q, 10, 0, filt)


def test_ties_fall_back_and_stay_exact(mv, orc):
    rng = np.random.default_rng(45)
    base = rng.integers(0, 4, size=(20000, 16)).astype(np.float32)
    base[:3000] = base[0]  # 3000 equal rows: ties far past any shortlist
    q = np.vstack([base[:20] + rng.integers(0, 2, size=(20, 16)),
                   rng.integers(0, 4, size=(40, 16))]).astype(np.float32)
    n, fb = _check(mv, orc, base, q, 10, 0)
    assert n == len(q) and fb > 0
