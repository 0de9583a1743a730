"""Fast k-means (mv_kmeans_train_ex, form FAST): tensor-core candidates with
an exact FP32 recheck for the assignment, FP64 sums in a fixed order for the
update. Checked against the plain (reference-exact) form: the objective
(sum of squared distances) per iteration and at the end agrees within the
stated tolerance, the run is deterministic, the reported objective is the
inertia of the returned centroids, and degenerate data (more clusters than
distinct rows, d <= 4) goes through the empty-cluster rule.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3  # objective, fast against plain, on these small cases


def _inertia(x, c):
    x64, c64 = x.astype(np.float64), c.astype(np.float64)
    best = np.full(len(x), np.inf)
    for c0 in range(0, len(c), 1024):
        cc = c64[c0:c0 + 1024]
        d2 = (x64 * x64).sum(1)[:, None] + (cc * cc).sum(1)[None, :] - 2 * x64 @ cc.T
        best = np.minimum(best, d2.min(1))
    return float(np.maximum(best, 0).sum())


def _train(mv, x, k, niter, form):
    km = mv.KMeans(x.shape[1], k, niter=niter, form=form)
    km.train(x)
    return km


@pytest.mark.parametrize("d,k", [(96, 256), (128, 1000), (32, 64)])
def test_fast_objective_matches_plain(mv, d, k):
    from mojovec_gb300 import synth

    x, _ = synth.cos_mixture(40000, d=d, n_centers=512, seed=5)
    plain = _train(mv, x, k, 10, mv.FORM_PLAIN)
    fast = _train(mv, x, k, 10, mv.FORM_FAST)
    rel = np.abs(fast.objective - plain.objective) / plain.objective
    assert rel.max() < REL_TOL, rel
    # the reported final objective is the inertia of the returned centroids
    assert abs(fast.objective[-1] - _inertia(x, fast.centroids)) <= 1e-5 * fast.objective[-1]
    assert abs(plain.objective[-1] - _inertia(x, plain.centroids)) <= 1e-5 * plain.objective[-1]


def test_fast_is_deterministic(mv):
    from mojovec_gb300 import synth

    x, _ = synth.sift_like(30000, d=64, n_centers=100, seed=9)
    a = _train(mv, x, 200, 6, mv.FORM_FAST)
    b = _train(mv, x, 200, 6, mv.FORM_FAST)
    assert np.array_equal(a.centroids, b.centroids)
    assert np.array_equal(a.assignments, b.assignments)
    assert np.array_equal(a.objective, b.objective)


def test_fast_first_step_assignments_equal_plain(mv):
    """Both forms start from the same rows, so the first assignment step sees
    the same centroids: on integer data, where every BF16 distance is exact,
    the fast assignment must equal the exact one."""
    from mojovec_gb300 import synth

    x, _ = synth.sift_like(20000, d=64, n_centers=80, seed=4)
    plain = _train(mv, x, 128, 1, mv.FORM_PLAIN)
    fast = _train(mv, x, 128, 1, mv.FORM_FAST)
    assert np.array_equal(fast.assignments, plain.assignments)
    assert fast.objective[0] == plain.objective[0]


@pytest.mark.parametrize("d", [2, 4, 8])
def test_fast_degenerate_and_small_dims(mv, d):
    rng = np.random.default_rng(3)
    x = rng.integers(0, 3, size=(5000, d)).astype(np.float32)  # few distinct rows
    for form in (mv.FORM_PLAIN, mv.FORM_FAST):
        km = _train(mv, x, 100, 4, form)
        assert np.isfinite(km.centroids).all()
        assert km.assignments.min() >= 0 and km.assignments.max() < 100
    a = _train(mv, x, 100, 4, mv.FORM_FAST)
    b = _train(mv, x, 100, 4, mv.FORM_FAST)
    assert np.array_equal(a.centroids, b.centroids)
