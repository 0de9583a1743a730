"""CPU tests of the host-side logic: synthetic workloads, recall, the
collection's argument validation (raised before any device work) and the
bench's aggregation helpers."""

import numpy as np
import pytest


def test_sift_like_is_integer_valued_and_seeded():
    from mojovec_gb300 import synth

    a, qa = synth.sift_like(2000, d=16, n_centers=8, nq=50, seed=1)
    b, qb = synth.sift_like(2000, d=16, n_centers=8, nq=50, seed=1)
    assert np.array_equal(a, b) and np.array_equal(qa, qb)
    assert a.dtype == np.float32 and (a == np.rint(a)).all()
    assert a.min() >= 0 and a.max() <= 255
    assert not np.array_equal(a[:50], qa)  # queries are fresh draws


def test_cos_mixture_rows_are_unit_norm():
    from mojovec_gb300 import synth

    x, q = synth.cos_mixture(1000, d=24, n_centers=16, nq=10)
    assert np.allclose(np.linalg.norm(x, axis=1), 1.0, atol=1e-5)
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-5)


def test_grid_vectors_match_reference_pattern():
    from mojovec_gb300 import synth

    g = synth.grid_vectors()
    assert g.shape == (256, 8)
    assert g[0, 0] == np.float32(0.0 / 251.0 + 2.0)
    assert g[3, 1] == np.float32(((3 * 17 + 29) % 251) / 251.0)


def test_recall_helper():
    import bench

    gt = np.array([[1, 2, 3], [4, 5, 6]])
    got = np.array([[3, 2, 9], [7, 8, 9]])
    assert bench.recall_at(gt, got, 3) == pytest.approx(2 / 6)


def test_aggregate_qps():
    import bench

    assert bench.aggregate_qps(4, 10000, 20, 1000.0) == pytest.approx(800000.0)


@pytest.mark.parametrize("kwargs,match", [
    (dict(dimension=0), "dimension"),
    (dict(dimension=10, pq_subvectors=3), "divide dimension"),
    (dict(dimension=8, pq_subvectors=2, nlist=0), "nlist"),
    (dict(dimension=8, nlist=4, pq_subvectors=2, nprobe=5), "nprobe"),
    (dict(dimension=8, pq_subvectors=2, metric="cos"), "metric"),
])
def test_collection_validation_before_device_work(kwargs, match):
    from mojovec_gb300 import IVFPQCollection

    with pytest.raises(ValueError, match=match):
        IVFPQCollection(**kwargs)


def test_search_result_arrays_checked():
    """Caller-provided result arrays (the reference's search writes into the
    caller's distances / labels spans): the exact shape, dtype and a
    writable C-contiguous layout, else ValueError; None allocates."""
    import numpy as np
    import pytest as _pytest
    from mojovec_gb300.index import _out

    a = _out(None, 3, 4, np.float32, "distances")
    assert a.shape == (3, 4) and a.dtype == np.float32
    mine = np.zeros((3, 4), np.int64)
    assert _out(mine, 3, 4, np.int64, "labels") is mine
    bad = [np.zeros((3, 5), np.int64), np.zeros((3, 4), np.int32),
           np.zeros((4, 3), np.int64).T, [[0] * 4] * 3]
    ro = np.zeros((3, 4), np.int64)
    ro.flags.writeable = False
    for b in bad + [ro]:
        with _pytest.raises(ValueError):
            _out(b, 3, 4, np.int64, "labels")
