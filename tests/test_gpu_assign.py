"""Certified nearest-centroid assignment (k_assign.cu): the BF16 tensor-core
candidates, their reference FP32 distances and the error bound must give
exactly the reference's assignment (index/index_flat.mojo:292-310 with k = 1;
clustering/kmeans.mojo:123-141), whatever the data. Checked bit-exactly
against the oracle on clustered data, on unclustered Gaussian data (small
margins between the nearest centroids), and against numpy on integer data with
duplicated centroids, where ties only the exact scan can settle sit outside
the 16 candidates."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stats(mv):
    return mv.Context.default().assign_stats()


def test_plain_kmeans_certified_matches_oracle(mv, orc):
    from mojovec_gb300 import synth

    x, _ = synth.sift_like(20000, d=32, n_centers=60, seed=21)
    r0, _ = _stats(mv)
    km = mv.KMeans(32, 100, 4)
    km.train(x)
    rows, _ = _stats(mv)
    assert rows - r0 >= 4 * 20000  # every iteration went through the certified path
    rc, ra = orc.kmeans_train(x, 100, niter=4)
    assert np.array_equal(km.centroids.view(np.uint32), rc.view(np.uint32))
    assert np.array_equal(km.assignments, ra)


@pytest.mark.parametrize("metric", [0, 1])
def test_ivfpq_train_add_certified_matches_oracle(mv, orc, metric):
    from mojovec_gb300 import synth

    d, nlist, M = 64, 256, 8
    x, _ = synth.sift_like(20000, d=d, n_centers=80, seed=22)
    if metric == 1:
        x = x / np.linalg.norm(x, axis=1, keepdims=True)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(x, niter_coarse=4, niter_pq=4)
    r = orc.IVFPQ(d, nlist, M, metric)
    r.train(x, niter_coarse=4, niter_pq=4)
    gc, gp = g.codebooks()
    rc, rp = r.codebooks()
    assert np.array_equal(gc.view(np.uint32), rc.view(np.uint32))
    assert np.array_equal(gp.view(np.uint32), rp.view(np.uint32))
    g.add(x)
    r.add(x)
    for a, b in zip(g.lists(), r.lists()):
        assert np.array_equal(a, b)


def test_unclustered_rows_stay_exact(mv, orc):
    d, nlist, M = 128, 2048, 16
    rng = np.random.default_rng(23)
    cent = rng.standard_normal((nlist, d)).astype(np.float32)
    pq = rng.standard_normal((M, 256, d // M)).astype(np.float32)
    x = rng.standard_normal((20000, d)).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M)
    g.set_codebooks(cent, pq)
    r = orc.IVFPQ(d, nlist, M)
    r.set_codebooks(cent, pq)
    r0, f0 = _stats(mv)
    g.add(x)
    rows, fb = _stats(mv)
    assert rows - r0 == 20000
    r.add(x)
    for a, b in zip(g.lists(), r.lists()):
        assert np.array_equal(a, b)


def test_duplicated_centroids_ties_settled_exactly(mv):
    d, nlist, M = 8, 64, 2
    rng = np.random.default_rng(24)
    cent = rng.integers(0, 8, size=(nlist, d)).astype(np.float32)
    cent[:40] = cent[0]  # 40 equal centroids: the smallest index must win
    pq = rng.standard_normal((M, 256, d // M)).astype(np.float32)
    x = rng.integers(0, 8, size=(8192, d)).astype(np.float32)
    x[:4096] = cent[0] + rng.integers(-1, 2, size=(4096, d))
    g = mv.IndexIVFPQ(d, nlist, M)
    g.set_codebooks(cent, pq)
    r0, f0 = _stats(mv)
    g.add(x)
    rows, fb = _stats(mv)
    assert rows - r0 == len(x) and fb - f0 > 0
    off, ids, _ = g.lists()
    where = np.empty(len(x), np.int64)
    where[ids] = np.repeat(np.arange(nlist), np.diff(off))
    x64, c64 = x.astype(np.float64), cent.astype(np.float64)
    dist = (x64 * x64).sum(1)[:, None] + (c64 * c64).sum(1)[None, :] - 2 * x64 @ c64.T
    assert np.array_equal(where, dist.argmin(1))
    assert (np.diff(off)[1:40] == 0).all()


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("nprobe", [1, 8, 32])
def test_plain_ivfpq_certified_coarse_matches_oracle(mv, orc, metric, nprobe):
    """The plain search's coarse step (k = nprobe, index_ivf_pq.mojo:264)
    through the certified path: probes, hence ids and distance bits, equal
    the oracle's."""
    from mojovec_gb300 import synth

    d, nlist, M = 64, 1024, 8
    x, q = synth.sift_like(30000, d=d, n_centers=100, seed=61, nq=300)
    if metric == 1:
        x = x / np.linalg.norm(x, axis=1, keepdims=True)
        q = q / np.linalg.norm(q, axis=1, keepdims=True)
    rng = np.random.default_rng(62)
    cent = x[rng.choice(len(x), nlist, replace=False)] + rng.standard_normal((nlist, d)).astype(np.float32) * 0.01
    pq = rng.standard_normal((M, 256, d // M)).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.set_codebooks(cent, pq)
    g.add(x)
    r = orc.IVFPQ(d, nlist, M, metric)
    r.set_codebooks(cent, pq)
    r.add(x)
    r0, _ = _stats(mv)
    gd, gl = g.search(q, 10, nprobe=nprobe)
    rows, _ = _stats(mv)
    assert rows - r0 == len(q)  # the coarse step went through the certified path
    rd, rl = r.search(q, 10, nprobe)
    assert np.array_equal(gl, rl) and np.array_equal(gd.view(np.uint32), rd.view(np.uint32))


def test_plain_coarse_ties_fall_back(mv, orc):
    d, nlist, M = 16, 256, 4
    rng = np.random.default_rng(63)
    cent = rng.integers(0, 4, size=(nlist, d)).astype(np.float32)
    cent[:120] = cent[0]  # 120 equal centroids: ties far past the candidates
    pq = rng.standard_normal((M, 256, d // M)).astype(np.float32)
    x = rng.integers(0, 4, size=(20000, d)).astype(np.float32)
    q = np.vstack([cent[:50] + rng.integers(0, 2, size=(50, d)),
                   rng.integers(0, 4, size=(50, d))]).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M)
    g.set_codebooks(cent, pq)
    g.add(x)
    r = orc.IVFPQ(d, nlist, M)
    r.set_codebooks(cent, pq)
    r.add(x)
    _, f0 = _stats(mv)
    gd, gl = g.search(q, 10, nprobe=8)
    _, f1 = _stats(mv)
    rd, rl = r.search(q, 10, 8)
    assert f1 > f0
    assert np.array_equal(gl, rl) and np.array_equal(gd.view(np.uint32), rd.view(np.uint32))


@pytest.mark.parametrize("metric", [0, 1])
def test_plain_ivfflat_certified_coarse_matches_oracle(mv, orc, metric):
    from mojovec_gb300 import synth

    d, nlist = 32, 512
    x, q = synth.sift_like(20000, d=d, n_centers=64, seed=64, nq=200)
    g = mv.IndexIVFFlat(d, nlist, metric)
    g.train(x, niter=4)
    g.add(x)
    r = orc.IVFFlat(d, nlist, metric)
    r.train(x, niter=4)
    r.add(x)
    for nprobe in (4, 16):
        gd, gl = g.search(q, 10, nprobe=nprobe)
        rd, rl = r.search(q, 10, nprobe)
        assert np.array_equal(gl, rl) and np.array_equal(gd.view(np.uint32), rd.view(np.uint32))
