"""The staged fast IVF-PQ scan (k_ivfpq_scan_staged, lut = 4).

It copies each round's list pieces (codes and per-vector terms) into shared
memory with bulk copies and selects the shortlist with a histogram select;
its distances use the same FP32 table arithmetic as the unstaged kernel
(lut = 2), so the two must return identical ids and distance bits: with the
shortlist as the answer (rerank 0, sorted) and after the exact rerank.
Covered: rounds that split one long list, dozens of consecutive empty lists
between probes, more probes than a round's 32 pieces, filters, both metrics,
M = 8 / 12 / 16 / 24 / 64 (each code-load width), k up to 2048 (staging
overflows and intermediate selects), ties (duplicated rows), and the
persistent batched scan.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(np.asarray(a[0]).view(np.uint32), np.asarray(b[0]).view(np.uint32))


def _clustered(n, d, nclusters, seed, spread=1.0, nq=60):
    rng = np.random.default_rng(seed)
    cent = rng.standard_normal((nclusters, d)).astype(np.float32) * 4
    lab = rng.integers(0, nclusters, n)
    base = (cent[lab] + spread * rng.standard_normal((n, d))).astype(np.float32)
    q = (cent[rng.integers(0, nclusters, nq)] + spread * rng.standard_normal((nq, d))).astype(np.float32)
    return base, q


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", [(64, 8), (96, 12), (128, 16), (96, 24), (128, 64)])
def test_staged_equals_unstaged(mv, d, M, metric):
    base, q = _clustered(12000, d, 40, seed=M + metric)
    g = mv.IndexIVFPQ(d, 64, M, metric)
    g.train(base[:8000], niter_coarse=4, niter_pq=4)
    g.add(base)
    for nprobe, k, rerank in ((4, 10, 0), (16, 100, 0), (8, 10, 64), (40, 2048, 0)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=4)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=2)
        _same(a, b)


def test_staged_long_lists_and_empty_lists(mv):
    """Centroids chosen so that queries probe 40 empty lists before the three
    filled ones (a run of more than a round's 32 pieces), and each filled
    list holds about 10,000 rows (one list spans several rounds)."""
    rng = np.random.default_rng(3)
    d, M = 32, 8
    centers = rng.standard_normal((3, d)).astype(np.float32) * 10
    base = (centers[rng.integers(0, 3, 30000)] + 0.3 * rng.standard_normal((30000, d))).astype(np.float32)
    qc = np.full(d, 6.0, np.float32)  # the queries' region holds no rows
    q = (qc + 0.3 * rng.standard_normal((40, d))).astype(np.float32)
    near = qc + 0.5 * rng.standard_normal((40, d)).astype(np.float32)
    far = 200.0 + rng.standard_normal((213, d)).astype(np.float32)
    cent = np.vstack([near, centers, far]).astype(np.float32)
    t = mv.IndexIVFPQ(d, 3, M)
    t.train(base[:20000], niter_coarse=3, niter_pq=3)
    _, pq = t.codebooks()
    g = mv.IndexIVFPQ(d, 256, M)
    g.set_codebooks(cent, pq)
    g.add(base)
    sizes = np.diff(g.lists()[0])
    assert (sizes[:40] == 0).all() and sizes[40:43].min() > 5000
    for nprobe, k, rerank in ((45, 10, 0), (45, 300, 0), (43, 50, 256), (256, 2048, 0)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=4)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=2)
        _same(a, b)
        assert (a[1][:, 0] >= 0).all()  # the filled lists were reached


def test_staged_filter_and_ties(mv):
    rng = np.random.default_rng(5)
    base, q = _clustered(15000, 64, 30, seed=6)
    base[5000:5400] = base[5000]  # 400 equal rows: equal distances at the boundary
    q[:10] = base[5000]
    g = mv.IndexIVFPQ(64, 64, 16)
    g.train(base[:10000], niter_coarse=4, niter_pq=4)
    g.add(base)
    flt = (rng.random(len(base)) < 0.3).astype(np.uint8)
    for k, rerank in ((10, 0), (300, 0), (10, 128)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=12, rerank=rerank, filter=flt, lut=4)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=12, rerank=rerank, filter=flt, lut=2)
        _same(a, b)
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=12, rerank=rerank, lut=4)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=12, rerank=rerank, lut=2)
        _same(a, b)


def test_staged_batch_plan_equals_direct(mv):
    """The persistent batched scan (plan, tuner, graph) keeps every query's
    results equal to its own direct search."""
    base, q = _clustered(20000, 64, 50, seed=9, nq=300)
    g = mv.IndexIVFPQ(64, 128, 16)
    g.train(base[:10000], niter_coarse=4, niter_pq=4)
    g.add(base)
    rng = np.random.default_rng(10)
    nprobe = rng.integers(1, 60, size=len(q)).astype(np.int32)
    k = rng.choice(np.array([1, 10, 100], np.int32), size=len(q))
    plan = mv.IVFPQBatchPlan(g, len(q), 64, 100, rerank=128, lut=4)
    plan.set_queries(q, nprobe, k)
    plan.tune(len(q))
    plan.run(len(q), use_graph=True)
    d, l = plan.results(len(q))
    for i in range(0, len(q), 7):
        dd, ll = g.search(q[i:i + 1], int(k[i]), form=mv.FORM_FAST, nprobe=int(nprobe[i]), rerank=128,
                          lut=4)
        assert np.array_equal(ll[0], l[i, :k[i]]) and np.array_equal(dd[0], d[i, :k[i]]), i
