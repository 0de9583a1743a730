"""The list-major tensor-core ADC scan (k_tc_scan + k_tc_select, lut = 5).

Its distances come from FP16 queries times FP16 reconstructions of the list
rows on the tensor cores, so they differ from the FP32-table scans in the
last bits. They are checked against an FP64 evaluation of the fast form's
distance (coarse term + ||y||^2 + 2<c, y> - 2<q, y>, or -<q, c> - <q, y>)
within the bound of two FP16 roundings per product, and the selection is
checked to be exact: with the shortlist as the answer (rerank 0, sorted),
the k smallest of any k are a prefix of the 2048 smallest. Once every
candidate is reranked the results must equal the exact Flat search. Covered:
both metrics, d / M = 8 and 4 (d 32, 64, 96, 128), lists longer than one
work item (1024 rows), more queries per list than one MMA tile holds (128),
filters, ties, per-query nprobe in the batched plan.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clustered(n, d, nclusters, seed, spread=1.0, nq=60):
    rng = np.random.default_rng(seed)
    cent = rng.standard_normal((nclusters, d)).astype(np.float32) * 4
    lab = rng.integers(0, nclusters, n)
    base = (cent[lab] + spread * rng.standard_normal((n, d))).astype(np.float32)
    q = (cent[rng.integers(0, nclusters, nq)] + spread * rng.standard_normal((nq, d))).astype(np.float32)
    return base, q


def _index(mv, base, d, nlist, M, metric=0, ntrain=20000):
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base[: min(len(base), ntrain)], niter_coarse=5, niter_pq=5)
    g.add(base)
    return g


def _check_distances(g, q, dist, lab, metric):
    """Every returned (query, id) distance against FP64 within the FP16 bound."""
    cent, pq = g.codebooks()
    off, ids, codes = g.lists()
    M, dsub = pq.shape[0], pq.shape[2]
    pos_of = np.full(int(ids.max()) + 1, -1, np.int64)
    pos_of[ids] = np.arange(len(ids))
    list_of = np.repeat(np.arange(len(off) - 1), np.diff(off))
    q64 = q.astype(np.float64)
    pq64 = pq.astype(np.float64)
    checked = 0
    for i in range(len(q)):
        ok = lab[i] >= 0
        if not ok.any():
            continue
        pos = pos_of[lab[i][ok]]
        L = list_of[pos]
        y = pq64[np.arange(M)[None, :], codes[pos].astype(np.int64)].reshape(len(pos), M * dsub)
        c = cent.astype(np.float64)[L]
        qy = y @ q64[i]
        s = np.abs(y) @ np.abs(q64[i])
        if metric == 0:
            term = ((q64[i] - c) ** 2).sum(1)
            vterm = (y * y).sum(1) + 2 * (c * y).sum(1)
            ref = term + vterm - 2 * qy
            tol = 2.0 ** -8 * 2 * s + 1e-5 * (np.abs(term) + np.abs(vterm) + np.abs(ref)) + 1e-3
        else:
            term = -(c @ q64[i])
            ref = term - qy
            tol = 2.0 ** -8 * s + 1e-5 * (np.abs(term) + np.abs(ref)) + 1e-3
        got = dist[i][ok].astype(np.float64)
        if metric == 1:
            got = -got  # the search returns IP scores un-negated
        bad = np.abs(got - ref) > tol
        assert not bad.any(), (i, got[bad][:4], ref[bad][:4], tol[bad][:4])
        checked += ok.sum()
    assert checked > 0


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", [(64, 8), (96, 24), (32, 8), (128, 16)])
def test_tc_exhaustive_equals_flat(mv, d, M, metric):
    rng = np.random.default_rng(d + M + metric)
    base = rng.standard_normal((3000, d)).astype(np.float32)
    q = rng.standard_normal((40, d)).astype(np.float32)
    g = _index(mv, base, d, 16, M, metric)
    a = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=3000, lut=5)
    b = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=3000, lut=0)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    flat = mv.IndexFlat(d, metric)
    flat.add(base)
    fd, fl = flat.search(q, 10)
    assert np.array_equal(a[1], fl)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", [(128, 16), (96, 24), (64, 16)])
def test_tc_distances_within_fp16_bound(mv, d, M, metric):
    base, q = _clustered(20000, d, 40, seed=d + metric, nq=50)
    g = _index(mv, base, d, 64, M, metric)
    dist, lab = g.search(q, 200, form=mv.FORM_FAST, nprobe=8, rerank=0, lut=5)
    assert (lab[:, :100] >= 0).all()
    key = dist if metric == 0 else -dist
    assert (np.diff(key, axis=1)[lab[:, 1:] >= 0] >= 0).all()  # sorted ascending
    _check_distances(g, q, dist, lab, metric)


@pytest.mark.parametrize("nprobe", [3, 12])
def test_tc_select_is_exact(mv, nprobe):
    """The k smallest keys for k = 10 ... 700 are the first k of the 2048
    smallest (complete candidate lists at nprobe 3, the histogram passes at
    nprobe 12)."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(24000, d=32, n_centers=64, nq=150, seed=23)
    g = _index(mv, base, 32, 64, 8)
    fd, fl = g.search(q, 2048, form=mv.FORM_FAST, nprobe=nprobe, lut=5)
    if nprobe == 3:
        assert np.mean((fl == -1).any(axis=1)) > 0.5
    for k in (10, 100, 256, 700):
        d, l = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, lut=5)
        assert np.array_equal(l, fl[:, :k]), k
        assert np.array_equal(d.view(np.uint32), fd[:, :k].view(np.uint32)), k


def test_tc_long_lists_and_crowded_lists(mv):
    """Four far-apart clusters of 1300 / 400 / 250 / 48 rows, one list each:
    the first list spans two 1024-row work items, and 300 queries probe
    every list (three query chunks of up to 128). With k = all 1998 rows,
    every row comes back once with its distance within the FP16 bound; the
    1000 smallest are the prefix of that list."""
    rng = np.random.default_rng(31)
    d, M = 64, 16
    centers = rng.standard_normal((4, d)).astype(np.float32) * 30
    sizes = [1300, 400, 250, 48]
    base = np.vstack([centers[i] + rng.standard_normal((s, d)).astype(np.float32)
                      for i, s in enumerate(sizes)]).astype(np.float32)
    q = (centers[rng.integers(0, 4, 300)] + rng.standard_normal((300, d))).astype(np.float32)
    t = _index(mv, base, d, 4, M)
    g = mv.IndexIVFPQ(d, 4, M)
    g.set_codebooks(centers, t.codebooks()[1])
    g.add(base)
    assert np.diff(g.lists()[0]).tolist() == sizes
    n = sum(sizes)
    dist, lab = g.search(q, n, form=mv.FORM_FAST, nprobe=4, lut=5)
    for i in range(0, 300, 37):
        assert np.array_equal(np.sort(lab[i]), np.arange(n)), i
    _check_distances(g, q[::10], dist[::10], lab[::10], 0)
    d2, l2 = g.search(q, 1000, form=mv.FORM_FAST, nprobe=4, lut=5)
    assert np.array_equal(l2, lab[:, :1000])
    assert np.array_equal(d2.view(np.uint32), dist[:, :1000].view(np.uint32))


@pytest.mark.parametrize("rerank", [0, 64])
def test_tc_filter_equals_index_without_filtered_rows(mv, rerank):
    rng = np.random.default_rng(41)
    base, q = _clustered(15000, 64, 30, seed=42)
    g = _index(mv, base, 64, 64, 16)
    flt = (rng.random(len(base)) < 0.3).astype(np.uint8)
    a_d, a_l = g.search(q, 20, form=mv.FORM_FAST, nprobe=10, rerank=rerank, filter=flt, lut=5)
    assert not flt[a_l[a_l >= 0]].any()
    keep = np.flatnonzero(flt == 0)
    h = mv.IndexIVFPQ(64, 64, 16)
    cent, pq = g.codebooks()
    h.set_codebooks(cent, pq)
    h.add_with_ids(base[keep], keep.astype(np.int64))
    b_d, b_l = h.search(q, 20, form=mv.FORM_FAST, nprobe=10, rerank=rerank, lut=5)
    assert np.array_equal(a_l, b_l)
    assert np.array_equal(a_d.view(np.uint32), b_d.view(np.uint32))


def test_tc_ties(mv):
    """400 equal rows: equal distances at the shortlist boundary are cut by
    the smaller position, the same way for any k."""
    base, q = _clustered(15000, 64, 30, seed=6)
    base[5000:5400] = base[5000]
    q[:10] = base[5000]
    g = _index(mv, base, 64, 64, 16)
    fd, fl = g.search(q, 1000, form=mv.FORM_FAST, nprobe=12, lut=5)
    for k in (10, 300):
        d, l = g.search(q, k, form=mv.FORM_FAST, nprobe=12, lut=5)
        assert np.array_equal(l, fl[:, :k]) and np.array_equal(d.view(np.uint32), fd[:, :k].view(np.uint32))


def test_tc_recall_and_determinism(mv):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(100000, d=128, n_centers=256, nq=500, seed=21)
    g = _index(mv, base, 128, 256, 16)
    flat = mv.IndexFlat(128, 0)
    flat.add(base)
    _, gt = flat.search(q, 10)

    def recall(lab):
        return np.mean([len(set(gt[i]) & set(lab[i])) / 10 for i in range(len(q))])

    runs = [g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=400, lut=5) for _ in range(3)]
    for d, l in runs[1:]:
        assert np.array_equal(l, runs[0][1]) and np.array_equal(d, runs[0][0])
    _, l0 = g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=400, lut=0)
    assert recall(runs[0][1]) >= recall(l0) - 0.01


def test_tc_batch_plan_equals_direct(mv):
    """Per-query nprobe and k in one plan (graph replay): each query's
    results equal its own direct search."""
    base, q = _clustered(20000, 64, 50, seed=9, nq=300)
    g = _index(mv, base, 64, 128, 16, ntrain=10000)
    rng = np.random.default_rng(10)
    nprobe = rng.integers(1, 60, size=len(q)).astype(np.int32)
    k = rng.choice(np.array([1, 10, 100], np.int32), size=len(q))
    plan = mv.IVFPQBatchPlan(g, len(q), 64, 100, rerank=128, lut=5)
    plan.set_queries(q, nprobe, k)
    plan.run(len(q), use_graph=True)
    d, l = plan.results(len(q))
    for i in range(0, len(q), 7):
        dd, ll = g.search(q[i:i + 1], int(k[i]), form=mv.FORM_FAST, nprobe=int(nprobe[i]), rerank=128,
                          lut=5)
        assert np.array_equal(ll[0], l[i, :k[i]]) and np.array_equal(dd[0], d[i, :k[i]]), i
