"""Plain-form parity: libmojovec_gpu.so against the oracle, bit for bit.

Every result here comes from the CUDA library through the C ABI; the oracle
(the C++ restatement of the reference CPU path) is the checker. Ids and codes
must be identical; distances must have identical FP32 bits (the plain form
reproduces the reference's operation order).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(12345)


def _rand(n, d, scale=1.0, integer=False):
    x = RNG.standard_normal((n, d)).astype(np.float32) * np.float32(scale)
    if integer:
        x = np.rint(np.abs(x)).astype(np.float32)
    return x


def _same(a, b):
    """Bitwise float equality (treats -0.0 and +0.0 as equal)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("d", [1, 3, 4, 7, 8, 12, 16, 31, 32, 33, 96, 128, 130, 256, 401, 768, 1000])
@pytest.mark.parametrize("metric", [0, 1])
def test_flat_exact_matches_oracle(mv, orc, d, metric):
    base = _rand(1500, d, 3.0)
    q = _rand(40, d, 3.0)
    ix = mv.IndexFlat(d, metric)
    ix.add(base[:700])
    ix.add(base[700:])
    gd, gl = ix.search(q, 10)
    rd, rl = orc.flat_search(base, q, 10, metric=metric)
    assert np.array_equal(gl, rl)
    assert _same(gd, rd)


def test_flat_ties_filter_and_tail(mv, orc):
    # integer rows: many exactly equal distances -> tie rule (smaller id first)
    base = np.rint(RNG.uniform(0, 3, size=(2000, 16))).astype(np.float32)
    q = np.rint(RNG.uniform(0, 3, size=(30, 16))).astype(np.float32)
    ix = mv.IndexFlat(16, 0)
    ix.add(base)
    flt = (RNG.uniform(size=2000) < 0.3).astype(np.uint8)
    gd, gl = ix.search(q, 25, filter=flt)
    rd, rl = orc.flat_search(base, q, 25, filter=flt)
    assert np.array_equal(gl, rl) and _same(gd, rd)
    assert not np.isin(gl, np.nonzero(flt)[0]).any()
    small = mv.IndexFlat(16, 0)
    small.add(base[:3])
    d3, l3 = small.search(q[:2], 5)
    assert (l3[:, 3:] == -1).all() and (d3[:, 3:] == 0.0).all()


def test_flat_reference_known_answers(mv):
    # tests/test_index_flat.mojo:6-81
    ix = mv.IndexFlat(4, 0)
    ix.add(np.array([[0] * 4, [1] * 4, [2] * 4], np.float32))
    d, l = ix.search(np.full((1, 4), 1.1, np.float32), 2)
    assert set(l[0].tolist()) == {1, 2}
    assert abs(d[0][0] - 0.04) < 1e-3 and abs(d[0][1] - 3.24) < 1e-3
    ip = mv.IndexFlat(4, 1)
    ip.add(np.array([[1] * 4, [2] * 4, [3] * 4], np.float32))
    d, l = ip.search(np.ones((1, 4), np.float32), 2)
    assert l[0].tolist() == [2, 1] and d[0].tolist() == [12.0, 8.0]


@pytest.mark.parametrize("n,d,k", [(1000, 16, 10), (257, 8, 17), (5, 16, 10), (600, 4, 7), (300, 2, 5), (2000, 33, 40)])
def test_kmeans_exact(mv, orc, n, d, k):
    x = _rand(n, d)
    km = mv.KMeans(d, k, 5)
    km.train(x)
    rc, ra = orc.kmeans_train(x, k, niter=5)
    assert _same(km.centroids, rc)
    assert np.array_equal(km.assignments, ra)


def test_kmeans_identical_points_no_nan(mv):
    # tests/test_kmeans.mojo:32-45
    km = mv.KMeans(16, 5, 5)
    km.train(np.ones((100, 16), np.float32))
    assert np.isfinite(km.centroids).all()


def test_kmeans_reproducible(mv):
    # tests/test_kmeans.mojo:48-72
    i = np.arange(257 * 8)
    x = (((i * 37 + (i // 8) * 11) % 101) / 50.0 - 1.0).astype(np.float32).reshape(257, 8)
    a = mv.KMeans(8, 17, 5)
    b = mv.KMeans(8, 17, 5)
    a.train(x)
    b.train(x)
    assert np.array_equal(a.centroids, b.centroids)


@pytest.mark.parametrize("d,M", [(16, 4), (32, 8), (128, 16), (96, 24), (64, 64), (40, 5)])
def test_pq_train_encode_tables_exact(mv, orc, d, M):
    x = _rand(1200, d)
    pq = mv.ProductQuantizer(d, M)
    pq.train(x, niter=4)
    ref = orc.pq_train(x, M, niter=4)
    assert _same(pq.centroids, ref)
    codes = pq.compute_codes(x)
    assert np.array_equal(codes, orc.pq_compute_codes(ref, x))
    for metric in (0, 1):
        t = pq.compute_distance_table(x[:5], metric)
        for i in range(5):
            assert _same(t[i], orc.pq_distance_table(ref, x[i], metric))


def test_pq_adc_identity(mv, orc):
    # tests/test_pq.mojo:57-114: ADC(q, code(q)) == ||q - decode(code(q))||^2
    x = orc.philox_uniform_matrix(191, 100, 16) * 2 - 1
    pq = mv.ProductQuantizer(16, 4)
    pq.train(x)
    codes = pq.compute_codes(x)
    dec = pq.decode(codes)
    t = pq.compute_distance_table(x[:1])[0]
    adc = sum(float(t[m, codes[0, m]]) for m in range(4))
    assert abs(adc - orc.l2_simd(x[0], dec[0], width=4)) <= 1e-5


def _ivf_pair(mv, orc, base, d, nlist, M, metric, niter=4):
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base, niter_coarse=niter, niter_pq=niter)
    r = orc.IVFPQ(d, nlist, M, metric)
    r.train(base, niter_coarse=niter, niter_pq=niter)
    return g, r


@pytest.mark.parametrize("d,nlist,M,metric", [(32, 16, 8, 0), (32, 16, 8, 1), (128, 64, 16, 0), (96, 32, 24, 0), (8, 8, 2, 0), (48, 20, 12, 1)])
def test_ivfpq_train_add_search_exact(mv, orc, d, nlist, M, metric):
    base = _rand(3000, d, 2.0)
    q = _rand(60, d, 2.0)
    g, r = _ivf_pair(mv, orc, base, d, nlist, M, metric)
    gc, gp = g.codebooks()
    rc, rp = r.codebooks()
    assert _same(gc, rc) and _same(gp, rp)
    g.add(base[:1000])
    r.add(base[:1000])
    g.add(base[1000:])
    r.add(base[1000:])
    go, gi, gk = g.lists()
    ro, ri, rk = r.lists()
    assert np.array_equal(go, ro) and np.array_equal(gi, ri) and np.array_equal(gk, rk)
    for nprobe in (1, 4, nlist, nlist + 5):
        g.nprobe = nprobe
        gd, gl = g.search(q, 10)
        rd, rl = r.search(q, 10, nprobe)
        assert np.array_equal(gl, rl), nprobe
        assert _same(gd, rd), nprobe


def test_ivfpq_given_codebooks_filter_and_tail(mv, orc):
    d, nlist, M = 32, 16, 8
    from mojovec_gb300 import synth

    base, q = synth.sift_like(4000, d=d, n_centers=40, nq=50, seed=3)
    r = orc.IVFPQ(d, nlist, M)
    r.train(base, niter_coarse=6, niter_pq=6)
    c, p = r.codebooks()
    g = mv.IndexIVFPQ(d, nlist, M)
    g.set_codebooks(c, p)
    ids = np.arange(4000, dtype=np.int64) * 3 + 7
    g.add_with_ids(base, ids)
    r.add(base, ids)
    flt = np.zeros(int(ids.max()) + 1, np.uint8)
    flt[ids[::5]] = 1
    g.nprobe = 3
    gd, gl = g.search(q, 30, filter=flt)
    rd, rl = r.search(q, 30, 3, filter=flt)
    assert np.array_equal(gl, rl) and _same(gd, rd)
    # k larger than the probed candidates: tail 1e38 / -1 (index_ivf_pq.mojo:284-286)
    g.nprobe = 1
    gd, gl = g.search(q[:4], 2048)
    rd, rl = r.search(q[:4], 2048, 1)
    assert np.array_equal(gl, rl) and _same(gd, rd)
    assert (gl == -1).any() and (gd[gl == -1] == np.float32(1e38)).all()


def test_ivfpq_untrained_and_empty(mv):
    g = mv.IndexIVFPQ(8, 4, 2)
    d, l = g.search(np.zeros((3, 8), np.float32), 5)
    assert (l == -1).all() and (d == np.float32(1e38)).all()


def test_ivfpq_grid_self_match(mv):
    # tests/test_ivf_pq.mojo:48-77 (collection lifecycle and self-match)
    from mojovec_gb300 import synth

    rows = synth.grid_vectors()
    col = mv.IVFPQCollection(8, nlist=8, pq_subvectors=2, nprobe=4, metric="l2", name="compressed")
    assert not col.is_trained()
    col.train(rows)
    col.add(list(range(10_000, 10_256)), rows)
    st = col.stats()
    assert st == {"count": 256, "dimension": 8, "nlist": 8, "M": 2, "nprobe": 4, "trained": True,
                  "metric": "l2", "code_size_bytes": 2}
    res = col.query(rows[:1], n_results=5)
    assert res["ids"][0][0] == 10_000 and res["distances"][0][0] < 1e-4
    col.set_nprobe(8)
    assert col.nprobe() == 8


@pytest.mark.parametrize("metric", ["cosine", "ip"])
def test_ivfpq_collection_metrics(mv, metric):
    # tests/test_ivf_pq.mojo:129-152
    from mojovec_gb300 import synth

    rows = synth.grid_vectors()
    query = rows[:1].copy()
    if metric == "ip":
        rows[0] *= 20.0
        query = rows[:1].copy()
    col = mv.IVFPQCollection(8, nlist=8, pq_subvectors=2, nprobe=8, metric=metric)
    col.add(list(range(256)), rows)
    res = col.query(query, n_results=1)
    assert res["ids"] == [[0]]
    if metric == "cosine":
        assert res["distances"][0][0] < 1e-4
    else:
        assert res["distances"][0][0] < 0.0


def test_collection_validation_messages(mv):
    # python/tests/test_binding_ivfpq.py:69-97
    from mojovec_gb300 import synth

    with pytest.raises(ValueError, match="dimension"):
        mv.IVFPQCollection(0, nlist=8, pq_subvectors=2)
    with pytest.raises(ValueError, match="divide dimension"):
        mv.IVFPQCollection(10, nlist=8, pq_subvectors=3)
    rows = synth.grid_vectors()
    col = mv.IVFPQCollection(8, nlist=8, pq_subvectors=2)
    col.add(list(range(256)), rows)
    with pytest.raises(ValueError, match="already exists"):
        col.add([0], rows[:1])
    with pytest.raises(ValueError, match="nprobe"):
        col.set_nprobe(9)
    with pytest.raises(ValueError, match="at least max"):
        mv.IVFPQCollection(8, nlist=8, pq_subvectors=2).train(rows[:255])
    with pytest.raises(ValueError, match="finite"):
        mv.IVFPQCollection(8, nlist=8, pq_subvectors=2).train(np.full((256, 8), np.nan, np.float32))


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d", [3, 16, 100, 128])
def test_sq8_exact(mv, orc, metric, d):
    x1 = _rand(800, d, 2.0)
    x2 = _rand(700, d, 3.0)  # widens the bounds -> requantize
    q = _rand(40, d, 2.0)
    g = mv.IndexFlatSQ8(d, metric)
    r = orc.SQ8(d, metric)
    for x in (x1, x2):
        g.add(x)
        r.add(x)
    gmin, gmax, gscale = r.params()
    assert g.global_min == gmin and g.global_max == gmax and g.scale == gscale
    gc, gn = g.codes()
    rc, rn = r.codes()
    assert np.array_equal(gc, rc) and np.array_equal(gn, rn)
    gd, gl = g.search(q, 10)
    rd, rl = r.search(q, 10)
    assert np.array_equal(gl, rl) and _same(gd, rd)
    # SQ8 shortlist of 2k + exact FP32 rerank (index_hnsw.mojo:433-497)
    gd2, gl2 = g.search_rerank(q, 10, 2)
    _, sl = r.search(q, 20)
    base = np.concatenate([x1, x2])
    rd2, rl2 = orc.rerank(base, q, sl, 10, metric=metric)
    assert np.array_equal(gl2, rl2) and _same(gd2, rd2)


def test_sq8_reference_known_answers(mv):
    # tests/test_metrics.mojo:56-96
    g = mv.IndexFlatSQ8(3, 1)
    g.add(np.array([[1, 0, 0], [-1, 0, 0], [0.5, 0, 0]], np.float32))
    d, l = g.search(np.array([[1, 0, 0]], np.float32), 3)
    assert l[0].tolist() == [0, 2, 1] and d[0][0] > d[0][1] > d[0][2]
    h = mv.IndexFlatSQ8(2, 1)
    h.add(np.array([[1.0, 0.25]], np.float32))
    h.add(np.array([[-4.0, 0.0]], np.float32))
    assert abs(h.scale - 4.0 / 127.0) < 1e-6


def test_sq8_encode_primitive(mv, orc):
    x = _rand(500, 37, 4.0)
    for sym in (False, True):
        mn = 0.0 if sym else float(x.min())
        inv = np.float32(1.0) / np.float32(0.05)
        gc, gn = mv.sq8_encode(x, mn, float(inv), sym)
        rc, rn = orc.sq8_encode(x, mn, float(inv), sym)
        assert np.array_equal(gc, rc) and np.array_equal(gn, rn)


def test_normalize_exact(mv, orc):
    x = _rand(300, 77, 5.0)
    assert np.array_equal(mv.normalize(x), orc.normalize(x))
    with pytest.raises(ValueError, match="non-zero"):
        mv.normalize(np.zeros((2, 4), np.float32))


def test_selection_is_deterministic_under_load(mv, orc):
    """Repeated large searches return identical results and match the
    oracle: the block top-k must never drop a candidate, whatever the warp
    timing (many rounds, frequent buffer flushes)."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(60000, d=64, n_centers=64, nq=3000, seed=11)
    r = orc.IVFPQ(64, 128, 8)
    r.train(base[:20000], niter_coarse=4, niter_pq=4)
    c, p = r.codebooks()
    g = mv.IndexIVFPQ(64, 128, 8)
    g.set_codebooks(c, p)
    g.add(base)
    r.add(base)
    g.nprobe = 24
    runs = [g.search(q, 50) for _ in range(4)]
    for d, l in runs[1:]:
        assert np.array_equal(l, runs[0][1]) and _same(d, runs[0][0])
    rd, rl = r.search(q[:400], 50, 24, lut_threads=8)
    assert np.array_equal(runs[0][1][:400], rl) and _same(runs[0][0][:400], rd)
    flat = mv.IndexFlat(64, 0)
    flat.add(base)
    fr = [flat.search(q[:500], 100) for _ in range(3)]
    for d, l in fr[1:]:
        assert np.array_equal(l, fr[0][1])
    od, ol = orc.flat_search(base, q[:100], 100)
    assert np.array_equal(fr[0][1][:100], ol) and _same(fr[0][0][:100], od)
