"""Fast-form (tensor-core) checks.

* The BF16 tcgen05 distance GEMM is exact when every input is an integer of
  small magnitude (BF16 represents it exactly and every FP32 partial sum is
  an integer below 2^24), so it is compared bit for bit with int64 numpy.
* On real-valued data it is compared with an FP64 reference within the BF16
  rounding bound.
* The fast IVF-PQ search becomes exact when every list is probed and the
  rerank shortlist holds every candidate: it must then return the exact
  Flat answer. Recall floors and determinism are checked at realistic sizes.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(777)


def _int_rows(n, d, lo=-8, hi=8):
    return RNG.integers(lo, hi + 1, size=(n, d)).astype(np.float32)


@pytest.mark.parametrize("d", [8, 32, 64, 96, 128, 200, 256])
@pytest.mark.parametrize("nx,ny", [(1, 1), (130, 77), (300, 600)])
def test_umma_exact_on_integers(mv, d, nx, ny):
    x = _int_rows(nx, d)
    y = _int_rows(ny, d)
    xi = x.astype(np.int64)
    yi = y.astype(np.int64)
    dot = xi @ yi.T
    l2 = (xi * xi).sum(1)[:, None] + (yi * yi).sum(1)[None, :] - 2 * dot
    got_l2 = mv.distance_matrix(x, y, metric=0, precision=1)
    got_ip = mv.distance_matrix(x, y, metric=1, precision=1)
    assert np.array_equal(got_l2, l2.astype(np.float32))
    assert np.array_equal(got_ip, (-dot).astype(np.float32))


def test_umma_real_valued_within_bf16_bound(mv):
    x = RNG.standard_normal((513, 128)).astype(np.float32)
    y = RNG.standard_normal((1031, 128)).astype(np.float32)
    ref = -(x.astype(np.float64) @ y.T.astype(np.float64))
    got = mv.distance_matrix(x, y, metric=1, precision=1)
    bound = 2.0 ** -7 * np.abs(x).astype(np.float64) @ np.abs(y).T.astype(np.float64) + 1e-4
    assert (np.abs(got - ref) <= bound).all()


def test_exact_matrix_matches_oracle_order(mv, orc):
    x = RNG.standard_normal((70, 100)).astype(np.float32)
    y = RNG.standard_normal((90, 100)).astype(np.float32)
    got = mv.distance_matrix(x, y, metric=0, precision=0)
    for i in range(0, 70, 7):
        for j in range(0, 90, 11):
            assert got[i, j] == np.float32(orc.l2_simd(x[i], y[j]))


def _index(mv, base, d, nlist, M, metric=0):
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base[: min(len(base), 20000)], niter_coarse=6, niter_pq=6)
    g.add(base)
    return g


@pytest.mark.parametrize("metric", [0, 1])
def test_fast_exhaustive_equals_flat(mv, metric):
    base = RNG.standard_normal((3000, 64)).astype(np.float32)
    q = RNG.standard_normal((40, 64)).astype(np.float32)
    g = _index(mv, base, 64, 16, 8, metric)
    d, l = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=3000)
    dh, lh = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=3000, lut_fp16=True)
    assert np.array_equal(l, lh) and np.array_equal(d, dh)  # every candidate reranked
    flat = mv.IndexFlat(64, metric)
    flat.add(base)
    fd, fl = flat.search(q, 10)
    assert np.array_equal(l, fl)
    assert np.allclose(d, fd, rtol=1e-5, atol=1e-4)


def test_fast_recall_and_determinism(mv):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(100000, d=128, n_centers=256, nq=500, seed=21)
    g = _index(mv, base, 128, 256, 16)
    flat = mv.IndexFlat(128, 0)
    flat.add(base)
    _, gt = flat.search(q, 10)

    def recall(lab):
        return np.mean([len(set(gt[i]) & set(lab[i])) / 10 for i in range(len(q))])

    g.nprobe = 32
    _, lp = g.search(q, 10)
    r_plain = recall(lp)
    _, lf = g.search(q, 10, form=mv.FORM_FAST, nprobe=32)
    r_fast = recall(lf)
    assert abs(r_fast - r_plain) < 0.05  # same PQ quantisation, different rounding
    runs = [g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=400) for _ in range(3)]
    for d, l in runs[1:]:
        assert np.array_equal(l, runs[0][1]) and np.array_equal(d, runs[0][0])
    r_rerank = recall(runs[0][1])
    assert r_rerank > r_plain + 0.2
    # FP16 tables (per-query power-of-two scale): same recall within 0.01
    h = [g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=400, lut_fp16=True) for _ in range(2)]
    assert np.array_equal(h[0][1], h[1][1])
    assert abs(recall(h[0][1]) - r_rerank) < 0.01
    _, lc = g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=400, coarse_fp32=True)
    assert abs(recall(lc) - r_rerank) < 0.02


@pytest.mark.parametrize("nprobe", [3, 12])
def test_fast_shortlist_select_is_exact(mv, nprobe):
    """With rerank 0 the shortlist is the answer, sorted by (table distance,
    position). At nprobe 3 most queries have fewer than 2048 candidates, so
    k = 2048 returns every candidate with no radix select; a smaller k runs
    the block radix select and must return exactly that list's first k
    entries. At nprobe 12 queries stage more keys than the staging area
    holds, so intermediate selects run first; the k smallest must still be
    a prefix of the 2048 smallest."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(24000, d=32, n_centers=64, nq=150, seed=23)
    g = _index(mv, base, 32, 64, 8)
    fd, fl = g.search(q, 2048, form=mv.FORM_FAST, nprobe=nprobe)
    if nprobe == 3:
        assert np.mean((fl == -1).any(axis=1)) > 0.5  # complete candidate lists
    for k in (10, 100, 256, 700):
        d, l = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe)
        assert np.array_equal(l, fl[:, :k]), k
        assert np.array_equal(d.view(np.uint32), fd[:, :k].view(np.uint32)), k


def test_search_into_caller_arrays(mv):
    """Results written into caller-provided pinned arrays equal the
    allocating call's, for IVF-PQ (both forms), IVF-Flat, Flat and SQ8."""
    import torch
    from mojovec_gb300 import synth

    base, q = synth.sift_like(20000, d=64, n_centers=64, nq=300, seed=24)
    g = _index(mv, base, 64, 64, 8)
    f = mv.IndexIVFFlat(64, 64, 0)
    f.train(base[:8000], niter=4)
    f.add(base)
    fl = mv.IndexFlat(64, 0)
    fl.add(base)
    sq = mv.IndexFlatSQ8(64, 0)
    sq.add(base)
    hq = torch.from_numpy(q).pin_memory().numpy()
    cases = [(g, dict(nprobe=8)), (g, dict(form=mv.FORM_FAST, nprobe=8, rerank=64)),
             (f, dict(nprobe=8)), (fl, {}), (sq, {}), (sq, dict(rerank_factor=2))]
    for ix, kw in cases:
        dt = torch.full((len(q), 10), -7.0).pin_memory()
        lt = torch.full((len(q), 10), -7, dtype=torch.int64).pin_memory()
        rd, rl = ix.search(hq, 10, **kw, distances=dt.numpy(), labels=lt.numpy())
        assert rd.ctypes.data == dt.data_ptr() and rl.ctypes.data == lt.data_ptr()
        ed, el = ix.search(q, 10, **kw)
        assert np.array_equal(lt.numpy(), el) and np.array_equal(dt.numpy(), ed), kw


def test_fast_untrained_and_small_lists(mv):
    g = mv.IndexIVFPQ(16, 8, 4)
    d, l = g.search(np.zeros((2, 16), np.float32), 5, form=mv.FORM_FAST, nprobe=4)
    assert (l == -1).all()
    base = RNG.standard_normal((300, 16)).astype(np.float32)
    g.train(base, niter_coarse=3, niter_pq=3)
    g.add(base[:20])
    d, l = g.search(base[:3], 50, form=mv.FORM_FAST, nprobe=8, rerank=100)
    assert (l[:, 20:] == -1).all() and set(l[0, :20].tolist()) == set(range(20))
    assert l[0, 0] == 0 and d[0, 0] == 0.0


def test_fast_search_in_fresh_process():
    """Each kernel's shared-memory limit is raised on first use; a search in
    a fresh process must not depend on an earlier call having raised it."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = (
        "import numpy as np, mojovec_gb300 as mv\n"
        "from mojovec_gb300 import synth\n"
        "b, q = synth.sift_like(20000, d=128, n_centers=64, nq=300, seed=5)\n"
        "g = mv.IndexIVFPQ(128, 64, 16); g.train(b, niter_coarse=3, niter_pq=3); g.add(b)\n"
        "d, l = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=256)\n"
        "d2, l2 = g.search(q, 10, form=mv.FORM_FAST, nprobe=16)\n"
        "assert (l >= 0).all() and (l2 >= 0).all()\n"
        "print('ok')\n"
    )
    r = subprocess.run([sys.executable, "-c", script], cwd=root, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]


def test_fast_fused_coarse_matches_matrix_coarse(mv):
    """The fused GEMM + per-row top-k coarse step (used while nprobe plus its
    margin fits 64 lists per query) and the distance-matrix path must pick
    the same probes as the exact FP32 coarse step up to BF16 near-ties."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(40000, d=96, n_centers=64, nq=400, seed=33)
    g = _index(mv, base, 96, 512, 24)
    # nprobe 4, 16, 48 keep at most 64 lists per query (fused GEMM + heap);
    # nprobe 80 keeps 100 (distance matrix + radix select)
    for nprobe in (4, 16, 48, 80):
        _, lf = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=100)
        _, lc = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=100, coarse_fp32=True)
        agree = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(lf, lc)])
        assert agree > 0.97, (nprobe, agree)


@pytest.mark.parametrize("metric", [0, 1])
def test_fast_paths_pick_the_same_lists(mv, metric):
    """coarse_path 1 (fused GEMM + per-row heap), 2 (distance matrix + one
    warp per query) and 3 (two-pass GEMM + per-row lists, also the automatic
    choice up to 32 lists per query) keep the same approximate top-nc
    lists, so the searches agree exactly."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(40000, d=96, n_centers=64, nq=300, seed=34)
    g = _index(mv, base, 96, 512, 24, metric)
    for nprobe in (1, 4, 16, 24, 48):
        a = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=64, coarse_path=1)
        for cpath in (0, 2, 3):
            b = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=64, coarse_path=cpath)
            assert np.array_equal(a[1], b[1]) and np.array_equal(a[0], b[0]), (nprobe, cpath)


@pytest.mark.parametrize("d", [64, 200])
def test_two_pass_coarse_lists_compact_exactly(mv, d):
    """200 identical centroids nearest to every query tie at the two-pass
    threshold: each row's list overflows its slots and is compacted, and the
    kept lists (the smallest list ids among the ties) must still equal the
    heap and matrix paths'."""
    rng = np.random.default_rng(35)
    nlist, M = 1024, 8
    cent = rng.standard_normal((nlist, d)).astype(np.float32) * 4
    cent[100:300] = cent[100]
    base = cent[rng.integers(0, nlist, 30000)] + rng.standard_normal((30000, d)).astype(np.float32)
    q = cent[100] + 0.01 * rng.standard_normal((257, d)).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M)
    g.train(base[:8000], niter_coarse=2, niter_pq=2)
    _, pq = g.codebooks()
    g.set_codebooks(cent, pq)
    g.add(base)
    for nprobe in (8, 24):
        a = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=50, coarse_path=1)
        for cpath in (2, 3):
            b = g.search(q, 10, form=mv.FORM_FAST, nprobe=nprobe, rerank=50, coarse_path=cpath)
            assert np.array_equal(a[1], b[1]) and np.array_equal(a[0], b[0]), (nprobe, cpath)


@pytest.mark.parametrize("rerank", [0, 128])
def test_fast_filter_equals_index_without_filtered_rows(mv, rerank):
    """index_ivf_pq.mojo:328-334 in the fast form: a filtered id never enters
    the shortlist, so the search equals the same search over an index that
    never held those rows (same codebooks, same ids). A filter shorter than
    the ids leaves the ids past its end unfiltered."""
    rng = np.random.default_rng(31)
    d, nlist, M, n = 64, 64, 8, 20000
    x = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((200, d)).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M)
    g.train(x[:8000], niter_coarse=4, niter_pq=4)
    cent, pq = g.codebooks()
    g.add(x)
    filt = (rng.random(n - 3000) < 0.3).astype(np.uint8)  # ids >= n - 3000 stay in
    keep = np.flatnonzero(np.concatenate([filt, np.zeros(3000, np.uint8)]) == 0)
    h = mv.IndexIVFPQ(d, nlist, M)
    h.set_codebooks(cent, pq)
    h.add_with_ids(x[keep], keep)
    a_d, a_l = g.search(q, 10, filter=filt, form=mv.FORM_FAST, nprobe=8, rerank=rerank)
    b_d, b_l = h.search(q, 10, form=mv.FORM_FAST, nprobe=8, rerank=rerank)
    hit = a_l[(a_l >= 0) & (a_l < len(filt))]
    assert not filt[hit].any()
    assert np.array_equal(a_l, b_l) and np.array_equal(a_d, b_d)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d", [64, 96, 130])
def test_certified_rerank_prescreen_is_exact(mv, metric, d):
    """The 8-bit prescreen of the rerank (default) must return the bits of the
    rerank that computes every shortlisted row in FP32 (rerank_fp32): on
    real-valued rows, on SIFT-like integer rows, with duplicated rows (exact
    ties across the k-th boundary) and with k from 1 to 32."""
    from mojovec_gb300 import synth

    rng = np.random.default_rng(36 + d)
    if d == 96:
        base, q = synth.sift_like(20000, d=d, n_centers=64, nq=150, seed=37)
    else:
        base = rng.standard_normal((20000, d)).astype(np.float32)
        base[5000:5400] = base[5000]  # 400 identical rows
        q = np.vstack([base[5000:5020] + 1e-3 * rng.standard_normal((20, d)).astype(np.float32),
                       rng.standard_normal((130, d)).astype(np.float32)])
    g = _index(mv, base, d, 64, 8 if d != 130 else 10, metric)
    for k, R in ((1, 16), (10, 256), (32, 100)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=6, rerank=R)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=6, rerank=R, rerank_fp32=True)
        assert np.array_equal(a[1], b[1]), (k, R)
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)), (k, R)


@pytest.mark.parametrize("metric", [0, 1])
def test_certified_rerank_offset_rows(mv, metric):
    """Rows and queries far from the origin against their spread (4096 plus
    noise of 1e-3, and a second cluster at -3e5): the 8-bit copy's
    per-dimension offsets and the per-query constants of the prescreen
    round, and the certified rerank must still return the full FP32
    rerank's bits."""
    rng = np.random.default_rng(39)
    d = 64
    base = (4096.0 + 1e-3 * rng.standard_normal((12000, d))).astype(np.float32)
    base[6000:] = (-3e5 + 0.25 * rng.standard_normal((6000, d))).astype(np.float32)
    base[100:140] = base[100]  # exact ties
    q = np.vstack([base[rng.integers(0, 12000, 60)] + 1e-4 * rng.standard_normal((60, d)),
                   base[100:104]]).astype(np.float32)
    g = _index(mv, base, d, 32, 8, metric)
    for k, R in ((1, 32), (10, 128), (32, 64)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=8, rerank=R)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=8, rerank=R, rerank_fp32=True)
        assert np.array_equal(a[1], b[1]), (k, R)
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)), (k, R)


@pytest.mark.parametrize("metric", [0, 1])
def test_certified_rerank_odd_queries(mv, metric):
    """Queries with a NaN component, all zeros, or huge values: the certified
    rerank keeps such candidates (non-finite intervals always survive) and
    must return the full FP32 rerank's bits."""
    rng = np.random.default_rng(38)
    d = 64
    base = rng.standard_normal((8000, d)).astype(np.float32)
    q = rng.standard_normal((8, d)).astype(np.float32)
    q[0, 3] = np.nan
    q[1] = 0.0
    q[2] *= 1e18
    q[3] *= 1e-20
    g = _index(mv, base, d, 32, 8, metric)
    a = g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=64, coarse_fp32=True)
    b = g.search(q, 10, form=mv.FORM_FAST, nprobe=32, rerank=64, coarse_fp32=True, rerank_fp32=True)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
