"""IVF-Flat (index/index_ivf_flat.mojo) and the exact rerank of candidate
lists (index/index_hnsw.mojo:433-497 semantics) against the oracle.

The plain IVF-Flat form must equal the oracle bit for bit: training
(k-means centroids), list assignment and order, and the search's ids and
distances (l2_distance_simd[8] / -inner_product_simd[4], canonical ties,
tail 1e38 / -1, IP un-negated). The fast form probes with the BF16 coarse
step; probing every list makes it exact again.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(31337)


def _same(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all(a == b))


@pytest.mark.parametrize("d", [16, 33, 128])
@pytest.mark.parametrize("metric", [0, 1])
def test_ivfflat_plain_matches_oracle(mv, orc, d, metric):
    x = (RNG.standard_normal((4000, d)) * 2).astype(np.float32)
    q = (RNG.standard_normal((50, d)) * 2).astype(np.float32)
    g = mv.IndexIVFFlat(d, 48, metric)
    g.train(x[:3000])
    o = orc.IVFFlat(d, 48, metric)
    o.train(x[:3000])
    assert np.array_equal(g.centroids(), o.centroids())
    g.add(x[:1500])
    g.add(x[1500:])
    o.add(x[:1500])
    o.add(x[1500:])
    for nprobe in (1, 7, 48):
        for k in (1, 10):
            gd, gl = g.search(q, k, nprobe=nprobe)
            od, ol = o.search(q, k, nprobe)
            assert np.array_equal(gl, ol), (nprobe, k)
            assert _same(gd, od), (nprobe, k)


def test_ivfflat_tail_untrained_and_fast(mv, orc):
    x = RNG.standard_normal((3000, 24)).astype(np.float32)
    g = mv.IndexIVFFlat(24, 32, 0)
    d, l = g.search(x[:3], 4)  # untrained: 1e38 / -1 (:176-180)
    assert (l == -1).all() and (d == 1e38).all()
    g.train(x)
    g.add(x[:20])
    d, l = g.search(x[:5], 30, nprobe=2)  # fewer candidates than k
    assert (l[:, -1] == -1).all() and (d[:, -1] == 1e38).all()
    g.add(x[20:])
    pd, pl = g.search(x[:200], 10, nprobe=32)
    fd, fl = g.search(x[:200], 10, nprobe=32, form=mv.FORM_FAST)  # every list probed
    assert np.array_equal(pl, fl) and _same(pd, fd)
    _, fl8 = g.search(x[:200], 10, nprobe=8, form=mv.FORM_FAST)
    _, pl8 = g.search(x[:200], 10, nprobe=8)
    agree = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(fl8, pl8)])
    assert agree > 0.98


@pytest.mark.parametrize("metric", [0, 1])
def test_flat_rerank_matches_oracle(mv, orc, metric):
    base = RNG.standard_normal((5000, 96)).astype(np.float32)
    q = RNG.standard_normal((64, 96)).astype(np.float32)
    cand = RNG.integers(-1, 5000, size=(64, 40)).astype(np.int64)  # -1 = empty slot
    cand[:3] = -1  # queries without candidates
    flat = mv.IndexFlat(96, metric)
    flat.add(base)
    gd, gl = flat.rerank(q, cand, 10)
    od, ol = orc.rerank(base, q, cand, 10, metric=metric)
    assert np.array_equal(gl, ol)
    assert _same(gd, od)
    assert (gl[:3] == -1).all() and (gd[:3] == 0.0).all()
    with pytest.raises(mv.MojoVecGPUError):
        flat.rerank(q[:1], np.array([[5000]], np.int64), 1)


def test_ivfflat_reference_known_answers(mv):
    # tests/test_ivf_flat.mojo: exact match (d 4, one row, nlist 1) and the
    # sparse tail (one row with id 42, k 5 -> then 1e38 / -1)
    row = np.arange(4, dtype=np.float32)[None, :]
    g = mv.IndexIVFFlat(4, 1, 0)
    g.train(row)
    g.add(row)
    d, l = g.search(row, 1)
    assert l[0, 0] == 0 and abs(d[0, 0]) < 1e-6
    z = np.zeros((1, 4), np.float32)
    t = mv.IndexIVFFlat(4, 1, 0)
    t.train(z)
    t.add(z, ids=np.array([42]))
    d, l = t.search(z, 5)
    assert l[0].tolist() == [42, -1, -1, -1, -1]
    assert d[0, 0] == 0.0 and (d[0, 1:] == 1e38).all()


def test_device_entry_points_match_host_calls(mv):
    """mv_ivfflat_search_device and mv_flat_rerank_device (device buffers,
    caller stream) return the host-buffer calls' bits."""
    torch = pytest.importorskip("torch")
    x = (RNG.standard_normal((6000, 48)) * 2).astype(np.float32)
    q = (RNG.standard_normal((70, 48)) * 2).astype(np.float32)
    g = mv.IndexIVFFlat(48, 32, 0)
    g.train(x[:3000])
    g.add(x)
    dq = torch.from_numpy(q).cuda()
    dd = torch.empty((70, 10), dtype=torch.float32, device="cuda")
    dl = torch.empty((70, 10), dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    for form in (mv.FORM_PLAIN, mv.FORM_FAST):
        hd, hl = g.search(q, 10, nprobe=5, form=form)
        g.search_device(dq.data_ptr(), 70, 10, dd.data_ptr(), dl.data_ptr(), stream=s.cuda_stream,
                        nprobe=5, form=form)
        torch.cuda.synchronize()
        assert np.array_equal(dl.cpu().numpy(), hl) and _same(dd.cpu().numpy(), hd)
    f = mv.IndexFlat(48, 1)
    f.add(x)
    cand = RNG.integers(-1, 6000, size=(70, 24)).astype(np.int64)
    hd, hl = f.rerank(q, cand, 10)
    dc = torch.from_numpy(cand).cuda()
    f.rerank_device(dq.data_ptr(), 70, dc.data_ptr(), 24, 10, dd.data_ptr(), dl.data_ptr(),
                    stream=s.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dl.cpu().numpy(), hl) and _same(dd.cpu().numpy(), hd)


@pytest.mark.parametrize("metric", [0, 1])
def test_ivfflat_list_major_chunks_and_k_limits(mv, orc, metric):
    """The list-major scan (k <= 32) and its fallback (k > 32) against the
    oracle: clustered queries put hundreds of queries on the same few lists
    (many 8-query chunks per list), k at both sides of the limit."""
    d = 37  # not a multiple of 4: the scalar staging path
    cent = (RNG.standard_normal((12, d)) * 6).astype(np.float32)
    x = (cent[RNG.integers(0, 12, 5000)] + RNG.standard_normal((5000, d))).astype(np.float32)
    q = (cent[RNG.integers(0, 3, 300)] + 0.5 * RNG.standard_normal((300, d))).astype(np.float32)
    g = mv.IndexIVFFlat(d, 40, metric)
    g.train(x[:3000])
    o = orc.IVFFlat(d, 40, metric)
    o.train(x[:3000])
    g.add(x)
    o.add(x)
    for k in (1, 32, 33):
        for nprobe in (3, 12):
            gd, gl = g.search(q, k, nprobe=nprobe)
            od, ol = o.search(q, k, nprobe)
            assert np.array_equal(gl, ol), (k, nprobe)
            assert _same(gd, od), (k, nprobe)
