"""Serving loop (mv_server_*): continuous batching over three resident
collections (IVF-PQ, Flat, SQ8). Every request must get the same bits when
it runs alone and when it is batched with concurrent requests of other
sizes, and the same as a direct search call; requests are batched
(fewer batches than requests) and the in-flight memory stays within the
budget; requests larger than a batch are split; lanes' batches overlap on
the device.
"""

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _collections(mv):
    from mojovec_gb300 import synth

    base, _ = synth.sift_like(40000, d=64, n_centers=100, seed=23)
    ivf = mv.IndexIVFPQ(64, 128, 16)
    ivf.train(base[:15000], niter_coarse=5, niter_pq=5)
    ivf.add(base)
    rng = np.random.default_rng(5)
    flat = mv.IndexFlat(32, mv.METRIC_IP)
    flat.add(rng.standard_normal((20000, 32)).astype(np.float32))
    sq8 = mv.IndexFlatSQ8(32, mv.METRIC_L2)
    sq8.add(rng.standard_normal((20000, 32)).astype(np.float32))
    return ivf, flat, sq8


def _direct(mv, idx, x, k):
    if isinstance(idx, mv.IndexIVFPQ):
        return idx.search(x, k, form=mv.FORM_FAST, nprobe=8, rerank=64)
    if isinstance(idx, mv.IndexFlat):
        return idx.search(x, k, form=mv.FORM_FAST, rerank=40)
    return idx.search(x, k, form=mv.FORM_FAST, rerank_factor=2)


def test_alone_equals_mix_and_direct(mv):
    ivf, flat, sq8 = _collections(mv)
    srv = mv.Server(hbm_budget=3 << 30, lanes=4, max_batch_queries=512)
    ids = [srv.add(ivf, form=mv.FORM_FAST, nprobe=8, rerank=64),
           srv.add(flat, form=mv.FORM_FAST, rerank=40),
           srv.add(sq8, form=mv.FORM_FAST, rerank_factor=2)]
    idxs = [ivf, flat, sq8]
    rng = np.random.default_rng(77)
    reqs = []
    for _ in range(120):
        c = int(rng.integers(0, 3))
        n = int(rng.integers(1, 48))
        k = int(rng.choice([10, 100]))
        x = rng.standard_normal((n, idxs[c].d)).astype(np.float32) * (30 if c == 0 else 1)
        reqs.append((c, x, k))
    alone = []
    for c, x, k in reqs:
        d, l, _ = srv.wait(srv.submit(ids[c], x, k))
        alone.append((d, l))
    before = srv.stats()
    mixed = [None] * len(reqs)

    def worker(part):
        rids = [(i, srv.submit(ids[reqs[i][0]], reqs[i][1], reqs[i][2])) for i in part]
        for i, rid in rids:
            d, l, lat = srv.wait(rid)
            assert lat > 0
            mixed[i] = (d, l)

    ths = [threading.Thread(target=worker, args=(list(range(t, len(reqs), 4)),)) for t in range(4)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    after = srv.stats()
    for i, (c, x, k) in enumerate(reqs):
        assert np.array_equal(alone[i][1], mixed[i][1]), i
        assert np.array_equal(alone[i][0], mixed[i][0]), i
        dd, ll = _direct(mv, idxs[c], x, k)
        assert np.array_equal(ll, mixed[i][1]) and np.array_equal(dd, mixed[i][0]), i
    assert after["completed"] - before["completed"] == len(reqs)
    assert after["batches"] - before["batches"] < len(reqs)  # requests were batched
    assert after["peak_inflight_bytes"] <= 3 << 30
    srv.close()


def test_large_requests_split_and_lanes_overlap(mv):
    """Requests above max_batch_queries are split into parts (batches of at
    most that many rows) and still equal the direct search; four large
    requests submitted together keep several lanes' batches on the device
    at the same instant (device intervals from CUDA events per batch)."""
    ivf, flat, sq8 = _collections(mv)
    srv = mv.Server(hbm_budget=8 << 30, lanes=4, max_batch_queries=256)
    cid = srv.add(ivf, form=mv.FORM_FAST, nprobe=8, rerank=64)
    rng = np.random.default_rng(9)
    reqs = [rng.standard_normal((n, 64)).astype(np.float32) * 30 for n in (1000, 700, 1024, 300)]
    b0 = srv.stats()["batches"]
    rids = [srv.submit(cid, x, 10) for x in reqs]
    outs = [srv.wait(r) for r in rids]
    st = srv.stats()
    # parts hold at most 256 rows (the last parts of different requests may share a batch)
    assert st["batches"] - b0 >= -(-sum(len(x) for x in reqs) // 256)
    for x, (d, l, _) in zip(reqs, outs):
        dd, ll = _direct(mv, ivf, x, 10)
        assert np.array_equal(ll, l) and np.array_equal(dd, d)
    peak, recorded = srv.device_overlap()
    assert recorded >= 4 and peak >= 2, (peak, recorded)
    srv.close()


def test_rejects_bad_requests(mv):
    ivf, flat, sq8 = _collections(mv)
    tiny = mv.Server(hbm_budget=1 << 20, lanes=1, max_batch_queries=64)
    tid = tiny.add(flat, form=mv.FORM_FAST, rerank=40)
    with pytest.raises(mv.MojoVecGPUError):
        tiny.submit(tid, np.zeros((10, 32), np.float32), 10)  # above the memory budget
    tiny.close()
    srv = mv.Server(hbm_budget=2 << 30, lanes=2, max_batch_queries=64)
    cid = srv.add(flat, form=mv.FORM_FAST, rerank=40)
    with pytest.raises((mv.MojoVecGPUError, KeyError)):
        srv.submit(cid + 5, np.zeros((1, 32), np.float32), 10)  # no such collection
    d, l, _ = srv.wait(srv.submit(cid, np.ones((3, 32), np.float32), 5))
    assert l.shape == (3, 5)
    d, l, _ = srv.wait(srv.submit(cid, np.ones((150, 32), np.float32), 5))  # three parts
    assert l.shape == (150, 5) and (l >= 0).all()
    srv.close()
