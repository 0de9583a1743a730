"""Rows longer than 256 elements: the fused top-k GEMM streams the query
block through shared memory with the base tiles (K streaming). The plain
Flat search must stay identical to the exact FP32 scan (and to the oracle),
the fast Flat form must keep its recall, SQ8 inner product at d = 768 must
return the integer scan's results bit for bit, and the certified
assignment must equal the exact one."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [320, 768])
@pytest.mark.parametrize("metric", [0, 1])
def test_flat_long_rows(mv, orc, d, metric):
    from mojovec_gb300 import synth

    base, q = synth.cos_mixture(12000, d=d, n_centers=128, seed=71, nq=120)
    ix = mv.IndexFlat(d, metric)
    ix.add(base)
    st0 = mv.Context.default().certify_stats()
    pd, pl = ix.search(q, 10)
    st1 = mv.Context.default().certify_stats()
    assert st1["flat_queries"] - st0["flat_queries"] == len(q)  # the certified path ran
    sd, sl = ix.search(q, 10, plain_scan=True)
    assert np.array_equal(pl, sl) and np.array_equal(pd.view(np.uint32), sd.view(np.uint32))
    rd, rl = orc.flat_search(base, q, 10, metric=metric)
    assert np.array_equal(pl, rl)
    fd, fl = ix.search(q, 10, form=mv.FORM_FAST, rerank=40)
    rec = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(fl, sl)])
    assert rec >= 0.99


def test_sq8_ip_768_tensor_equals_integer_scan(mv):
    from mojovec_gb300 import synth

    base, q = synth.cos_mixture(20000, d=768, n_centers=256, seed=72, nq=100)
    ix = mv.IndexFlatSQ8(768, mv.METRIC_IP)
    ix.add(base)
    td, tl = ix.search(q, 10, rerank_factor=2)  # tensor-core keys (exact for s8 at d <= 1040)
    sd, sl = ix.search(q, 10, rerank_factor=2, plain_scan=True)  # integer scan
    assert np.array_equal(tl, sl) and np.array_equal(td.view(np.uint32), sd.view(np.uint32))


def test_assign_and_kmeans_long_rows(mv, orc):
    from mojovec_gb300 import synth

    x, _ = synth.cos_mixture(20000, d=512, n_centers=64, seed=73)
    km = mv.KMeans(512, 100, 3)
    r0, _ = mv.Context.default().assign_stats()
    km.train(x)
    r1, _ = mv.Context.default().assign_stats()
    assert r1 - r0 >= 3 * 20000  # certified assignment with streamed K
    rc, ra = orc.kmeans_train(x, 100, niter=3)
    assert np.array_equal(km.centroids.view(np.uint32), rc.view(np.uint32))
    assert np.array_equal(km.assignments, ra)
    fast = mv.KMeans(512, 100, 3, form=mv.FORM_FAST)
    fast.train(x)
    rel = abs(fast.objective[-1] - km.objective[-1]) / km.objective[-1]
    assert rel < 1e-3


@pytest.mark.parametrize("metric", [0, 1])
def test_ivfpq_long_rows(mv, orc, metric):
    """d = 384: certified coarse step (streamed K) and device assignment in
    the plain form equal the oracle; both fast coarse paths (fused GEMM, and
    the exact matrix that replaces the BF16 one past d = 256) keep recall."""
    from mojovec_gb300 import synth

    d, nlist, M = 384, 64, 16
    base, q = synth.cos_mixture(12000, d=d, n_centers=48, seed=74, nq=150)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base[:6000], niter_coarse=4, niter_pq=3)
    cent, pq = g.codebooks()
    r = orc.IVFPQ(d, nlist, M, metric)
    r.set_codebooks(cent, pq)
    g.add(base)
    r.add(base)
    for nprobe in (4, 16):
        gd, gl = g.search(q, 10, nprobe=nprobe)
        rd, rl = r.search(q, 10, nprobe)
        assert np.array_equal(gl, rl), nprobe
        assert np.array_equal(np.asarray(gd, np.float32).view(np.uint32),
                              np.asarray(rd, np.float32).view(np.uint32)), nprobe
    # The shortlist quality is PQ's (24-dim subspaces on noisy rows); what the
    # streamed coarse step must show is that it picks the FP32 coarse lists.
    _, ref = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=100, coarse_fp32=True)
    for cpath in (1, 2):
        _, fl = g.search(q, 10, form=mv.FORM_FAST, nprobe=16, rerank=100, coarse_path=cpath)
        agree = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(fl, ref)])
        assert agree >= 0.97, (cpath, agree)


def test_ivfflat_long_rows(mv, orc):
    from mojovec_gb300 import synth

    d = 512
    base, q = synth.cos_mixture(8000, d=d, n_centers=40, seed=75, nq=80)
    g = mv.IndexIVFFlat(d, 48, 0)
    g.train(base[:5000], niter=4)
    o = orc.IVFFlat(d, 48, 0)
    o.train(base[:5000], niter=4)
    assert np.array_equal(g.centroids(), o.centroids())
    g.add(base)
    o.add(base)
    for nprobe in (3, 20):
        gd, gl = g.search(q, 10, nprobe=nprobe)
        od, ol = o.search(q, 10, nprobe)
        assert np.array_equal(gl, ol), nprobe
        assert np.array_equal(np.asarray(gd, np.float32), np.asarray(od, np.float32)), nprobe
    _, fl = g.search(q, 10, nprobe=48, form=mv.FORM_FAST)
    _, pl = g.search(q, 10, nprobe=48)
    assert np.mean([len(set(a) & set(b)) / 10 for a, b in zip(fl, pl)]) >= 0.99
