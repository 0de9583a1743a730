"""Batched fast IVF-PQ (mv_ivfpq_search_batch and the CUDA-graph plan).

With the exact FP32 coarse step and a shortlist at least as deep as the
largest k, every query of a batch must get exactly what a separate fast
search with its own nprobe and k returns, whatever the launch shape: the
tuner's candidates (fused or matrix coarse, 128/256/512 scan threads,
persistent or one-CTA-per-query grids) and the graph replay all give the
same bits.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(2468)


def _index(mv):
    from mojovec_gb300 import synth

    base, q = synth.sift_like(60000, d=64, n_centers=120, nq=300, seed=17)
    ix = mv.IndexIVFPQ(64, 256, 16)
    ix.train(base[:20000], niter_coarse=6, niter_pq=6)
    ix.add(base)
    return ix, q


def _reference_rows(mv, ix, q, nprobe, k, rerank):
    kmax = int(k.max())
    dist = np.full((len(q), kmax), 1e38, np.float32)
    lab = np.full((len(q), kmax), -1, np.int64)
    for np_, k_ in set(zip(nprobe.tolist(), k.tolist())):
        rows = np.where((nprobe == np_) & (k == k_))[0]
        d, l = ix.search(q[rows], k_, form=mv.FORM_FAST, nprobe=np_, rerank=rerank, coarse_fp32=True)
        dist[rows, :k_] = d
        lab[rows, :k_] = l
    return dist, lab


def test_batch_equals_per_query_searches(mv):
    ix, q = _index(mv)
    nprobe = RNG.integers(1, 40, size=len(q)).astype(np.int32)
    k = RNG.choice([1, 10, 50], size=len(q)).astype(np.int32)
    rerank = 64
    d, l = ix.search_batch(q, nprobe, k, rerank=rerank, coarse_fp32=True)
    rd, rl = _reference_rows(mv, ix, q, nprobe, k, rerank)
    assert np.array_equal(l, rl)
    assert np.array_equal(d, rd)


def test_plan_graph_and_tuner_keep_results(mv):
    ix, q = _index(mv)
    nprobe = RNG.integers(1, 60, size=len(q)).astype(np.int32)
    k = RNG.choice([1, 10, 100], size=len(q)).astype(np.int32)
    rd, rl = ix.search_batch(q, nprobe, k, rerank=128, coarse_fp32=True)
    plan = mv.IVFPQBatchPlan(ix, 512, int(nprobe.max()), int(k.max()), rerank=128, coarse_fp32=True)
    plan.set_queries(q, nprobe, k)
    plan.run(len(q), use_graph=False)
    d0, l0 = plan.results(len(q))
    assert np.array_equal(l0, rl) and np.array_equal(d0, rd)
    plan.run(len(q), use_graph=True)
    plan.run(len(q), use_graph=True)  # replay of the captured graph
    d1, l1 = plan.results(len(q))
    assert np.array_equal(l1, rl) and np.array_equal(d1, rd)
    cfg = plan.tune(len(q))
    assert cfg["scan_threads"] in (128, 256, 512) and cfg["best_ms"] > 0
    plan.run(len(q), use_graph=True)
    d2, l2 = plan.results(len(q))
    assert np.array_equal(l2, rl) and np.array_equal(d2, rd)
    # a smaller batch reuses the plan with its own graph
    plan.set_queries(q[:77], nprobe[:77], k[:77])
    plan.run(77, use_graph=True)
    d3, l3 = plan.results(77)
    assert np.array_equal(l3, rl[:77]) and np.array_equal(d3, rd[:77])


def test_batch_fused_coarse_and_argument_checks(mv):
    ix, q = _index(mv)
    nprobe = RNG.integers(1, 20, size=len(q)).astype(np.int32)
    k = np.full(len(q), 10, np.int32)
    d, l = ix.search_batch(q, nprobe, k, rerank=40)  # BF16 coarse (fused top-k GEMM)
    assert (l >= 0).all() and np.isfinite(d).all()
    with pytest.raises(mv.MojoVecGPUError):
        ix.search_batch(q[:4], np.array([0, 1, 2, 3], np.int32), k[:4], rerank=40)


def test_batch_certified_rerank_per_query_k(mv):
    """k <= 32 takes the certified rerank (BF16 prescreen) with per-query k:
    the batch must still equal per-query searches, and the prescreen-free
    rerank of the same batch."""
    ix, q = _index(mv)
    nprobe = RNG.integers(1, 30, size=len(q)).astype(np.int32)
    k = RNG.choice([1, 5, 20, 32], size=len(q)).astype(np.int32)
    d, l = ix.search_batch(q, nprobe, k, rerank=96, coarse_fp32=True)
    rd, rl = _reference_rows(mv, ix, q, nprobe, k, 96)
    assert np.array_equal(l, rl)
    assert np.array_equal(d, rd)
