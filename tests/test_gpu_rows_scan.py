"""Two-kernel fast IVF-PQ scan (lut 7, and the default where a query's
candidates are few enough): per-candidate distance rows, then a per-query
select (k_ivfpq_rows.cu).

Its candidates' distance words are computed with the single-kernel FP32
scan's arithmetic and it selects the R smallest (distance, CSR position)
keys, so it must return the single-kernel scan's bits (lut 2): with and without
the exact rerank, shortlists up to 256 (streaming warp select) and above
(histogram warp select), both metrics, FP16 and FP32 codebooks, the
exclusion filter, and per-query nprobe in a batch plan."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(64, 8), (128, 16), (96, 24), (80, 16), (128, 32)]  # (80, 16): dsub 5, FP32 codebook


def _index(mv, d, M, metric, n=8000, nlist=48, seed=0, nq=64):
    rng = np.random.default_rng(seed)
    cent = rng.standard_normal((32, d)).astype(np.float32) * 3
    base = (cent[rng.integers(0, 32, n)] + rng.standard_normal((n, d))).astype(np.float32)
    q = (cent[rng.integers(0, 32, nq)] + rng.standard_normal((nq, d))).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base, niter_coarse=4, niter_pq=4)
    g.add(base)
    return g, base, q


def _same(a, b):
    return np.array_equal(a[1], b[1]) and np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", CASES)
def test_rows_scan_equals_single_kernel_scan(mv, d, M, metric):
    g, base, q = _index(mv, d, M, metric)
    for k, rerank, nprobe in ((10, 64, 4), (10, 0, 4), (300, 0, 6), (10, 400, 6)):
        a = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=7)
        b = g.search(q, k, form=mv.FORM_FAST, nprobe=nprobe, rerank=rerank, lut=2)
        assert _same(a, b), (k, rerank, nprobe)
    flt = np.zeros(base.shape[0], np.uint8)
    flt[1::4] = 1
    a = g.search(q, 20, form=mv.FORM_FAST, nprobe=5, rerank=80, filter=flt, lut=7)
    b = g.search(q, 20, form=mv.FORM_FAST, nprobe=5, rerank=80, filter=flt, lut=2)
    assert _same(a, b)
    assert not np.isin(a[1][a[1] >= 0], np.nonzero(flt)[0]).any()


def test_rows_scan_in_a_batch_plan(mv):
    """Per-query nprobe and k: the plan with the two-kernel scan returns the
    bits of the same plan with the single-kernel scan."""
    g, base, q = _index(mv, 64, 8, 0, nq=200, seed=4)
    rng = np.random.default_rng(9)
    nprobe = rng.integers(1, 9, size=q.shape[0]).astype(np.int32)
    k = rng.choice(np.array([1, 5, 10], np.int32), size=q.shape[0])
    out = []
    for lut in (7, 2):
        plan = mv.IVFPQBatchPlan(g, q.shape[0], 8, 10, rerank=40, lut=lut)
        plan.set_queries(q, nprobe, k)
        plan.run(q.shape[0], use_graph=False)
        out.append(plan.results(q.shape[0]))
    assert _same(out[0], out[1])
