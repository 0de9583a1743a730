"""Bank-rotated fixed-point table scan of the fast IVF-PQ form.

The rotated-table fast scan (lut 6) keeps each query's
table as 32-bit fixed-point entries in a bank-rotated layout and stages
every candidate's distance in its own slot before a range select
(k_ivfpq_rt.cu). Its approximate distances must agree with the FP32-table
scan (lut 2) within FP32 rounding, for every pass width (M <= 8, <= 16,
<= 32) with unused slots (M 12, 24), both metrics and both codebook widths
(dsub 4 and 8). With rerank 0 and k above the candidate count the result
rows hold every probed candidate, so the comparison is per (query, id).
Lists longer than the staging area run in chunks with the R kept keys
carried between them.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [  # (d, M): pass width, slots in use, code-load class, dsub
    (64, 8),     # S 8, uint2 loads, dsub 8
    (32, 8),     # S 8, dsub 4
    (48, 12),    # S 16 with 4 zero slots, 4-byte loads, dsub 4
    (128, 16),   # S 16, uint4 loads, dsub 8
    (96, 24),    # S 32 with 8 zero slots, uint2 loads, dsub 4
    (128, 32),   # S 32, dsub 4
]


def _index(mv, d, M, metric, n=6000, nlist=64, seed=0, nq=40):
    rng = np.random.default_rng(seed)
    cent = rng.standard_normal((32, d)).astype(np.float32) * 3
    base = (cent[rng.integers(0, 32, n)] + rng.standard_normal((n, d))).astype(np.float32)
    q = (cent[rng.integers(0, 32, nq)] + rng.standard_normal((nq, d))).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base, niter_coarse=4, niter_pq=4)
    g.add(base)
    return g, base, q


def _by_id(dist, lab):
    return [{int(i): float(v) for i, v in zip(lr, dr) if i >= 0} for dr, lr in zip(dist, lab)]


def _close(a, b):
    ids = sorted(a)
    x = np.array([a[i] for i in ids])
    y = np.array([b[i] for i in ids])
    scale = max(np.abs(y).max(), 1e-6)
    return np.allclose(x, y, rtol=2e-5, atol=2e-5 * scale)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", CASES)
def test_rt_tables_match_fp32_tables(mv, d, M, metric):
    g, base, q = _index(mv, d, M, metric)
    k = 2048  # above nearly every query's candidate count at nprobe 3
    rd, rl = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=6)
    fd, fl = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=2)
    complete = (rl == -1).any(axis=1) & (fl == -1).any(axis=1)  # every candidate returned
    assert complete.mean() >= 0.75
    for a, b in zip(_by_id(rd[complete], rl[complete]), _by_id(fd[complete], fl[complete])):
        assert a.keys() == b.keys()  # the same candidates, every one kept
        assert _close(a, b)
    # the answer rows are sorted by distance (IP rows hold the inner product)
    for dr, lr in zip(rd, rl):
        v = dr[lr >= 0] * (1.0 if metric == 0 else -1.0)
        assert np.all(v[:-1] <= v[1:])
    # order-independent sums: identical bits on a repeat and by default
    rd2, rl2 = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=6)
    assert np.array_equal(rl2, rl) and np.array_equal(rd2.view(np.uint32), rd.view(np.uint32))


@pytest.mark.parametrize("metric", [0, 1])
def test_rt_chunks_of_long_lists(mv, metric):
    """Four lists of about 10 000 rows, two probed: 20 000 candidates per
    query run in chunks of at most 8192. The shortlist of 256 equals the
    FP32-table scan's on the ids that are not at a rounding tie, and a query
    gets the same bits alone and in the batch."""
    g, base, q = _index(mv, 64, 8, metric, n=40000, nlist=4, seed=3, nq=24)
    a = g.search(q, 256, form=mv.FORM_FAST, nprobe=2, lut=6)
    b = g.search(q, 256, form=mv.FORM_FAST, nprobe=2, lut=2)
    assert (a[1] >= 0).all()
    overlap = np.mean([len(set(x) & set(y)) / 256 for x, y in zip(a[1], b[1])])
    assert overlap >= 0.99, overlap
    for x, y in zip(a[0], b[0]):
        scale = max(np.abs(y).max(), 1e-6)
        assert np.allclose(x, y, rtol=2e-5, atol=2e-5 * scale)
    for i in (0, 7, 23):
        s = g.search(q[i:i + 1], 256, form=mv.FORM_FAST, nprobe=2, lut=6)
        assert np.array_equal(s[1][0], a[1][i])
        assert np.array_equal(s[0][0].view(np.uint32), a[0][i].view(np.uint32))


def test_rt_headline_shape_with_rerank(mv):
    """The headline operating point's shape (M 16, dsub 8): results after the
    exact rerank equal those of the FP32-table scan on nearly every query."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(60000, d=128, n_centers=128, nq=300, seed=5)
    g = mv.IndexIVFPQ(128, 128, 16)
    g.train(base[:30000], niter_coarse=5, niter_pq=5)
    g.add(base)
    a = g.search(q, 10, form=mv.FORM_FAST, nprobe=8, rerank=256, lut=6)
    b = g.search(q, 10, form=mv.FORM_FAST, nprobe=8, rerank=256, lut=2)
    same = np.mean([np.array_equal(x, y) for x, y in zip(a[1], b[1])])
    assert same >= 0.98, same


def test_rt_unsupported_shape_is_refused(mv):
    g, base, q = _index(mv, 80, 16, 0, n=3000)  # dsub 5: no FP16 codebook
    with pytest.raises(Exception):
        g.search(q, 10, form=mv.FORM_FAST, nprobe=3, lut=6)
    d, l = g.search(q, 10, form=mv.FORM_FAST, nprobe=3)  # the default scan serves it
    assert (l >= 0).all()
