"""Bank-rotated fixed-point tables of the fast IVF-PQ scan.

With lut = 3 the fast scan keeps each query's tables in a bank-rotated
layout with 32-bit fixed-point entries (k_ivfpq_scan_fast, MODE 8/16/32).
Its approximate distances must agree with the FP32 tables in the plain
layout (lut = 2) to within FP32 rounding, for every pass width (M <= 8, <= 16,
<= 32, and two passes above 32), with unused slots (M = 12, 24, 48), every
code-load width (M a multiple of 16, 8 or only 4), FP16 and FP32 codebooks
(dsub 4 / 8 read the FP16 copy, other dsub the FP32 one) and both metrics.
With rerank 0 and k above the candidate count the result rows hold every
probed candidate, so the comparison is per (query, id). Integer sums do not
depend on the summation order, so repeated searches, launch shapes (the
persistent batch scan) and filters cannot change a distance bit.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [  # (d, M): pass width, slots in use, code-load class, dsub
    (64, 8),     # S 8, uint2 loads, dsub 8 (FP16 codebook)
    (32, 8),     # S 8, dsub 4
    (96, 12),    # S 16 with 4 zero slots, 4-byte loads, dsub 8
    (128, 16),   # S 16, uint4 loads
    (80, 16),    # S 16, dsub 5 (FP32 codebook)
    (96, 24),    # S 32 with 8 zero slots, uint2 loads, dsub 4
    (128, 32),   # S 32, dsub 4
    (96, 48),    # two passes of 32, the second with 16 zero slots, dsub 2
    (128, 64),   # two passes, dsub 2
]


def _index(mv, d, M, metric, n=6000, nlist=64, seed=0):
    rng = np.random.default_rng(seed)
    cent = rng.standard_normal((32, d)).astype(np.float32) * 3
    base = (cent[rng.integers(0, 32, n)] + rng.standard_normal((n, d))).astype(np.float32)
    q = (cent[rng.integers(0, 32, 40)] + rng.standard_normal((40, d))).astype(np.float32)
    g = mv.IndexIVFPQ(d, nlist, M, metric)
    g.train(base, niter_coarse=4, niter_pq=4)
    g.add(base)
    return g, base, q


def _by_id(dist, lab):
    return [{int(i): float(v) for i, v in zip(lr, dr) if i >= 0} for dr, lr in zip(dist, lab)]


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("d,M", CASES)
def test_rotated_tables_match_fp32_tables(mv, d, M, metric):
    g, base, q = _index(mv, d, M, metric)
    k = 2048  # above nearly every query's candidate count at nprobe 3
    rd, rl = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=3)
    fd, fl = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=2)
    complete = (rl == -1).any(axis=1) & (fl == -1).any(axis=1)  # every candidate returned
    assert complete.mean() >= 0.75
    for a, b in zip(_by_id(rd[complete], rl[complete]), _by_id(fd[complete], fl[complete])):
        assert a.keys() == b.keys()  # the same candidates, every one kept
        ids = sorted(a)
        x = np.array([a[i] for i in ids])
        y = np.array([b[i] for i in ids])
        scale = max(np.abs(y).max(), 1e-6)
        assert np.allclose(x, y, rtol=2e-5, atol=2e-5 * scale)
    # order-independent sums: identical bits on a repeat
    rd2, rl2 = g.search(q, k, form=mv.FORM_FAST, nprobe=3, lut=3)
    assert np.array_equal(rl2, rl) and np.array_equal(rd2.view(np.uint32), rd.view(np.uint32))


def test_rotated_tables_recall_with_rerank(mv):
    """The headline operating point's shape (M 16, dsub 8): results after the
    exact rerank equal those of the FP32-table scan on nearly every query."""
    from mojovec_gb300 import synth

    base, q = synth.sift_like(60000, d=128, n_centers=128, nq=300, seed=5)
    g = mv.IndexIVFPQ(128, 128, 16)
    g.train(base[:30000], niter_coarse=5, niter_pq=5)
    g.add(base)
    a = g.search(q, 10, form=mv.FORM_FAST, nprobe=8, rerank=256, lut=3)
    b = g.search(q, 10, form=mv.FORM_FAST, nprobe=8, rerank=256, lut=2)
    same = np.mean([np.array_equal(x, y) for x, y in zip(a[1], b[1])])
    assert same >= 0.98, same

