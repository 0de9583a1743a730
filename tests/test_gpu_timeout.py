"""Failure detection on the device: a bounded wait that expires.

Every wait inside the tensor-core kernels (TMA stage landed, accumulator
ready, accumulator free) is bounded. When one gives up the kernel records
the error flag, stops issuing work, waits (with the full limit) for the
copies and MMAs it already issued, frees its tensor memory and returns; the
call returns MV_ERR_TIMEOUT and the context stays usable. The context's
wait limit set to 0 makes every pipeline wait that is not already satisfied
give up at once, so the path runs without any broken kernel: no GPU fault,
no hang. After the limit is restored, the same context must give the same
results as before, and the plain form's results must still equal the
oracle's.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_expired_wait_returns_timeout_and_context_recovers(mv, orc):
    from mojovec_gb300 import synth

    ctx = mv.Context(0)
    base, q = synth.sift_like(20000, d=96, n_centers=64, nq=64, seed=77)
    x, y = base[:300], base[300:1000]
    flat = mv.IndexFlat(96, mv.METRIC_L2, ctx=ctx)
    flat.add(base)
    dm = mv.distance_matrix(x, y, precision=1, ctx=ctx)  # k_umma_dist
    fd, fl = flat.search(q, 10, form=mv.FORM_FAST, rerank=40)  # k_umma_topk
    pd, pl = flat.search(q, 10)  # certified plain form (k_umma_topk + certificate)

    ctx.set_wait_limit(0)
    try:
        calls = (lambda: mv.distance_matrix(x, y, precision=1, ctx=ctx),
                 lambda: flat.search(q, 10, form=mv.FORM_FAST, rerank=40),
                 lambda: flat.search(q, 10))
        for call in calls:
            with pytest.raises(mv.MojoVecGPUError) as e:
                call()
            assert e.value.code == mv._lib.MV_ERR_TIMEOUT, str(e.value)
    finally:
        ctx.set_wait_limit(None)

    assert np.array_equal(mv.distance_matrix(x, y, precision=1, ctx=ctx), dm)
    fd2, fl2 = flat.search(q, 10, form=mv.FORM_FAST, rerank=40)
    assert np.array_equal(fl2, fl) and np.array_equal(fd2, fd)
    pd2, pl2 = flat.search(q, 10)
    od, ol = orc.flat_search(base, q, 10)
    assert np.array_equal(pl2, ol) and np.array_equal(pd2.view(np.uint32), od.view(np.uint32))
    assert np.array_equal(pl2, pl)
