"""The host-buffer IVF-PQ search runs batches of 8 192 queries or more as two
halves on two streams (their copies overlap the other half's kernels). Its
results must be the bits of the same search over device buffers in one
launch sequence, for the plain and the fast form, both metrics, with and
without the exclusion filter, and the plain form must equal the oracle; and
a query's results must not depend on the batch it is searched in (one
device-buffer search of 9 001 queries against slices of 3 000, on the
library's stream and on the caller's)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", [0, 1])
def test_split_host_search_equals_device_search(mv, orc, metric):
    import torch

    from mojovec_gb300 import synth

    base, q = synth.sift_like(20000, d=32, n_centers=64, nq=9001, seed=21)
    g = mv.IndexIVFPQ(32, 64, 8, metric)
    g.train(base[:8000], niter_coarse=4, niter_pq=4)
    g.add(base)
    k = 12
    dq = torch.from_numpy(q).cuda()
    for opts in (dict(form=mv.FORM_PLAIN, nprobe=4), dict(form=mv.FORM_FAST, nprobe=4, rerank=48)):
        hd, hl = g.search(q, k, **opts)
        dd = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
        dl = torch.empty((q.shape[0], k), dtype=torch.int64, device="cuda")
        g.search_device(dq.data_ptr(), q.shape[0], k, dd.data_ptr(), dl.data_ptr(), **opts)
        torch.cuda.synchronize()
        assert np.array_equal(hl, dl.cpu().numpy())
        assert np.array_equal(hd.view(np.uint32), dd.cpu().numpy().view(np.uint32))
    # plain form against the oracle over the same codebooks and lists
    ref = orc.IVFPQ(32, 64, 8, metric)
    ref.set_codebooks(*g.codebooks())
    off, ids, codes = g.lists()
    ref.set_lists(off, ids, codes)
    rd, rl = ref.search(q, k, 4)
    hd, hl = g.search(q, k, form=mv.FORM_PLAIN, nprobe=4)
    assert np.array_equal(hl, rl)
    assert np.array_equal(hd.view(np.uint32), rd.view(np.uint32))
    # exclusion filter: a filtered id never appears, in both halves
    flt = np.zeros(base.shape[0], np.uint8)
    flt[::3] = 1
    fd, fl = g.search(q, k, form=mv.FORM_FAST, nprobe=4, rerank=48, filter=flt)
    assert not np.isin(fl[fl >= 0], np.nonzero(flt)[0]).any()


@pytest.mark.parametrize("metric", [0, 1])
def test_split_device_search_equals_sliced_searches(mv, metric):
    import torch

    from mojovec_gb300 import synth

    base, q = synth.sift_like(20000, d=32, n_centers=64, nq=9001, seed=22)
    g = mv.IndexIVFPQ(32, 64, 8, metric)
    g.train(base[:8000], niter_coarse=4, niter_pq=4)
    g.add(base)
    k = 10
    n = q.shape[0]
    dq = torch.from_numpy(q).cuda()
    for opts in (dict(form=mv.FORM_PLAIN, nprobe=4), dict(form=mv.FORM_FAST, nprobe=4, rerank=64)):
        # unsplit reference: three slices of 3 000 queries
        rd = torch.empty((n, k), dtype=torch.float32, device="cuda")
        rl = torch.empty((n, k), dtype=torch.int64, device="cuda")
        for q0 in range(0, n, 3000):
            m = min(3000, n - q0)
            g.search_device(dq[q0:].data_ptr(), m, k, rd[q0:].data_ptr(), rl[q0:].data_ptr(), **opts)
        torch.cuda.synchronize()
        for use_stream in (False, True):
            dd = torch.full((n, k), -7.0, dtype=torch.float32, device="cuda")
            dl = torch.full((n, k), -7, dtype=torch.int64, device="cuda")
            st = torch.cuda.current_stream().cuda_stream if use_stream else 0
            g.search_device(dq.data_ptr(), n, k, dd.data_ptr(), dl.data_ptr(), stream=st, **opts)
            # on the caller's stream the results are ordered before the copies
            got_l, got_d = dl.cpu().numpy(), dd.cpu().numpy()
            assert np.array_equal(got_l, rl.cpu().numpy()), (opts, use_stream)
            assert np.array_equal(got_d.view(np.uint32), rd.cpu().numpy().view(np.uint32)), (opts, use_stream)
