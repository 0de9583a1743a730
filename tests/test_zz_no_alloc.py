"""The allocation-free IVF-PQ search (mv_ivfpq_search_noalloc).

Callers that cannot allocate device memory while they search (a server whose
GPU memory all belongs to its own pool, or a host loop that must not absorb
cudaFree's device-wide synchronisation) use this entry point with their own
device buffers; its scratch is a fixed array inside the library. This test
calls it through the C ABI twice in a row (the second call finds the first
call's scratch contents) and requires the same ids and distance bits as the
allocating entry point, mv_ivfpq_search. It lives in its own file so that
pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_search_matches_allocating_search(mv):
    torch = pytest.importorskip("torch")
    from mojovec_gb300 import _lib, synth

    lib = _lib.load()
    d, nlist, M, k = 64, 4096, 8, 10
    base, q = synth.sift_like(60000, d=d, n_centers=128, nq=2500, seed=19)
    ix = mv.IndexIVFPQ(d, nlist, M)
    ix.train(base[:30000], niter_coarse=3, niter_pq=3)
    ix.add(base)
    ix.nprobe = 12
    ref_d, ref_l = ix.search(q, k)  # allocating entry point (host buffers)

    dq = torch.from_numpy(q).cuda()
    dd = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    dl = torch.empty((q.shape[0], k), dtype=torch.int64, device="cuda")
    for _ in range(2):
        dd.fill_(-7.0)
        dl.fill_(-7)
        torch.cuda.synchronize()
        st = lib.mv_ivfpq_search_noalloc(ix._h, ctypes.c_void_p(dq.data_ptr()), q.shape[0], k, 0,
                                         ctypes.c_void_p(dd.data_ptr()),
                                         ctypes.c_void_p(dl.data_ptr()), None)
        torch.cuda.synchronize()
        assert st == 0, _lib.last_error()
        assert np.array_equal(dl.cpu().numpy(), ref_l)
        assert np.array_equal(dd.cpu().numpy(), ref_d)


def test_noalloc_rejects_bad_arguments(mv):
    from mojovec_gb300 import _lib

    lib = _lib.load()
    ix = mv.IndexIVFPQ(16, 8, 4)
    assert lib.mv_ivfpq_search_noalloc(None, None, 1, 10, 0, None, None, None) == _lib.MV_ERR_ARG
    assert lib.mv_ivfpq_search_noalloc(ix._h, ctypes.c_void_p(16), 1, 0, 0, ctypes.c_void_p(16),
                                       ctypes.c_void_p(16), None) == _lib.MV_ERR_ARG
