"""The allocation-free IVF-PQ search (mv_ivfpq_search_noalloc).

Callers that cannot allocate device memory while they search (a server whose
GPU memory all belongs to its own pool, or a host loop that must not absorb
cudaFree's device-wide synchronisation) use this entry point with their own
device buffers; its scratch is a fixed array inside the library. These tests
call it through the C ABI twice in a row (the second call finds the first
call's scratch contents) and require the same ids and distance bits as the
allocating entry point, mv_ivfpq_search, for both metrics; they also check
that the device memory in use does not change across a call, and that an
untrained index gives the reference's empty results (1e38 / -1). The file
is named so that pytest collects it last.

The scratch array holds 8 MiB. One query needs at most nlist * 4 bytes plus
12 bytes per probe, and nlist is capped at 1,000,000 (index_ivf_pq.mojo:52-59),
so every valid index fits; larger batches are split to fit.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, ix, dq, n, k, nprobe, dd, dl):
    return lib.mv_ivfpq_search_noalloc(ix._h, ctypes.c_void_p(dq.data_ptr()), n, k, nprobe,
                                       ctypes.c_void_p(dd.data_ptr()),
                                       ctypes.c_void_p(dl.data_ptr()), None)


@pytest.mark.parametrize("metric", [0, 1])
def test_noalloc_search_matches_allocating_search(mv, metric):
    torch = pytest.importorskip("torch")
    from mojovec_gb300 import _lib, synth

    lib = _lib.load()
    d, nlist, M, k = 64, 4096, 8, 10
    base, q = synth.sift_like(60000, d=d, n_centers=128, nq=2500, seed=19)
    ix = mv.IndexIVFPQ(d, nlist, M, metric)
    ix.train(base[:30000], niter_coarse=3, niter_pq=3)
    ix.add(base)
    ix.nprobe = 12
    ref_d, ref_l = ix.search(q, k)  # allocating entry point (host buffers)

    dq = torch.from_numpy(q).cuda()
    dd = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    dl = torch.empty((q.shape[0], k), dtype=torch.int64, device="cuda")
    for call in range(2):
        dd.fill_(-7.0)
        dl.fill_(-7)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        st = _call(lib, ix, dq, q.shape[0], k, 0, dd, dl)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert st == 0, _lib.last_error()
        if call == 1:  # the first call on a device may load the library's module
            assert free1 == free0, f"device memory in use changed by {free0 - free1} bytes"
        assert np.array_equal(dl.cpu().numpy(), ref_l)
        assert np.array_equal(dd.cpu().numpy(), ref_d)


def test_noalloc_untrained_index_fills_empty_results(mv):
    torch = pytest.importorskip("torch")
    from mojovec_gb300 import _lib

    lib = _lib.load()
    ix = mv.IndexIVFPQ(16, 8, 4)
    dq = torch.zeros((3, 16), dtype=torch.float32, device="cuda")
    dd = torch.zeros((3, 5), dtype=torch.float32, device="cuda")
    dl = torch.zeros((3, 5), dtype=torch.int64, device="cuda")
    assert _call(lib, ix, dq, 3, 5, 0, dd, dl) == 0, _lib.last_error()
    torch.cuda.synchronize()
    assert (dl.cpu().numpy() == -1).all()
    assert (dd.cpu().numpy() == np.float32(1e38)).all()


def test_noalloc_rejects_bad_arguments(mv):
    from mojovec_gb300 import _lib

    lib = _lib.load()
    ix = mv.IndexIVFPQ(16, 8, 4)
    assert lib.mv_ivfpq_search_noalloc(None, None, 1, 10, 0, None, None, None) == _lib.MV_ERR_ARG
    assert lib.mv_ivfpq_search_noalloc(ix._h, ctypes.c_void_p(16), 1, 0, 0, ctypes.c_void_p(16),
                                       ctypes.c_void_p(16), None) == _lib.MV_ERR_ARG
    assert "n_results" in _lib.last_error()
    assert lib.mv_ivfpq_search_noalloc(ix._h, None, -1, 10, 0, None, None, None) == _lib.MV_ERR_ARG
    assert "negative" in _lib.last_error()
