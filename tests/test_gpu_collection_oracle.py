"""The managed collection's query path against the oracle's restatement of
api/collection_ivfpq.mojo (oracle.CollectionIVFPQ): for the l2, cosine and
ip metrics, with user ids that are neither sequential nor small, in two add
batches (the first one auto-trains), the plain-form collection query returns
the oracle's user ids and distance bits (1 - d for cosine and ip, -1 and the
index's fill distance for empty slots)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", ["l2", "cosine", "ip"])
def test_collection_query_matches_oracle(mv, orc, metric):
    from mojovec_gb300 import synth
    from mojovec_gb300.collection import IVFPQCollection

    base, q = synth.sift_like(3000, d=32, n_centers=48, nq=40, seed=11)
    if metric == "ip":
        base = base / 64.0
        q = q / 64.0
    rng = np.random.default_rng(3)
    ids = rng.choice(10**12, size=base.shape[0], replace=False).astype(np.int64)
    nlist, M, nprobe, k = 24, 8, 5, 12
    gpu = IVFPQCollection(32, nlist=nlist, pq_subvectors=M, nprobe=nprobe, metric=metric)
    ref = orc.CollectionIVFPQ(32, nlist, M, nprobe, metric)
    half = 1800  # the first batch trains (at least max(nlist, 256) rows)
    for lo, hi in ((0, half), (half, base.shape[0])):
        gpu.add(ids[lo:hi].tolist(), base[lo:hi])
        ref.add(ids[lo:hi].tolist(), base[lo:hi])
    got = gpu.query(q, n_results=k)
    want_ids, want_d = ref.query(q, n_results=k)
    assert got["ids"] == want_ids
    gd = np.asarray(got["distances"], np.float32)
    wd = np.asarray(want_d, np.float32)
    assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32))
    # more results than candidates: empty slots keep -1 and the fill distance
    got = gpu.query(q[:3], n_results=2048)
    want_ids, want_d = ref.query(q[:3], n_results=2048)
    assert got["ids"] == want_ids
    assert np.array_equal(np.asarray(got["distances"], np.float32).view(np.uint32),
                          np.asarray(want_d, np.float32).view(np.uint32))
