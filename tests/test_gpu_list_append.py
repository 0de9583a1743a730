"""List append on the device (storage/inverted_lists.mojo:162-186,
index_ivf_pq.mojo:199-213): the rebuilt CSR equals a stable sort of the
entries by list number, old entries first, new ones in input order. A NaN
row goes to list 0: the k = 1 coarse heap takes the first centroid
unconditionally and no NaN distance replaces it (index/index_flat.mojo:
292-310).

Rows and centroids are small integers, so every FP32 distance is exact in
any summation order and numpy's first-minimum argmin is the reference's
strict-`<` rule. Cases cover both metrics, two appends, the shared-memory
and the global bucket counts (nlist above 24575), and the tile growth that
keeps the tile x bucket table bounded (4.7M rows x 30000 lists)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _assign(x, c, metric, mv):
    x64, c64 = x.astype(np.float64), c.astype(np.float64)
    out = np.empty(len(x), np.int64)
    for r0 in range(0, len(x), 512):
        xb = x64[r0:r0 + 512]
        ip = xb @ c64.T
        if metric == mv.METRIC_L2:
            score = (xb * xb).sum(1)[:, None] + (c64 * c64).sum(1)[None, :] - 2 * ip
        else:
            score = -ip
        out[r0:r0 + 512] = score.argmin(1)
    out[np.isnan(x).any(1)] = 0
    return out


def _index(mv, d, nlist, M, metric, seed):
    rng = np.random.default_rng(seed)
    cent = rng.integers(0, 16, size=(nlist, d)).astype(np.float32)
    pq = rng.standard_normal((M, 256, d // M)).astype(np.float32)
    ix = mv.IndexIVFPQ(d, nlist, M, metric)
    ix.set_codebooks(cent, pq)
    return ix, cent


def _expected_lists(assign_all, nlist):
    keep = assign_all >= 0
    ids = np.flatnonzero(keep)
    order = np.argsort(assign_all[keep], kind="stable")
    off = np.zeros(nlist + 1, np.int64)
    np.add.at(off, assign_all[keep] + 1, 1)
    return np.cumsum(off), ids[order]


@pytest.mark.parametrize("metric_name", ["l2", "ip"])
def test_two_appends_equal_stable_sort(mv, metric_name):
    metric = mv.METRIC_L2 if metric_name == "l2" else mv.METRIC_IP
    d, nlist, M = 8, 300, 4
    ix, cent = _index(mv, d, nlist, M, metric, 1)
    rng = np.random.default_rng(2)
    a = rng.integers(0, 16, size=(20000, d)).astype(np.float32)
    b = rng.integers(0, 16, size=(15000, d)).astype(np.float32)
    b[[5, 777, 14999]] = np.nan
    ix.add(a)
    ix.add(b)
    assert ix.ntotal == 35000
    off, ids, codes = ix.lists()
    e_off, e_ids = _expected_lists(_assign(np.vstack([a, b]), cent, metric, mv), nlist)
    assert np.array_equal(off, e_off)
    assert np.array_equal(ids, e_ids)
    # codes travel with their ids: re-adding the same rows alone gives the same code per id
    ix2, _ = _index(mv, d, nlist, M, metric, 1)
    ix2.add(np.vstack([a, b]))
    off2, ids2, codes2 = ix2.lists()
    assert np.array_equal(off2, off) and np.array_equal(ids2, ids) and np.array_equal(codes2, codes)


def test_global_bucket_counts_large_nlist(mv):
    d, nlist, M = 8, 30000, 2
    ix, cent = _index(mv, d, nlist, M, mv.METRIC_L2, 3)
    x = np.random.default_rng(4).integers(0, 16, size=(60000, d)).astype(np.float32)
    ix.add(x[:10000])
    ix.add(x[10000:])
    off, ids, _ = ix.lists()
    e_off, e_ids = _expected_lists(_assign(x, cent, mv.METRIC_L2, mv), nlist)
    assert np.array_equal(off, e_off) and np.array_equal(ids, e_ids)


def test_tile_growth_many_rows(mv):
    d, nlist, M = 8, 30000, 2
    n = 4_700_000
    ix, cent = _index(mv, d, nlist, M, mv.METRIC_L2, 5)
    x = np.random.default_rng(6).integers(0, 16, size=(n, d)).astype(np.float32)
    ix.add(x)
    off, ids, _ = ix.lists()
    assert off[-1] == n and ix.ntotal == n
    assert np.array_equal(np.sort(ids), np.arange(n))
    lists = np.repeat(np.arange(nlist), np.diff(off))
    # input order inside every list
    same = lists[1:] == lists[:-1]
    assert (np.diff(ids)[same] > 0).all()
    # the list of a sample of rows is their nearest centroid
    where = np.empty(n, np.int64)
    where[ids] = lists
    sample = np.random.default_rng(7).choice(n, 3000, replace=False)
    assert np.array_equal(where[sample], _assign(x[sample], cent, mv.METRIC_L2, mv))
