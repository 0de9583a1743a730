"""Host-side merge of per-shard search results.

Every query over an index is independent and the base partitions cleanly:
Flat and SQ8 shard by row ranges, IVF-PQ and IVF-Flat by list ranges (each
shard holds the lists of its range, every shard keeps all centroids, so the
coarse step picks the same probes everywhere). Each shard returns its local
top-k with global ids; one gather and this k-way merge give the unsharded
result, with the canonical tie rule of every search here: ascending
(distance, id) for L2, descending inner product then ascending id for IP
(index/index_flat.mojo:260-325 and index/index_ivf_pq.mojo:326-360 keep the
k smallest keys; the tie rule is the library's canonical order). Empty slots
(label -1) sort after every result.

The library runs one index per GPU process (replicas); this merge is the
exchange step a sharded deployment adds on the host.
"""

from __future__ import annotations

import numpy as np

from ._lib import METRIC_IP, METRIC_L2


def shard_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous [lo, hi) share of n items (rows or lists) for rank."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def merge_topk(distances, labels, k: int, metric: int = METRIC_L2, fill_distance: float = 0.0):
    """Merge per-shard (nq, k_i) results into the global (nq, k) top-k.

    distances / labels: sequences of per-shard arrays (float32 distances as
    the searches return them, int64 global labels, -1 for an empty slot).
    fill_distance is written beside label -1 when fewer than k results exist
    (0.0 for Flat / SQ8, 1e38 for IVF-PQ and IVF-Flat).
    """
    if metric not in (METRIC_L2, METRIC_IP):
        raise ValueError("metric must be METRIC_L2 or METRIC_IP")
    if len(distances) != len(labels) or not distances:
        raise ValueError("one distance and one label array per shard")
    d = np.concatenate([np.asarray(x, np.float32) for x in distances], axis=1)
    lab = np.concatenate([np.asarray(x, np.int64) for x in labels], axis=1)
    if d.shape != lab.shape:
        raise ValueError("distance and label arrays differ in shape")
    nq = d.shape[0]
    key = d.astype(np.float64) if metric == METRIC_L2 else -d.astype(np.float64)
    empty = lab < 0
    key = np.where(empty, np.inf, key)
    idk = np.where(empty, np.iinfo(np.int64).max, lab)
    order = np.lexsort((idk, key), axis=1)  # last key primary: distance, then id
    take = order[:, :k]
    out_d = np.take_along_axis(d, take, axis=1)
    out_l = np.take_along_axis(lab, take, axis=1)
    if take.shape[1] < k:  # fewer candidates than k over all shards
        pad = k - take.shape[1]
        out_d = np.concatenate([out_d, np.full((nq, pad), fill_distance, np.float32)], axis=1)
        out_l = np.concatenate([out_l, np.full((nq, pad), -1, np.int64)], axis=1)
    gone = out_l < 0
    out_d = np.where(gone, np.float32(fill_distance), out_d).astype(np.float32)
    return out_d, out_l
