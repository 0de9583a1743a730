"""Sharded search, merged on the host (mojovec_gb300.shard), on CPU.

world_size-2 gloo ranks each search their share of the base with the
oracle and return their local top-k with global ids; rank 0 gathers the
shards and merges them. The merged result must equal the unsharded search
bit for bit: Flat split by row ranges, IVF-PQ split by list ranges (every
rank keeps all centroids and codebooks, so the coarse step picks the same
probes). The merge itself is also checked against a full sort on random
splits with ties and empty slots, for both metrics."""

import os
import socket

import numpy as np
import pytest

from mojovec_gb300 import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _data(seed=0, n=3000, d=24, nq=30):
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 16, size=(n, d)).astype(np.float32)  # many equal distances
    q = rng.integers(0, 16, size=(nq, d)).astype(np.float32)
    return base, q


def _rank(rank, world, port, out):
    import torch

    from oracle import oracle as orc

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    base, q = _data()
    k = 15
    res = {}
    for metric in (orc.METRIC_L2, orc.METRIC_IP):
        # Flat by row ranges: local ids + the range start are global ids
        lo, hi = shard.shard_range(base.shape[0], world, rank)
        d, lab = orc.flat_search(base[lo:hi], q, k, metric)
        lab = np.where(lab >= 0, lab + lo, -1)
        res[("flat", metric)] = _gather(torch, world, d, lab)
        # IVF-PQ by list ranges: the same trained codebooks on every rank,
        # each keeping the lists of its range (the others empty)
        full = orc.IVFPQ(base.shape[1], 16, 8, metric)
        full.train(base, niter_coarse=5, niter_pq=5)
        full.add(base)
        off, ids, codes = full.lists()
        llo, lhi = shard.shard_range(16, world, rank)
        keep = np.zeros(ids.shape[0], bool)
        keep[off[llo]:off[lhi]] = True
        lens = np.diff(off)
        lens[:llo] = 0
        lens[lhi:] = 0
        part = orc.IVFPQ(base.shape[1], 16, 8, metric)
        part.set_codebooks(*full.codebooks())
        part.set_lists(np.concatenate([[0], np.cumsum(lens)]), ids[keep], codes[keep])
        d, lab = part.search(q, k, 6)
        res[("ivfpq", metric)] = _gather(torch, world, d, lab)
    if rank == 0:
        out.update(res)
    torch.distributed.destroy_process_group()


def _gather(torch, world, d, lab):
    dt = torch.from_numpy(np.ascontiguousarray(d))
    lt = torch.from_numpy(np.ascontiguousarray(lab))
    ds = [torch.empty_like(dt) for _ in range(world)]
    ls = [torch.empty_like(lt) for _ in range(world)]
    torch.distributed.all_gather(ds, dt)
    torch.distributed.all_gather(ls, lt)
    return [x.numpy() for x in ds], [x.numpy() for x in ls]


def test_two_rank_sharded_search_equals_unsharded(orc):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    port = _free_port()
    ctx = tmp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        res = dict(out)
    base, q = _data()
    k = 15
    for metric in (orc.METRIC_L2, orc.METRIC_IP):
        want_d, want_l = orc.flat_search(base, q, k, metric)
        ds, ls = res[("flat", metric)]
        got_d, got_l = shard.merge_topk(ds, ls, k, metric, fill_distance=0.0)
        assert np.array_equal(got_l, want_l)
        assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))
        full = orc.IVFPQ(base.shape[1], 16, 8, metric)
        full.train(base, niter_coarse=5, niter_pq=5)
        full.add(base)
        want_d, want_l = full.search(q, k, 6)
        ds, ls = res[("ivfpq", metric)]
        got_d, got_l = shard.merge_topk(ds, ls, k, metric, fill_distance=1e38)
        assert np.array_equal(got_l, want_l)
        assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))


@pytest.mark.parametrize("metric", [0, 1])
def test_merge_matches_full_sort(metric):
    rng = np.random.default_rng(7)
    nq, n, k = 20, 400, 25
    dist = rng.integers(0, 40, size=(nq, n)).astype(np.float32)  # ties
    lab = np.tile(np.arange(n, dtype=np.int64), (nq, 1))
    lab[:, ::17] = -1  # empty slots
    key = np.where(lab < 0, np.inf, dist if metric == 0 else -dist)
    order = np.lexsort((np.where(lab < 0, np.iinfo(np.int64).max, lab), key), axis=1)[:, :k]
    want_l = np.take_along_axis(lab, order, axis=1)
    cuts = [0, 90, 91, 300, n]
    parts_d, parts_l = [], []
    for a, b in zip(cuts[:-1], cuts[1:]):
        perm = rng.permutation(b - a) + a  # shard order does not matter
        parts_d.append(dist[:, perm])
        parts_l.append(lab[:, perm])
    got_d, got_l = shard.merge_topk(parts_d, parts_l, k, metric)
    assert np.array_equal(got_l, want_l)
    assert np.array_equal(got_d, np.take_along_axis(dist, order, axis=1))
    # fewer results than k: -1 and the fill distance
    d2, l2 = shard.merge_topk([dist[:, :3]], [lab[:, :3]], 5, metric, fill_distance=1e38)
    assert (l2[:, 3:] == -1).all() and (d2[:, 3:] == np.float32(1e38)).all()
    assert shard.shard_range(10, 3, 0) == (0, 4) and shard.shard_range(10, 3, 2) == (7, 10)
