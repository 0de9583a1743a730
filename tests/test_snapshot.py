"""IVF-PQ collection snapshots (api/collection_ivfpq.mojo:335-476).

CPU: the library's checksum (mv_snapshot_checksum, host code) equals the
restated one (io/snapshot_file.mojo:19-61) on ragged lengths and across the
8 MiB chunk edge; the restated writer and reader round-trip and reject the
corruptions the reference rejects.

GPU: the reference's own round-trip cases (tests/test_ivf_pq.mojo:155-206:
d 8, 256 rows, nlist 8, M 2, nprobe 4, cosine; an untrained "ip"
collection), byte equality between the native writer and the restated one,
an oracle-built index written by the restated writer and loaded onto the GPU
searching exactly as the oracle does, and the loader's rejections.
"""

import os

import numpy as np
import pytest

from oracle import snapshot as S

DIM, COUNT = 8, 256


# --- CPU ---------------------------------------------------------------------

@pytest.mark.parametrize("n", [0, 1, 7, 8, 9, 15, 16, 1000, 4097])
def test_checksum_matches_restatement(mv, n):
    from mojovec_gb300 import _lib

    data = np.random.default_rng(n).integers(0, 256, size=n, dtype=np.uint8).tobytes()
    got = _lib.load().mv_snapshot_checksum(data, len(data))
    assert got == S.checksum(data)


def test_checksum_across_chunk_edge(mv):
    from mojovec_gb300 import _lib

    n = S.CHUNK + 13  # two chunks, the second ragged
    data = np.random.default_rng(1).integers(0, 256, size=n, dtype=np.uint8).tobytes()
    assert _lib.load().mv_snapshot_checksum(data, n) == S.checksum(data)
    # chunking matters: one pass over all bytes gives another value
    assert S.checksum(data) != S.checksum_update(S.CHECKSUM_SEED, data)


def _small_contents(trained=True, nlist=4, d=8, M=2, n=10, seed=0):
    rng = np.random.default_rng(seed)
    assign = rng.integers(0, nlist, size=n)
    order = np.argsort(assign, kind="stable")
    off = np.zeros(nlist + 1, np.int64)
    np.add.at(off, assign + 1, 1)
    off = np.cumsum(off)
    return dict(name="c", metric="l2", user_ids=np.arange(n) + 100, d=d, nlist=nlist, M=M,
                nprobe=2, is_trained=trained,
                centroids=rng.standard_normal((nlist, d)).astype(np.float32),
                pq_centroids=rng.standard_normal((M, 256, d // M)).astype(np.float32),
                offsets=off, ids=order.astype(np.int64),
                codes=rng.integers(0, 256, size=(n, M), dtype=np.uint8))


def test_restated_writer_reader_round_trip():
    c = _small_contents()
    r = S.read_collection_ivfpq(S.write_collection_ivfpq(**c))
    assert r["name"] == "c" and r["metric"] == "l2" and r["nprobe"] == 2
    for key in ("user_ids", "offsets", "ids", "codes", "centroids"):
        assert np.array_equal(r[key], c[key]), key
    assert np.array_equal(r["pq_centroids"], c["pq_centroids"])


def test_restated_reader_rejects_corruption():
    blob = bytearray(S.write_collection_ivfpq(**_small_contents()))
    for pos in (0, 40, len(blob) - 17, len(blob) - 16, len(blob) - 1):
        bad = bytearray(blob)
        bad[pos] ^= 0xFF
        with pytest.raises(S.SnapshotError):
            S.read_collection_ivfpq(bytes(bad))
    with pytest.raises(S.SnapshotError):
        S.read_collection_ivfpq(bytes(blob[:10]))


# --- GPU ---------------------------------------------------------------------

def _tmp(tmp_path, name):
    return os.fspath(tmp_path / name)


@pytest.mark.gpu
def test_reference_round_trip_cosine(mv, tmp_path):
    """test_ivfpq_save_load_round_trip (tests/test_ivf_pq.mojo:155-186)."""
    from mojovec_gb300 import synth

    v = synth.grid_vectors(COUNT, DIM)
    v /= np.linalg.norm(v, axis=1, keepdims=True)  # the collection stores cosine rows unit-normalized
    ix = mv.IndexIVFPQ(DIM, 8, 2, mv.METRIC_IP)
    ix.nprobe = 4
    ix.train(v)
    ix.add(v)
    ids = np.arange(COUNT, dtype=np.int64) + 50_000
    exp_d, exp_l = ix.search(v[:1], 3)
    path = _tmp(tmp_path, "persistent.bin")
    ix.save_snapshot(path, "persistent", "cosine", ids)
    assert not os.path.exists(path + ".tmp")
    ld = mv.IndexIVFPQ.load_snapshot(path)
    name, metric, uids = ld.collection
    assert (name, metric) == ("persistent", "cosine")
    assert ld.ntotal == COUNT and ld.nprobe == 4 and ld.is_trained
    assert np.array_equal(uids, ids)
    got_d, got_l = ld.search(v[:1], 3)
    assert np.array_equal(got_l, exp_l) and np.array_equal(got_d, exp_d)
    # the file is what the restated writer writes for the same contents
    off, lid, codes = ix.lists()
    cent, pq = ix.codebooks()
    blob = S.write_collection_ivfpq("persistent", "cosine", ids, DIM, 8, 2, 4, True, cent, pq,
                                    off, lid, codes)
    assert open(path, "rb").read() == blob


@pytest.mark.gpu
def test_reference_untrained_round_trip(mv, tmp_path):
    """test_ivfpq_untrained_snapshot_round_trip (tests/test_ivf_pq.mojo:189-206)."""
    ix = mv.IndexIVFPQ(DIM, 8, 2, mv.METRIC_IP)
    ix.nprobe = 4
    path = _tmp(tmp_path, "empty.bin")
    ix.save_snapshot(path, "empty", "ip", np.zeros(0, np.int64))
    ld = mv.IndexIVFPQ.load_snapshot(path)
    assert not ld.is_trained and ld.ntotal == 0 and ld.nprobe == 4
    assert ld.collection[:2] == ("empty", "ip")
    r = S.read_collection_ivfpq(open(path, "rb").read())
    assert not r["is_trained"] and r["centroids"].shape == (0, DIM)


@pytest.mark.gpu
@pytest.mark.parametrize("metric", ["l2", "ip"])
def test_oracle_index_loads_and_searches_exactly(mv, orc, tmp_path, metric):
    """An index built by the oracle, written with reference capacities above
    the sizes, searched on the GPU in the plain form: bit-exact with the
    oracle. The fast form without rerank runs; with rerank it needs rows."""
    from mojovec_gb300 import synth

    d, nlist, M, n = 32, 64, 8, 6000
    x, q = synth.sift_like(n, d=d, n_centers=50, seed=3, nq=40)
    om = orc.METRIC_L2 if metric == "l2" else orc.METRIC_IP
    o = orc.IVFPQ(d, nlist, M, om)
    o.train(x)
    o.add(x)
    off, ids, codes = o.lists()
    cent, pq = o.codebooks()
    caps = [int(off[l + 1] - off[l]) + (l % 3) for l in range(nlist)]
    uids = np.arange(n, dtype=np.int64) * 7 + 3
    path = _tmp(tmp_path, "oracle.bin")
    with open(path, "wb") as f:
        f.write(S.write_collection_ivfpq("oracle", metric, uids, d, nlist, M, 8, True, cent, pq,
                                         off, ids, codes, quantizer_capacity=nlist + 5,
                                         list_capacities=caps))
    ld = mv.IndexIVFPQ.load_snapshot(path)
    assert np.array_equal(ld.collection[2], uids)
    for k, nprobe in ((10, 8), (100, 64), (1, 1)):
        gd, gl = ld.search(q, k, nprobe=nprobe)
        od, ol = o.search(q, k, nprobe)
        assert np.array_equal(gl, ol) and np.array_equal(gd, od)
    fd, fl = ld.search(q, 10, nprobe=8, form=mv.FORM_FAST)
    assert fl.shape == (q.shape[0], 10) and (fl >= 0).all()
    with pytest.raises(mv.MojoVecGPUError) as e:
        ld.search(q, 10, nprobe=8, form=mv.FORM_FAST, rerank=64)
    assert e.value.code == mv._lib.MV_ERR_STATE
    # rows appended after the load go through the normal add path
    extra = x[:500] + 0.25
    ld.add(extra)
    o.add(extra)
    gd, gl = ld.search(q, 10, nprobe=16)
    od, ol = o.search(q, 10, 16)
    assert np.array_equal(gl, ol) and np.array_equal(gd, od)


def _expect_rejected(mv, path, blob, needle):
    with open(path, "wb") as f:
        f.write(blob)
    with pytest.raises(mv.MojoVecGPUError) as e:
        mv.IndexIVFPQ.load_snapshot(path)
    assert e.value.code == mv._lib.MV_ERR_ARG
    assert needle in str(e.value), str(e.value)


def _refresh(payload: bytes) -> bytes:
    """A deliberately altered payload with a valid trailer, like the
    reference's refresh_snapshot_checksum (tests/test_mmap.mojo:83-92)."""
    import struct

    return payload + struct.pack("<QQ", S.CHECKSUM_MAGIC, S.checksum(payload))


@pytest.mark.gpu
def test_loader_rejections(mv, tmp_path):
    path = _tmp(tmp_path, "bad.bin")
    c = _small_contents()
    good = S.write_collection_ivfpq(**c)
    flip = bytearray(good)
    flip[50] ^= 0xFF
    _expect_rejected(mv, path, bytes(flip), "checksum mismatch")
    trailer = bytearray(good)
    trailer[-16] ^= 0xFF
    _expect_rejected(mv, path, bytes(trailer), "checksum trailer")
    _expect_rejected(mv, path, good[:8], "trailer is missing")
    # trailing payload data under a valid checksum (tests/test_mmap.mojo:121-136)
    _expect_rejected(mv, path, _refresh(good[:-16] + b"\x00"), "unexpected payload data")
    dup = dict(c, ids=np.where(c["ids"] == 1, 2, c["ids"]))
    _expect_rejected(mv, path, S.write_collection_ivfpq(**dup), "duplicate internal ID")
    oob = dict(c, ids=np.where(c["ids"] == 1, 99, c["ids"]))
    _expect_rejected(mv, path, S.write_collection_ivfpq(**oob), "invalid internal ID")
    uid = dict(c, user_ids=np.where(c["user_ids"] == 101, 100, c["user_ids"]))
    _expect_rejected(mv, path, S.write_collection_ivfpq(**uid), "duplicate IDs")
    payload = bytearray(good[:-16])
    payload[8] = 2  # version
    _expect_rejected(mv, path, _refresh(bytes(payload)), "version")
    bad_metric = S.write_collection_ivfpq(**dict(c, metric="dot"))
    _expect_rejected(mv, path, bad_metric, "metric must be")
    # nprobe outside 1..nlist (io/serialization.mojo:1052-1055)
    _expect_rejected(mv, path, S.write_collection_ivfpq(**dict(c, nprobe=0)), "nprobe")
    _expect_rejected(mv, path, S.write_collection_ivfpq(**dict(c, nprobe=c["nlist"] + 1)),
                     "out of valid range")
    ok = mv.IndexIVFPQ.load_snapshot(_write(path, good))
    assert ok.ntotal == 10 and ok.nprobe == 2


def _write(path, blob):
    with open(path, "wb") as f:
        f.write(blob)
    return path
