"""CollectionIVFPQ snapshot format restated in Python.

TEST INFRASTRUCTURE. Only tests/ import this module, as the checker of the
native snapshot codec. It writes and reads the bytes the reference writes
(paths relative to the MojoVec project root):

* checksum            io/snapshot_file.mojo:19-61 (seed, 8 MiB chunks, the
                      per-word mix and the tail / length fold)
* trailer             io/snapshot_file.mojo:64-108 (magic, checksum)
* collection header   api/collection_ivfpq.mojo:335-370 (magic, version,
                      dimension, name, metric, user ids) and
                      api/collection_codec.mojo:49-64 (strings)
* IndexIVFPQ          io/serialization.mojo:1024-1039 (header, quantizer,
                      inverted lists, product quantizer), :229-238
                      (IndexFlat), :903-914 (lists), :946-952 (PQ)

Parity status: unpinned by golden bytes (the reference's tests hold no
snapshot fixtures and the Mojo reference cannot run here); the layout and the
checksum follow the reference's writer and reader line by line.
"""

from __future__ import annotations

import struct

import numpy as np

COLLECTION_IVFPQ_MAGIC = 0x43495650
COLLECTION_IVFPQ_VERSION = 1
MAGIC_FLAT = 0x4D4A4F46
MAGIC_IVF_PQ = 0x4D4A4F50
MAGIC_INVLISTS = 0x4D4A4F4C
MAGIC_PQ = 0x4D4A4F51
CHECKSUM_MAGIC = 0x4D4F4A4F534E4150
CHECKSUM_SEED = 0xD6E8FEB86659FD93
CHUNK = 8 * 1024 * 1024
_MASK = (1 << 64) - 1


def _rotl(v: int, a: int) -> int:
    return ((v << a) | (v >> (64 - a))) & _MASK


def checksum_update(cs: int, chunk: bytes) -> int:
    """_checksum_update (io/snapshot_file.mojo:19-42)."""
    r = cs
    words = len(chunk) // 8
    for w in np.frombuffer(chunk, dtype="<u8", count=words).tolist():
        r ^= w
        r = _rotl(r, 27) ^ _rotl(w, 17)
        r ^= r >> 23
    tail = 0
    for i, b in enumerate(chunk[words * 8:]):
        tail |= b << (8 * i)
    r ^= tail
    r ^= (len(chunk) << 32) & _MASK
    return _rotl(r, 11)


def checksum(payload: bytes) -> int:
    """_checksum_prefix (io/snapshot_file.mojo:45-61)."""
    cs = CHECKSUM_SEED
    for off in range(0, len(payload), CHUNK):
        cs = checksum_update(cs, payload[off:off + CHUNK])
    return cs


class _W:
    def __init__(self):
        self.parts = []

    def i64(self, v):
        self.parts.append(struct.pack("<q", int(v)))

    def boolean(self, v):
        self.parts.append(b"\x01" if v else b"\x00")

    def string(self, s: str):
        b = s.encode("utf-8")
        self.i64(len(b))
        self.parts.append(b)

    def raw(self, a, dtype):
        self.parts.append(np.ascontiguousarray(a, dtype=dtype).tobytes())

    def bytes(self):
        return b"".join(self.parts)


def write_collection_ivfpq(name, metric, user_ids, d, nlist, M, nprobe, is_trained,
                           centroids, pq_centroids, offsets, ids, codes,
                           quantizer_capacity=None, list_capacities=None):
    """The bytes CollectionIVFPQ.save writes for these contents, trailer
    included. The quantizer holds nlist rows when trained (none before);
    capacities default to the sizes."""
    mi = 0 if metric == "l2" else 1
    w = _W()
    w.i64(COLLECTION_IVFPQ_MAGIC)
    w.i64(COLLECTION_IVFPQ_VERSION)
    w.i64(d)
    w.string(name)
    w.string(metric)
    user_ids = np.asarray(user_ids, dtype=np.int64)
    w.i64(user_ids.shape[0])
    w.raw(user_ids, "<i8")
    # write_index_ivf_pq
    w.i64(MAGIC_IVF_PQ)
    for v in (d, nlist, M, nprobe, int(offsets[-1])):
        w.i64(v)
    w.boolean(is_trained)
    w.i64(mi)
    # write_index_flat (quantizer)
    qn = nlist if is_trained else 0
    qcap = qn if quantizer_capacity is None else quantizer_capacity
    w.i64(MAGIC_FLAT)
    w.i64(d)
    w.i64(qn)
    w.i64(qcap)
    w.i64(mi)
    q = np.zeros((qcap, d), np.float32)
    q[:qn] = np.asarray(centroids, np.float32).reshape(-1, d)[:qn]
    w.raw(q, "<f4")
    # write_invlists
    w.i64(MAGIC_INVLISTS)
    w.i64(nlist)
    w.i64(M)
    codes = np.asarray(codes, np.uint8).reshape(-1, M)
    ids = np.asarray(ids, np.int64)
    for l in range(nlist):
        a, b = int(offsets[l]), int(offsets[l + 1])
        w.i64(b - a)
        w.i64((b - a) if list_capacities is None else list_capacities[l])
        w.raw(ids[a:b], "<i8")
        w.raw(codes[a:b], np.uint8)
    # write_pq
    w.i64(MAGIC_PQ)
    w.i64(d)
    w.i64(M)
    w.i64(256)
    w.boolean(is_trained)
    w.raw(np.asarray(pq_centroids, np.float32).reshape(-1), "<f4")
    payload = w.bytes()
    return payload + struct.pack("<QQ", CHECKSUM_MAGIC, checksum(payload))


class SnapshotError(ValueError):
    pass


def read_collection_ivfpq(data: bytes) -> dict:
    """CollectionIVFPQ.load's parse (api/collection_ivfpq.mojo:372-476),
    returning the contents as arrays; raises SnapshotError where the
    reference raises."""
    if len(data) < 16:
        raise SnapshotError("IVF-PQ snapshot checksum trailer is missing.")
    payload = data[:-16]
    magic, expected = struct.unpack("<QQ", data[-16:])
    if magic != CHECKSUM_MAGIC:
        raise SnapshotError("Invalid snapshot checksum trailer.")
    if checksum(payload) != expected:
        raise SnapshotError("Snapshot checksum mismatch.")
    pos = 0

    def take(n):
        nonlocal pos
        if n < 0 or pos + n > len(payload):
            raise SnapshotError("Unexpected end of serialized data.")
        b = payload[pos:pos + n]
        pos += n
        return b

    def i64():
        return struct.unpack("<q", take(8))[0]

    def boolean():
        v = take(1)[0]
        if v > 1:
            raise SnapshotError("Invalid serialized Bool value.")
        return v == 1

    def string():
        n = i64()
        if n < 0 or n > 1_048_576:
            raise SnapshotError("Security Error: size out of range")
        return take(n).decode("utf-8")

    if i64() != COLLECTION_IVFPQ_MAGIC:
        raise SnapshotError("Invalid CollectionIVFPQ snapshot magic.")
    if i64() != COLLECTION_IVFPQ_VERSION:
        raise SnapshotError("Unsupported CollectionIVFPQ snapshot version.")
    out = {"dimension": i64(), "name": string(), "metric": string()}
    if out["metric"] not in ("l2", "cosine", "ip"):
        raise SnapshotError('metric must be "l2", "cosine", or "ip".')
    n = i64()
    out["user_ids"] = np.frombuffer(take(8 * n), "<i8").astype(np.int64)
    if i64() != MAGIC_IVF_PQ:
        raise SnapshotError("Invalid magic for IndexIVFPQ")
    d, nlist, M, nprobe, ntotal = (i64() for _ in range(5))
    is_trained = boolean()
    mi = i64()
    out.update(d=d, nlist=nlist, M=M, nprobe=nprobe, ntotal=ntotal, is_trained=is_trained,
               metric_int=mi)
    if i64() != MAGIC_FLAT:
        raise SnapshotError("Invalid magic for IndexFlat")
    qd, qn, qcap, qm = i64(), i64(), i64(), i64()
    if qd != d or qn != (nlist if is_trained else 0) or (1 if qm == 1 else 0) != mi:
        raise SnapshotError("IndexIVFPQ coarse quantizer header mismatch.")
    q = np.frombuffer(take(4 * qcap * d), "<f4").reshape(qcap, d)
    out["centroids"] = q[:qn].copy()
    if i64() != MAGIC_INVLISTS:
        raise SnapshotError("Invalid magic for ArrayInvertedLists")
    if i64() != nlist or i64() != M:
        raise SnapshotError("Inverted-list shape does not match its index header.")
    off = [0]
    ids, codes = [], []
    for _ in range(nlist):
        size, cap = i64(), i64()
        if size < 0 or size > cap:
            raise SnapshotError("Security Error: size out of range")
        ids.append(np.frombuffer(take(8 * size), "<i8"))
        codes.append(np.frombuffer(take(size * M), np.uint8))
        off.append(off[-1] + size)
    out["offsets"] = np.array(off, np.int64)
    out["ids"] = np.concatenate(ids).astype(np.int64) if ids else np.zeros(0, np.int64)
    out["codes"] = (np.concatenate(codes) if codes else np.zeros(0, np.uint8)).reshape(-1, M)
    if i64() != MAGIC_PQ:
        raise SnapshotError("Invalid magic for ProductQuantizer")
    if (i64(), i64(), i64()) != (d, M, 256):
        raise SnapshotError("ProductQuantizer shape does not match its index header.")
    if boolean() != is_trained:
        raise SnapshotError("IndexIVFPQ training state mismatch.")
    out["pq_centroids"] = np.frombuffer(take(4 * 256 * d), "<f4").reshape(M, 256, d // M).copy()
    if pos != len(payload):
        raise SnapshotError("IVF-PQ snapshot contains unexpected payload data.")
    return out
