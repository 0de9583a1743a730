"""ctypes binding for the MojoVec CPU-path oracle.

TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module, and only as the checker. Each wrapper
names the reference function it restates (paths relative to the MojoVec
project root); the C++ source cites the exact lines.

Parity status: pinned by the reference's known-answer tests only (the Mojo
reference cannot run here); Mojo's reduce_add lane order, fp contraction and
round-tie rule are fixed by documented choice.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

METRIC_L2 = 0
METRIC_IP = 1
MODE_REFERENCE_HEAP = 0
MODE_CANONICAL = 1

_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_i64 = C.c_int64
_int = C.c_int


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = build_oracle.build()
    L = C.CDLL(path)
    _sig(L, "orc_l2_simd", C.c_float, [_int, _f32p, _f32p, _i64])
    _sig(L, "orc_ip_simd", C.c_float, [_int, _f32p, _f32p, _i64])
    _sig(L, "orc_l2_short4", C.c_float, [_f32p, _f32p, _i64])
    _sig(L, "orc_ip_short4", C.c_float, [_f32p, _f32p, _i64])
    _sig(L, "orc_sq8_dot_u8", C.c_uint32, [_u8p, _u8p, _i64])
    _sig(L, "orc_sq8_dot_s8", C.c_int32, [_i8p, _i8p, _i64])
    _sig(L, "orc_philox_block", None, [_u32p, _u32p, _u32p])
    _sig(L, "orc_philox_steps", None, [C.c_uint64, _i64, _u32p])
    _sig(L, "orc_kmeans_train", None, [_f32p, _i64, _int, _int, _int, _int, _f32p, _i64p])
    _sig(L, "orc_pq_train", None, [_f32p, _i64, _int, _int, _int, _int, _int, _f32p])
    _sig(L, "orc_pq_compute_codes", None, [_f32p, _int, _int, _int, _f32p, _i64, _u8p])
    _sig(L, "orc_pq_decode", None, [_f32p, _int, _int, _int, _u8p, _i64, _f32p])
    _sig(L, "orc_pq_distance_table", None, [_f32p, _int, _int, _int, _f32p, _int, _f32p])
    _sig(L, "orc_flat_search", None,
         [_f32p, _i64, _int, _int, _f32p, _i64, _i64, _vp, _int, _f32p, _i64p, _int])
    _sig(L, "orc_ivfpq_create", _vp, [_int, _int, _int, _int])
    _sig(L, "orc_ivfpq_destroy", None, [_vp])
    _sig(L, "orc_ivfpq_train", None, [_vp, _f32p, _i64, _int, _int, _int])
    _sig(L, "orc_ivfpq_set_codebooks", None, [_vp, _f32p, _f32p])
    _sig(L, "orc_ivfpq_get_codebooks", None, [_vp, _f32p, _f32p])
    _sig(L, "orc_ivfpq_add_with_ids", None, [_vp, _f32p, _i64, _i64p, _int])
    _sig(L, "orc_ivfpq_add", None, [_vp, _f32p, _i64, _int])
    _sig(L, "orc_ivfpq_ntotal", _i64, [_vp])
    _sig(L, "orc_ivfpq_get_lists", None, [_vp, _i64p, _i64p, _u8p])
    _sig(L, "orc_ivfpq_set_lists", None, [_vp, _i64p, _i64p, _u8p])
    _sig(L, "orc_ivfpq_search", None,
         [_vp, _f32p, _i64, _i64, _i64, _vp, _i64, _int, _f32p, _i64p, _int, _int])
    _sig(L, "orc_ivfflat_create", _vp, [_int, _int, _int])
    _sig(L, "orc_ivfflat_destroy", None, [_vp])
    _sig(L, "orc_ivfflat_train", None, [_vp, _f32p, _i64, _int, _int])
    _sig(L, "orc_ivfflat_add", None, [_vp, _f32p, _i64, _int])
    _sig(L, "orc_ivfflat_centroids", None, [_vp, _f32p])
    _sig(L, "orc_ivfflat_search", None, [_vp, _f32p, _i64, _i64, _i64, _int, _f32p, _i64p, _int])
    _sig(L, "orc_sq8_create", _vp, [_int, _int])
    _sig(L, "orc_sq8_destroy", None, [_vp])
    _sig(L, "orc_sq8_add", None, [_vp, _f32p, _i64])
    _sig(L, "orc_sq8_params", None, [_vp, _f32p])
    _sig(L, "orc_sq8_get_codes", None, [_vp, _u8p, _u32p])
    _sig(L, "orc_sq8_search", None,
         [_vp, _f32p, _i64, _i64, _vp, _int, _f32p, _i64p, _int])
    _sig(L, "orc_sq8_encode", None, [_int, _f32p, _i64, _int, C.c_float, C.c_float, _u8p, _u32p])
    _sig(L, "orc_rerank", None,
         [_f32p, _int, _int, _f32p, _i64, _i64p, _i64, _i64, _int, _f32p, _i64p, _int])
    _sig(L, "orc_normalize", _int, [_f32p, _i64, _int, _f32p])
    _sig(L, "orc_ground_truth", None,
         [_f32p, _i64, _int, _int, _f32p, _i64, _i64, _f64p, _i64p, _int])
    _lib = L
    return L


def _threads(n):
    return int(n) if n else (os.cpu_count() or 1)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr_or_none(a):
    return None if a is None else a.ctypes.data


# --- utils/distances.mojo ---------------------------------------------------
def l2_simd(x, y, width=8):
    x, y = _f32(x), _f32(y)
    return lib().orc_l2_simd(width, x, y, x.size)


def ip_simd(x, y, width=8):
    x, y = _f32(x), _f32(y)
    return lib().orc_ip_simd(width, x, y, x.size)


def l2_short4(x, y):
    x, y = _f32(x), _f32(y)
    return lib().orc_l2_short4(x, y, x.size)


def ip_short4(x, y):
    x, y = _f32(x), _f32(y)
    return lib().orc_ip_short4(x, y, x.size)


def sq8_dot_u8(x, y):
    x = np.ascontiguousarray(x, np.uint8)
    y = np.ascontiguousarray(y, np.uint8)
    return lib().orc_sq8_dot_u8(x, y, x.size)


def sq8_dot_s8(x, y):
    x = np.ascontiguousarray(x, np.int8)
    y = np.ascontiguousarray(y, np.int8)
    return lib().orc_sq8_dot_s8(x, y, x.size)


# --- Philox4x32-10 ----------------------------------------------------------
def philox_block(counter, key):
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox_block(c, k, out)
    return out


def philox_steps(seed, nsteps):
    out = np.zeros(4 * nsteps, np.uint32)
    lib().orc_philox_steps(seed, nsteps, out)
    return out.reshape(nsteps, 4)


def philox_uniform_matrix(seed, n, d):
    """Rows filled the way the reference tests fill them from
    Random(seed).step_uniform() (tests/test_accuracy.mojo:24-37): one
    step per 4 values. step_uniform is taken as (word >> 8) * 2**-24."""
    total = n * d
    words = philox_steps(seed, (total + 3) // 4).reshape(-1)[:total]
    u = (words >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -24)
    return u.reshape(n, d)


# --- clustering/kmeans.mojo -------------------------------------------------
def kmeans_train(x, k, niter=15, nthreads=0):
    x = _f32(x)
    n, d = x.shape
    cent = np.zeros((k, d), np.float32)
    assign = np.zeros(n, np.int64)
    lib().orc_kmeans_train(x, n, d, k, niter, _threads(nthreads), cent, assign)
    return cent, assign


# --- quantization/pq.mojo ---------------------------------------------------
def pq_train(x, M, niter=15, ksub=256, nthreads=0):
    x = _f32(x)
    n, d = x.shape
    out = np.zeros((M, ksub, d // M), np.float32)
    lib().orc_pq_train(x, n, d, M, ksub, niter, _threads(nthreads), out)
    return out


def pq_compute_codes(pq_centroids, x):
    pq_centroids = _f32(pq_centroids)
    x = _f32(x)
    M, ksub, dsub = pq_centroids.shape
    n = x.shape[0]
    codes = np.zeros((n, M), np.uint8)
    lib().orc_pq_compute_codes(pq_centroids, M * dsub, M, ksub, x, n, codes)
    return codes


def pq_decode(pq_centroids, codes):
    pq_centroids = _f32(pq_centroids)
    codes = np.ascontiguousarray(codes, np.uint8)
    M, ksub, dsub = pq_centroids.shape
    n = codes.shape[0]
    out = np.zeros((n, M * dsub), np.float32)
    lib().orc_pq_decode(pq_centroids, M * dsub, M, ksub, codes, n, out)
    return out


def pq_distance_table(pq_centroids, q, metric=METRIC_L2):
    pq_centroids = _f32(pq_centroids)
    q = _f32(q)
    M, ksub, dsub = pq_centroids.shape
    table = np.zeros((M, ksub), np.float32)
    lib().orc_pq_distance_table(pq_centroids, M * dsub, M, ksub, q, metric, table)
    return table


# --- index/index_flat.mojo --------------------------------------------------
def flat_search(base, q, k, metric=METRIC_L2, filter=None, mode=MODE_CANONICAL, nthreads=0):
    base, q = _f32(base), _f32(q)
    nb, d = base.shape
    nq = q.shape[0]
    dist = np.zeros((nq, k), np.float32)
    lab = np.full((nq, k), -1, np.int64)
    flt = None if filter is None else np.ascontiguousarray(filter, np.uint8)
    lib().orc_flat_search(base, nb, d, metric, q, nq, k, _ptr_or_none(flt), mode, dist, lab,
                          _threads(nthreads))
    return dist, lab


# --- index/index_ivf_pq.mojo ------------------------------------------------
class IVFPQ:
    """Restatement of IndexIVFPQ[IndexFlat] (index/index_ivf_pq.mojo:12)."""

    def __init__(self, d, nlist, M, metric=METRIC_L2):
        self.d, self.nlist, self.M, self.metric = d, nlist, M, metric
        self._h = lib().orc_ivfpq_create(d, nlist, M, metric)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.orc_ivfpq_destroy(h)
            self._h = None

    def train(self, x, niter_coarse=15, niter_pq=15, nthreads=0):
        x = _f32(x)
        lib().orc_ivfpq_train(self._h, x, x.shape[0], niter_coarse, niter_pq, _threads(nthreads))

    def set_codebooks(self, centroids, pq_centroids):
        lib().orc_ivfpq_set_codebooks(self._h, _f32(centroids), _f32(pq_centroids))

    def codebooks(self):
        c = np.zeros((self.nlist, self.d), np.float32)
        p = np.zeros((self.M, 256, self.d // self.M), np.float32)
        lib().orc_ivfpq_get_codebooks(self._h, c, p)
        return c, p

    def add(self, x, ids=None, nthreads=0):
        x = _f32(x)
        if ids is None:
            lib().orc_ivfpq_add(self._h, x, x.shape[0], _threads(nthreads))
        else:
            ids = np.ascontiguousarray(ids, np.int64)
            lib().orc_ivfpq_add_with_ids(self._h, x, x.shape[0], ids, _threads(nthreads))

    @property
    def ntotal(self):
        return lib().orc_ivfpq_ntotal(self._h)

    def lists(self):
        """CSR export: (offsets[nlist+1], ids[ntotal], codes[ntotal, M])."""
        n = self.ntotal
        off = np.zeros(self.nlist + 1, np.int64)
        ids = np.zeros(max(n, 1), np.int64)
        codes = np.zeros((max(n, 1), self.M), np.uint8)
        lib().orc_ivfpq_get_lists(self._h, off, ids, codes)
        return off, ids[:n], codes[:n]

    def set_lists(self, offsets, ids, codes):
        lib().orc_ivfpq_set_lists(self._h, np.ascontiguousarray(offsets, np.int64),
                                  np.ascontiguousarray(ids, np.int64),
                                  np.ascontiguousarray(codes, np.uint8))

    def search(self, q, k, nprobe, filter=None, mode=MODE_CANONICAL, nthreads=0, lut_threads=1):
        q = _f32(q)
        nq = q.shape[0]
        dist = np.zeros((nq, k), np.float32)
        lab = np.zeros((nq, k), np.int64)
        flt = None if filter is None else np.ascontiguousarray(filter, np.uint8)
        flen = 0 if flt is None else flt.size
        lib().orc_ivfpq_search(self._h, q, nq, k, nprobe, _ptr_or_none(flt), flen, mode, dist,
                               lab, _threads(nthreads), _threads(lut_threads))
        return dist, lab


# --- index/index_flat_sq8.mojo ----------------------------------------------
class IVFFlat:
    """IndexIVFFlat restated (index/index_ivf_flat.mojo)."""

    def __init__(self, d, nlist, metric=METRIC_L2):
        self.d, self.nlist, self.metric = d, nlist, metric
        self._h = lib().orc_ivfflat_create(d, nlist, metric)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_ivfflat_destroy(h)
            self._h = None

    def train(self, x, niter=15, nthreads=0):
        x = _f32(x)
        lib().orc_ivfflat_train(self._h, x, x.shape[0], niter, _threads(nthreads))

    def add(self, x, nthreads=0):
        x = _f32(x)
        lib().orc_ivfflat_add(self._h, x, x.shape[0], _threads(nthreads))

    def centroids(self):
        out = np.zeros((self.nlist, self.d), np.float32)
        lib().orc_ivfflat_centroids(self._h, out)
        return out

    def search(self, q, k, nprobe, mode=MODE_CANONICAL, nthreads=0):
        q = _f32(q)
        n = q.shape[0]
        dist = np.zeros((n, k), np.float32)
        lab = np.zeros((n, k), np.int64)
        lib().orc_ivfflat_search(self._h, q, n, k, nprobe, mode, dist, lab, _threads(nthreads))
        return dist, lab


class SQ8:
    """Restatement of IndexFlatSQ8 (index/index_flat_sq8.mojo:271)."""

    def __init__(self, d, metric=METRIC_L2):
        self.d, self.metric = d, metric
        self._h = lib().orc_sq8_create(d, metric)
        self.ntotal = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.orc_sq8_destroy(h)
            self._h = None

    def add(self, x):
        x = _f32(x)
        lib().orc_sq8_add(self._h, x, x.shape[0])
        self.ntotal += x.shape[0]

    def params(self):
        out = np.zeros(3, np.float32)
        lib().orc_sq8_params(self._h, out)
        return float(out[0]), float(out[1]), float(out[2])

    def codes(self):
        c = np.zeros((max(self.ntotal, 1), self.d), np.uint8)
        nrm = np.zeros(max(self.ntotal, 1), np.uint32)
        lib().orc_sq8_get_codes(self._h, c, nrm)
        return c[: self.ntotal], nrm[: self.ntotal]

    def search(self, q, k, filter=None, mode=MODE_CANONICAL, nthreads=0):
        q = _f32(q)
        nq = q.shape[0]
        dist = np.zeros((nq, k), np.float32)
        lab = np.zeros((nq, k), np.int64)
        flt = None if filter is None else np.ascontiguousarray(filter, np.uint8)
        lib().orc_sq8_search(self._h, q, nq, k, _ptr_or_none(flt), mode, dist, lab,
                             _threads(nthreads))
        return dist, lab


def sq8_encode(x, minimum, inv_scale, symmetric):
    x = _f32(x)
    n, d = x.shape
    codes = np.zeros((n, d), np.uint8)
    norms = np.zeros(n, np.uint32)
    lib().orc_sq8_encode(1 if symmetric else 0, x, n, d, minimum, inv_scale, codes, norms)
    return codes, norms


def rerank(base, q, cand, k, metric=METRIC_L2, mode=MODE_CANONICAL, nthreads=0):
    base, q = _f32(base), _f32(q)
    cand = np.ascontiguousarray(cand, np.int64)
    nq, nc = cand.shape
    dist = np.zeros((nq, k), np.float32)
    lab = np.zeros((nq, k), np.int64)
    lib().orc_rerank(base, base.shape[1], metric, q, nq, cand, nc, k, mode, dist, lab,
                     _threads(nthreads))
    return dist, lab


def normalize(x):
    x = _f32(x)
    out = np.zeros_like(x)
    rc = lib().orc_normalize(x, x.shape[0], x.shape[1], out)
    if rc == -1:
        raise ValueError("Vector components must be finite.")
    if rc == -2:
        raise ValueError("Cosine embeddings must be non-zero vectors.")
    return out


def ground_truth(base, q, k, metric=METRIC_L2, nthreads=0):
    base, q = _f32(base), _f32(q)
    nq = q.shape[0]
    dist = np.zeros((nq, k), np.float64)
    lab = np.zeros((nq, k), np.int64)
    lib().orc_ground_truth(base, base.shape[0], base.shape[1], metric, q, nq, k, dist, lab,
                           _threads(nthreads))
    return dist, lab


def recall(gt_labels, labels):
    """Fraction of ground-truth ids found in the returned ids, as
    compute_recall in tests/test_accuracy.mojo:58-69."""
    gt = np.asarray(gt_labels)
    got = np.asarray(labels)
    hits = 0
    for i in range(gt.shape[0]):
        hits += len(set(gt[i].tolist()) & set(got[i].tolist()))
    return hits / gt.size


class CollectionIVFPQ:
    """Restatement of the managed IVF-PQ collection's query path over the
    oracle index (api/collection_ivfpq.mojo): training validation and
    cosine normalisation (:170-185), id validation and auto-train on the
    first add (:187-242), query validation and preparation (:254-285), and
    the id map with 1 - d for the cosine and inner-product metrics
    (:287-333). Test infrastructure only."""

    MAX_QUERY_RESULTS = 2048
    PQ_CENTROIDS = 256

    def __init__(self, d, nlist, M, nprobe, metric="l2"):
        if metric not in ("l2", "cosine", "ip"):
            raise ValueError('metric must be "l2", "cosine", or "ip".')
        self.d, self.metric, self.nprobe = d, metric, nprobe
        self.index = IVFPQ(d, nlist, M, METRIC_L2 if metric == "l2" else METRIC_IP)
        self.nlist = nlist
        self.trained = False
        self.user_ids = []
        self.id_to_internal = {}

    def _prepare(self, rows):
        rows = _f32(rows).reshape(-1, self.d)
        if self.metric == "cosine":  # collection_vector_query.mojo:24-46
            return normalize(rows)
        if rows.size and not np.isfinite(rows).all():
            raise ValueError("Vector components must be finite.")
        return rows

    def train(self, rows):
        rows = _f32(rows).reshape(-1, self.d)
        if rows.shape[0] < max(self.nlist, self.PQ_CENTROIDS):
            raise ValueError("IVF-PQ training requires at least max(nlist, 256) vectors.")
        if self.trained:
            return
        self.index.train(self._prepare(rows))
        self.trained = True

    def add(self, ids, rows):
        rows = _f32(rows).reshape(-1, self.d)
        if rows.shape[0] != len(ids):
            raise ValueError("Embeddings length must equal len(ids) * dimension.")
        if len(ids) == 0:
            return
        seen = set()
        for rid in ids:
            if rid in seen:
                raise ValueError("Duplicate IDs are not allowed within an add batch.")
            if rid in self.id_to_internal:
                raise ValueError("Cannot add an ID that already exists.")
            seen.add(rid)
        if not self.trained:
            self.train(rows)
        self.index.add(self._prepare(rows))
        for rid in ids:
            self.id_to_internal[int(rid)] = len(self.user_ids)
            self.user_ids.append(int(rid))

    def query(self, rows, n_results=10):
        """(ids, distances) as lists of rows, collection_ivfpq.mojo:287-333."""
        rows = _f32(rows).reshape(-1, self.d)
        if n_results <= 0 or n_results > self.MAX_QUERY_RESULTS:
            raise ValueError("n_results must be between 1 and 2048.")
        if rows.shape[0] == 0:
            return [], []
        dist, lab = self.index.search(self._prepare(rows), n_results, self.nprobe)
        all_ids, all_dist = [], []
        for drow, lrow in zip(dist, lab):
            ids, ds = [], []
            for dv, iv in zip(drow, lrow):
                if 0 <= iv < len(self.user_ids):
                    ids.append(self.user_ids[iv])
                    ds.append(np.float32(1.0) - dv if self.metric != "l2" else dv)
                else:
                    ids.append(-1)
                    ds.append(dv)
            all_ids.append(ids)
            all_dist.append(np.array(ds, np.float32))
        return all_ids, all_dist
