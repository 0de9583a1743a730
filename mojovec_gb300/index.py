"""Host-side mirror of MojoVec's index and quantizer interfaces, backed by
libmojovec_gpu.so.

Class and method names follow the reference so code (and tests) written
against it read the same:

* IndexIVFPQ      -> mojovec/index/index_ivf_pq.mojo:12 (train, add,
                     add_with_ids, search, nprobe)
* IndexFlat       -> mojovec/index/index_flat.mojo:117 (add, search)
* IndexFlatSQ8    -> mojovec/index/index_flat_sq8.mojo:271 (add, search,
                     scale / global_min / global_max)
* KMeans          -> mojovec/clustering/kmeans.mojo:8 (train, centroids)
* ProductQuantizer-> mojovec/quantization/pq.mojo:80 (train, compute_codes,
                     decode, compute_distance_table)

Search results come back as numpy arrays (distances float32 (n, k), labels
int64 (n, k)) instead of filling caller Spans.
"""

from __future__ import annotations

import atexit
import ctypes as C
import os
import threading
import weakref

import numpy as np

from . import _lib
from ._lib import FORM_FAST, METRIC_IP, METRIC_L2, SearchParams, check


# Native objects still alive at interpreter exit are destroyed by an atexit
# hook, servers first, then plans, then indexes (servers and plans use their
# indexes), before the interpreter's teardown would run their finalizers in
# an arbitrary order (a plan's CUDA graphs outliving its index).
_LIVE = (weakref.WeakSet(), weakref.WeakSet(), weakref.WeakSet())
_TIER_SERVER, _TIER_PLAN, _TIER_INDEX = 0, 1, 2


def _release_all():
    for tier in _LIVE:
        for obj in list(tier):
            try:
                obj._release()
            except Exception:  # noqa: BLE001 - best effort at exit
                pass


atexit.register(_release_all)


def _f32(a, d=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if d is not None:
        a = a.reshape(-1, d)
    return a


def _p(a):
    return None if a is None else a.ctypes.data


def _out(a, n, k, dtype, name):
    """Result array of a search: a new (n, k) array, or the caller's own
    (the reference's search writes into caller-provided distances and
    labels spans, index/index_ivf_pq.mojo:215-232). A caller's array must
    be C-contiguous with that shape and dtype (pinned host memory, e.g.
    from torch's pin_memory(), lets the device copy straight into it)."""
    if a is None:
        return np.empty((n, k), dtype)
    if (not isinstance(a, np.ndarray) or a.dtype != dtype or a.shape != (n, k)
            or not a.flags.c_contiguous or not a.flags.writeable):
        raise ValueError(f"{name} must be a writable C-contiguous {np.dtype(dtype).name} "
                         f"array of shape ({n}, {k})")
    return a


class Context:
    """One CUDA device (mv_ctx)."""

    _default = None
    _default_lock = threading.Lock()

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.mv_ctx_create(device, C.byref(h)))
        self._h = h
        self.device = device

    @classmethod
    def default(cls) -> "Context":
        with cls._default_lock:
            if cls._default is None:
                cls._default = Context(0)
            return cls._default

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        check(_lib.load().mv_ctx_synchronize(self._h))

    def kernel_launches(self) -> int:
        return int(_lib.load().mv_ctx_kernel_launches(self._h))

    def set_wait_limit(self, cycles: int | None):
        """Cycles a tensor-core kernel's pipeline wait may take before the call
        gives up with MV_ERR_TIMEOUT (mv_ctx_set_wait_limit); 0 gives up at
        once unless the wait is already satisfied, None restores the default."""
        check(_lib.load().mv_ctx_set_wait_limit(self._h, -1 if cycles is None else int(cycles)))

    def certify_stats(self) -> dict:
        """Plain-form selections settled on the tensor cores by the error
        bound, and those recomputed by the exact FP32 scan (mv_ctx_certify_stats)."""
        out = np.zeros(4, np.int64)
        check(_lib.load().mv_ctx_certify_stats(self._h, _p(out)))
        return {"assign_rows": int(out[0]), "assign_fallback": int(out[1]),
                "flat_queries": int(out[2]), "flat_fallback": int(out[3])}

    def assign_stats(self) -> tuple:
        """(rows assigned through the certified path, rows of those that took
        the exact FP32 scan)."""
        st = self.certify_stats()
        return st["assign_rows"], st["assign_fallback"]

    def profile(self, enable: bool = True):
        """Enables (and resets) per-stage CUDA-event timing."""
        check(_lib.load().mv_ctx_profile(self._h, 1 if enable else 0))

    def stage_times(self) -> dict:
        """{stage: (total_ms, launches)} since the last profile(True)."""
        n = len(_lib.STAGES)
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int64)
        check(_lib.load().mv_ctx_stage_times(self._h, _p(ms), _p(cnt), n))
        return {name: (float(ms[i]), int(cnt[i])) for i, name in enumerate(_lib.STAGES) if cnt[i]}


def _params(form=None, nprobe=0, rerank=0, coarse_fp32=False, lut_fp16=False, coarse_path=0,
            plain_scan=False, e4m3=False, rerank_fp32=False, lut=None):
    """lut: fast-form table / scan variant (0 FP32 tables, with the two-kernel
    scan where it pays; 2 FP32 in one kernel; 1 FP16; 3 bank-rotated fixed
    point; 4 FP32 with staged lists; 6 bank-rotated fixed point with
    per-candidate slots and a range select; 7 the two-kernel scan: distance
    rows then a per-query select); None takes it from lut_fp16."""
    p = SearchParams()
    p.rerank_fp32 = 1 if rerank_fp32 else 0
    p.coarse_path = int(coarse_path)
    p.plain_scan = 1 if plain_scan else 0
    p.flat_e4m3 = 1 if e4m3 else 0
    p.form = _lib.FORM_PLAIN if form is None else int(form)
    p.nprobe = int(nprobe)
    p.rerank = int(rerank)
    p.coarse_fp32 = 1 if coarse_fp32 else 0
    p.lut_fp16 = int(lut) if lut is not None else (1 if lut_fp16 else 0)
    return p


class IndexIVFPQ:
    """IVF-PQ index on the GPU (index/index_ivf_pq.mojo:12)."""

    def __init__(self, d: int, nlist: int, M: int, metric: int = METRIC_L2, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        check(_lib.load().mv_ivfpq_create(self.ctx.handle, d, nlist, M, metric, C.byref(h)))
        self._h = h
        _LIVE[_TIER_INDEX].add(self)
        self.d, self.nlist, self.M, self.metric_type = d, nlist, M, metric
        self.ksub = 256

    def _release(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_ivfpq_destroy(h)
        self._h = None

    def __del__(self):
        self._release()

    def _info(self):
        out = np.zeros(7, np.int64)
        check(_lib.load().mv_ivfpq_info(self._h, _p(out)))
        return out

    @property
    def nprobe(self) -> int:
        return int(self._info()[3])

    @nprobe.setter
    def nprobe(self, v: int):
        check(_lib.load().mv_ivfpq_set_nprobe(self._h, int(v)))

    @property
    def ntotal(self) -> int:
        return int(self._info()[4])

    @property
    def is_trained(self) -> bool:
        return bool(self._info()[6])

    def set_codebooks(self, centroids, pq_centroids):
        """Loads trained coarse centroids (nlist, d) and PQ codebooks
        (M, 256, d/M), e.g. the reference's own, and marks the index trained."""
        c = _f32(centroids)
        p = _f32(pq_centroids)
        assert c.size == self.nlist * self.d and p.size == 256 * self.d
        check(_lib.load().mv_ivfpq_set_codebooks(self._h, _p(c), _p(p)))

    def codebooks(self):
        c = np.zeros((self.nlist, self.d), np.float32)
        p = np.zeros((self.M, 256, self.d // self.M), np.float32)
        check(_lib.load().mv_ivfpq_get_codebooks(self._h, _p(c), _p(p)))
        return c, p

    def train(self, x, niter_coarse: int = 15, niter_pq: int = 15, form=None):
        """IndexIVFPQ.train; the reference hard-codes 15 iterations for both
        k-means runs (index_ivf_pq.mojo:98, pq.mojo:64). form=FORM_FAST runs
        the coarse k-means in its fast form."""
        x = _f32(x, self.d)
        if form is None:
            check(_lib.load().mv_ivfpq_train(self._h, _p(x), x.shape[0], niter_coarse, niter_pq))
        else:
            p = _params(form)
            check(_lib.load().mv_ivfpq_train_ex(self._h, _p(x), x.shape[0], niter_coarse,
                                                niter_pq, C.byref(p)))

    def add(self, x):
        x = _f32(x, self.d)
        check(_lib.load().mv_ivfpq_add(self._h, _p(x), x.shape[0]))

    def add_with_ids(self, x, ids):
        x = _f32(x, self.d)
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        assert ids.shape[0] == x.shape[0]
        check(_lib.load().mv_ivfpq_add_with_ids(self._h, _p(x), _p(ids), x.shape[0]))

    def lists(self):
        """CSR export: (offsets (nlist+1,), ids (ntotal,), codes (ntotal, M))."""
        off = np.zeros(self.nlist + 1, np.int64)
        check(_lib.load().mv_ivfpq_get_lists(self._h, _p(off), None, None))
        n = int(off[-1])
        ids = np.zeros(max(n, 1), np.int64)
        codes = np.zeros((max(n, 1), self.M), np.uint8)
        check(_lib.load().mv_ivfpq_get_lists(self._h, None, _p(ids), _p(codes)))
        return off, ids[:n], codes[:n]

    def set_lists(self, offsets, ids, codes):
        """Replaces the lists with CSR data (e.g. the reference's own). The
        index then has no rows: the fast form runs without rerank."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        codes = np.ascontiguousarray(codes, dtype=np.uint8)
        assert off.shape == (self.nlist + 1,) and ids.shape[0] == off[-1]
        assert codes.size == ids.shape[0] * self.M
        check(_lib.load().mv_ivfpq_set_lists(self._h, _p(off), _p(ids), _p(codes)))

    def save_snapshot(self, path: str, name: str, metric: str, user_ids):
        """CollectionIVFPQ.save (api/collection_ivfpq.mojo:335-370): user_ids
        holds the collection's record id of each internal id."""
        u = np.ascontiguousarray(user_ids, dtype=np.int64)
        check(_lib.load().mv_ivfpq_save_snapshot(self._h, os.fsencode(path), name.encode(),
                                                 metric.encode(), _p(u), u.shape[0]))

    @classmethod
    def load_snapshot(cls, path: str, ctx: Context | None = None) -> "IndexIVFPQ":
        """CollectionIVFPQ.load (api/collection_ivfpq.mojo:372-476) onto the
        GPU: the checksum and the reference's validation, then the lists go
        straight to device CSR. .collection holds (name, metric, user_ids)."""
        ctx = ctx or Context.default()
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.mv_ivfpq_load_snapshot(ctx.handle, os.fsencode(path), C.byref(h)))
        self = cls.__new__(cls)
        self.ctx, self._h, self.ksub = ctx, h, 256
        _LIVE[_TIER_INDEX].add(self)
        info = np.zeros(7, np.int64)
        check(lib.mv_ivfpq_info(h, _p(info)))
        self.d, self.nlist, self.M = int(info[0]), int(info[1]), int(info[2])
        n = C.c_int64()
        name, metric = C.create_string_buffer(1 << 20), C.create_string_buffer(16)
        check(lib.mv_ivfpq_snapshot_info(h, name, len(name), metric, len(metric), None, C.byref(n)))
        u = np.zeros(max(n.value, 1), np.int64)
        check(lib.mv_ivfpq_snapshot_info(h, None, 0, None, 0, _p(u), None))
        m = metric.value.decode()
        self.metric_type = METRIC_L2 if m == "l2" else METRIC_IP
        self.collection = (name.value.decode("utf-8"), m, u[: n.value])
        return self

    def search(self, x, k: int, filter=None, form=None, nprobe: int = 0, rerank: int = 0,
               coarse_fp32: bool = False, lut_fp16: bool = False, coarse_path: int = 0,
               rerank_fp32: bool = False, distances=None, labels=None, lut=None):
        x = _f32(x, self.d)
        n = x.shape[0]
        dist = _out(distances, n, k, np.float32, "distances")
        lab = _out(labels, n, k, np.int64, "labels")
        flt = None if filter is None else np.ascontiguousarray(filter, dtype=np.uint8)
        p = _params(form, nprobe, rerank, coarse_fp32, lut_fp16, coarse_path,
                    rerank_fp32=rerank_fp32, lut=lut)
        check(_lib.load().mv_ivfpq_search(self._h, _p(x), n, k, _p(flt),
                                          0 if flt is None else flt.size, C.byref(p), _p(dist),
                                          _p(lab)))
        return dist, lab

    def search_batch(self, x, nprobe, k, rerank: int = 0, coarse_fp32: bool = False, lut=None):
        """Fast-form search with per-query nprobe and k (mv_ivfpq_search_batch).
        Returns (distances, labels) of shape (n, max(k)); slots past a
        query's k read 1e38 / -1."""
        x = _f32(x, self.d)
        n = x.shape[0]
        nprobe = np.ascontiguousarray(nprobe, dtype=np.int32)
        k = np.ascontiguousarray(k, dtype=np.int32)
        kmax = int(k.max()) if n else 1
        dist = np.empty((n, kmax), np.float32)
        lab = np.empty((n, kmax), np.int64)
        p = _params(FORM_FAST, 0, rerank, coarse_fp32, lut=lut)
        check(_lib.load().mv_ivfpq_search_batch(self._h, _p(x), n, _p(nprobe), _p(k), kmax,
                                                C.byref(p), _p(dist), _p(lab)))
        return dist, lab

    def search_device(self, x_ptr: int, n: int, k: int, dist_ptr: int, lab_ptr: int,
                      stream: int = 0, form=None, nprobe: int = 0, rerank: int = 0,
                      coarse_fp32: bool = False, lut_fp16: bool = False, coarse_path: int = 0,
                      lut=None):
        """Device-pointer search (e.g. torch tensors' data_ptr())."""
        p = _params(form, nprobe, rerank, coarse_fp32, lut_fp16, coarse_path, lut=lut)
        check(_lib.load().mv_ivfpq_search_device(self._h, x_ptr, n, k, None, 0, C.byref(p),
                                                 dist_ptr, lab_ptr, stream or None))


class IndexIVFFlat:
    """IVF-Flat index on the GPU (index/index_ivf_flat.mojo:10)."""

    def __init__(self, d: int, nlist: int, metric: int = METRIC_L2, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        check(_lib.load().mv_ivfflat_create(self.ctx.handle, d, nlist, metric, C.byref(h)))
        self._h = h
        _LIVE[_TIER_INDEX].add(self)
        self.d, self.nlist, self.metric_type = d, nlist, metric

    def _release(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_ivfflat_destroy(h)
        self._h = None

    def __del__(self):
        self._release()

    @property
    def ntotal(self) -> int:
        return int(_lib.load().mv_ivfflat_ntotal(self._h))

    @property
    def nprobe(self) -> int:
        return getattr(self, "_nprobe", 1)

    @nprobe.setter
    def nprobe(self, v: int):
        check(_lib.load().mv_ivfflat_set_nprobe(self._h, int(v)))
        self._nprobe = int(v)

    def train(self, x, niter: int = 15, form=None):
        x = _f32(x, self.d)
        p = _params(form)
        check(_lib.load().mv_ivfflat_train(self._h, _p(x), x.shape[0], niter, C.byref(p)))

    def centroids(self):
        out = np.zeros((self.nlist, self.d), np.float32)
        check(_lib.load().mv_ivfflat_get_centroids(self._h, _p(out)))
        return out

    def add(self, x, ids=None):
        x = _f32(x, self.d)
        if ids is None:
            check(_lib.load().mv_ivfflat_add(self._h, _p(x), x.shape[0]))
        else:
            ids = np.ascontiguousarray(ids, dtype=np.int64)
            check(_lib.load().mv_ivfflat_add_with_ids(self._h, _p(x), _p(ids), x.shape[0]))

    def search(self, x, k: int, nprobe: int = 0, form=None, distances=None, labels=None):
        x = _f32(x, self.d)
        n = x.shape[0]
        dist = _out(distances, n, k, np.float32, "distances")
        lab = _out(labels, n, k, np.int64, "labels")
        p = _params(form, nprobe)
        check(_lib.load().mv_ivfflat_search(self._h, _p(x), n, k, C.byref(p), _p(dist), _p(lab)))
        return dist, lab

    def search_device(self, x_ptr: int, n: int, k: int, dist_ptr: int, lab_ptr: int,
                      stream: int = 0, nprobe: int = 0, form=None):
        p = _params(form, nprobe)
        check(_lib.load().mv_ivfflat_search_device(self._h, x_ptr, n, k, C.byref(p), dist_ptr,
                                                   lab_ptr, stream or None))


class IndexFlat:
    """Exact index over raw FP32 rows (index/index_flat.mojo:117)."""

    def __init__(self, d: int, metric: int = METRIC_L2, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        check(_lib.load().mv_flat_create(self.ctx.handle, d, metric, C.byref(h)))
        self._h = h
        _LIVE[_TIER_INDEX].add(self)
        self.d, self.metric_type = d, metric

    def _release(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_flat_destroy(h)
        self._h = None

    def __del__(self):
        self._release()

    @property
    def ntotal(self) -> int:
        return int(_lib.load().mv_flat_ntotal(self._h))

    def add(self, x):
        x = _f32(x, self.d)
        check(_lib.load().mv_flat_add(self._h, _p(x), x.shape[0]))

    def search(self, x, k: int, filter=None, form=None, rerank: int = 0, plain_scan: bool = False,
               e4m3: bool = False, distances=None, labels=None):
        """IndexFlat.search. The plain form returns the reference's exact
        results, from the certified tensor-core shortlist where it applies;
        plain_scan=True runs the exact FP32 scan alone. The fast form takes
        its shortlist from a BF16 GEMM, or with e4m3=True an FP8 one.
        distances / labels: optional caller-provided result arrays."""
        x = _f32(x, self.d)
        n = x.shape[0]
        dist = _out(distances, n, k, np.float32, "distances")
        lab = _out(labels, n, k, np.int64, "labels")
        flt = None if filter is None else np.ascontiguousarray(filter, dtype=np.uint8)
        p = _params(form, 0, rerank, plain_scan=plain_scan, e4m3=e4m3)
        check(_lib.load().mv_flat_search(self._h, _p(x), n, k, _p(flt), C.byref(p), _p(dist),
                                         _p(lab)))
        return dist, lab

    def rerank(self, x, cand, k: int):
        """Exact FP32 rerank of candidate ids (n, ncand; -1 = empty) against
        this index's rows (the HNSW SQ8 shortlist rerank)."""
        x = _f32(x, self.d)
        n = x.shape[0]
        cand = np.ascontiguousarray(cand, dtype=np.int64).reshape(n, -1)
        dist = np.empty((n, k), np.float32)
        lab = np.empty((n, k), np.int64)
        check(_lib.load().mv_flat_rerank(self._h, _p(x), n, _p(cand), cand.shape[1], k, _p(dist),
                                         _p(lab)))
        return dist, lab

    def search_device(self, x_ptr: int, n: int, k: int, dist_ptr: int, lab_ptr: int,
                      stream: int = 0, form=None, rerank: int = 0, plain_scan: bool = False,
                      e4m3: bool = False):
        p = _params(form, 0, rerank, plain_scan=plain_scan, e4m3=e4m3)
        check(_lib.load().mv_flat_search_device(self._h, x_ptr, n, k, None, C.byref(p), dist_ptr,
                                                lab_ptr, stream or None))

    def rerank_device(self, x_ptr: int, n: int, cand_ptr: int, ncand: int, k: int, dist_ptr: int,
                      lab_ptr: int, stream: int = 0):
        """rerank with device buffers (n x ncand int64 candidate ids)."""
        check(_lib.load().mv_flat_rerank_device(self._h, x_ptr, n, cand_ptr, ncand, k, dist_ptr,
                                                lab_ptr, stream or None))


class IndexFlatSQ8:
    """SQ8 brute-force index (index/index_flat_sq8.mojo:271)."""

    def __init__(self, d: int, metric: int = METRIC_L2, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        check(_lib.load().mv_sq8_create(self.ctx.handle, d, metric, C.byref(h)))
        self._h = h
        _LIVE[_TIER_INDEX].add(self)
        self.d, self.metric_type = d, metric

    def _release(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_sq8_destroy(h)
        self._h = None

    def __del__(self):
        self._release()

    def _params(self):
        out = np.zeros(3, np.float32)
        check(_lib.load().mv_sq8_params(self._h, _p(out)))
        return out

    @property
    def global_min(self) -> float:
        return float(self._params()[0])

    @property
    def global_max(self) -> float:
        return float(self._params()[1])

    @property
    def scale(self) -> float:
        return float(self._params()[2])

    @property
    def ntotal(self) -> int:
        return int(_lib.load().mv_sq8_ntotal(self._h))

    def add(self, x):
        x = _f32(x, self.d)
        check(_lib.load().mv_sq8_add(self._h, _p(x), x.shape[0]))

    def codes(self):
        n = self.ntotal
        c = np.zeros((max(n, 1), self.d), np.uint8)
        nm = np.zeros(max(n, 1), np.uint32)
        check(_lib.load().mv_sq8_get_codes(self._h, _p(c), _p(nm)))
        return c[:n], nm[:n]

    def search(self, x, k: int, filter=None, form=None, rerank_factor: int = 0,
               plain_scan: bool = False, distances=None, labels=None):
        """IndexFlatSQ8.search; with rerank_factor > 0 the shortlist of
        k * rerank_factor is reranked with exact FP32 distances. Both forms
        take the shortlist from the tensor cores where that is exact (the
        same results as the integer scan); plain_scan=True runs the integer
        scan alone. distances / labels: optional caller-provided result
        arrays."""
        x = _f32(x, self.d)
        n = x.shape[0]
        dist = _out(distances, n, k, np.float32, "distances")
        lab = _out(labels, n, k, np.int64, "labels")
        flt = None if filter is None else np.ascontiguousarray(filter, dtype=np.uint8)
        if form is None and rerank_factor == 0 and not plain_scan:
            check(_lib.load().mv_sq8_search(self._h, _p(x), n, k, _p(flt), _p(dist), _p(lab)))
        else:
            p = _params(form, plain_scan=plain_scan)
            check(_lib.load().mv_sq8_search_ex(self._h, _p(x), n, k, _p(flt), rerank_factor,
                                               C.byref(p), _p(dist), _p(lab)))
        return dist, lab

    def search_device(self, x_ptr: int, n: int, k: int, dist_ptr: int, lab_ptr: int,
                      stream: int = 0, form=None, rerank_factor: int = 0, filter_ptr: int = 0,
                      plain_scan: bool = False):
        p = _params(form, plain_scan=plain_scan)
        check(_lib.load().mv_sq8_search_device(self._h, x_ptr, n, k, filter_ptr or None,
                                               rerank_factor, C.byref(p), dist_ptr, lab_ptr,
                                               stream or None))

    def search_rerank(self, x, k: int, rerank_factor: int = 2):
        x = _f32(x, self.d)
        n = x.shape[0]
        dist = np.empty((n, k), np.float32)
        lab = np.empty((n, k), np.int64)
        check(_lib.load().mv_sq8_search_rerank(self._h, _p(x), n, k, rerank_factor, _p(dist),
                                               _p(lab)))
        return dist, lab


class KMeans:
    """KMeans(d, k, niter) (clustering/kmeans.mojo:8). form=None/FORM_PLAIN is
    the reference-exact form; FORM_FAST assigns on the tensor cores with an
    exact FP32 recheck and sums in FP64. After train, `objective` holds the
    sum of squared distances at each assignment step and for the final
    centroids (niter + 1 values)."""

    def __init__(self, d: int, k: int, niter: int = 15, ctx: Context | None = None, form=None):
        self.ctx = ctx or Context.default()
        self.d, self.k, self.niter, self.form = d, k, niter, form
        self.centroids = np.zeros((k, d), np.float32)
        self.assignments = np.zeros(0, np.int64)
        self.objective = np.zeros(0, np.float64)

    def train(self, x):
        x = _f32(x, self.d)
        n = x.shape[0]
        self.assignments = np.zeros(n, np.int64)
        self.objective = np.zeros(self.niter + 1, np.float64)
        p = _params(self.form)
        check(_lib.load().mv_kmeans_train_ex(self.ctx.handle, _p(x), n, self.d, self.k,
                                             self.niter, C.byref(p), _p(self.centroids),
                                             _p(self.assignments), _p(self.objective)))
        return self.centroids


class ProductQuantizer:
    """ProductQuantizer(d, M, 256) (quantization/pq.mojo:80)."""

    def __init__(self, d: int, M: int, ksub: int = 256, ctx: Context | None = None):
        if ksub != 256:
            raise ValueError("the GPU product quantizer uses 256 centroids per subspace")
        if M <= 0 or M > d or d % M != 0:
            raise ValueError("PQ M must divide dimension and be between 1 and dimension.")
        self.ctx = ctx or Context.default()
        self.d, self.M, self.ksub, self.dsub = d, M, ksub, d // M
        self.centroids = np.zeros((M, ksub, d // M), np.float32)
        self.is_trained = False

    def train(self, x, niter: int = 15):
        x = _f32(x, self.d)
        check(_lib.load().mv_pq_train(self.ctx.handle, _p(x), x.shape[0], self.d, self.M, niter,
                                      _p(self.centroids)))
        self.is_trained = True

    def compute_codes(self, x):
        x = _f32(x, self.d)
        n = x.shape[0]
        codes = np.zeros((n, self.M), np.uint8)
        check(_lib.load().mv_pq_encode(self.ctx.handle, _p(self.centroids), self.d, self.M, _p(x),
                                       n, _p(codes)))
        return codes

    def decode(self, codes):
        codes = np.asarray(codes, np.uint8).reshape(-1, self.M)
        out = np.empty((codes.shape[0], self.M, self.dsub), np.float32)
        for m in range(self.M):
            out[:, m, :] = self.centroids[m][codes[:, m]]
        return out.reshape(codes.shape[0], self.d)

    def compute_distance_table(self, x, metric: int = METRIC_L2):
        x = _f32(x, self.d)
        n = x.shape[0]
        t = np.zeros((n, self.M, self.ksub), np.float32)
        check(_lib.load().mv_pq_distance_tables(self.ctx.handle, _p(self.centroids), self.d,
                                                self.M, _p(x), n, metric, _p(t)))
        return t


def sq8_encode(x, minimum: float, inverse_scale: float, symmetric: bool, ctx: Context | None = None):
    """_encode_sq8_batch (quantization/sq8.mojo:41-59) on the GPU."""
    ctx = ctx or Context.default()
    x = _f32(x)
    n, d = x.shape
    codes = np.zeros((n, d), np.uint8)
    norms = np.zeros(n, np.uint32)
    check(_lib.load().mv_sq8_encode(ctx.handle, _p(x), n, d, minimum, inverse_scale,
                                    1 if symmetric else 0, _p(codes), _p(norms)))
    return codes, norms


def distance_matrix(x, y, metric: int = METRIC_L2, precision: int = 0,
                    ctx: Context | None = None):
    """Distances between the rows of x and y: precision 0 = exact FP32 in the
    reference order, 1 = BF16 tensor cores with FP32 accumulation."""
    ctx = ctx or Context.default()
    x = _f32(x)
    y = _f32(y)
    assert x.shape[1] == y.shape[1]
    out = np.empty((x.shape[0], y.shape[0]), np.float32)
    check(_lib.load().mv_distance_matrix(ctx.handle, _p(x), x.shape[0], _p(y), y.shape[0],
                                         x.shape[1], metric, precision, _p(out)))
    return out


def normalize(x, ctx: Context | None = None):
    """_normalize_vectors (api/collection_vector_query.mojo:24-46) on the GPU."""
    ctx = ctx or Context.default()
    x = _f32(x)
    out = np.empty_like(x)
    st = _lib.load().mv_normalize(ctx.handle, _p(x), x.shape[0], x.shape[1], _p(out))
    if st != 0:
        raise ValueError(_lib.last_error())
    return out


class IVFPQBatchPlan:
    """A batched fast IVF-PQ search replayed as a CUDA graph
    (mv_ivfpq_plan_*): per-query nprobe and k, persistent scan, tuner."""

    def __init__(self, index: IndexIVFPQ, max_nq: int, nprobe_max: int, kmax: int,
                 rerank: int = 0, coarse_fp32: bool = False, lut=None):
        self.index = index
        self.max_nq, self.kmax, self.d = max_nq, kmax, index.d
        h = C.c_void_p()
        p = _params(FORM_FAST, 0, rerank, coarse_fp32, lut=lut)
        check(_lib.load().mv_ivfpq_plan_create(index._h, max_nq, nprobe_max, kmax, C.byref(p),
                                               C.byref(h)))
        self._h = h
        _LIVE[_TIER_PLAN].add(self)
        ptrs = [C.c_void_p() for _ in range(6)]
        check(_lib.load().mv_ivfpq_plan_buffers(h, *[C.byref(q) for q in ptrs]))
        (self.d_x, self.d_nprobe, self.d_k, self.d_order, self.d_dist,
         self.d_labels) = [q.value for q in ptrs]

    def _release(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_ivfpq_plan_destroy(h)
        self._h = None

    def __del__(self):
        self._release()

    def set_queries(self, x, nprobe, k):
        """Host queries (or None when d_x was filled on the device), per-query
        nprobe and k."""
        n = len(nprobe)
        xp = None
        if x is not None:
            x = _f32(x, self.d)
            xp = _p(x)
        nprobe = np.ascontiguousarray(nprobe, dtype=np.int32)
        k = np.ascontiguousarray(k, dtype=np.int32)
        check(_lib.load().mv_ivfpq_plan_set_queries(self._h, xp, n, _p(nprobe), _p(k)))

    def tune(self, n: int):
        cfg = np.zeros(3, np.int32)
        ms = C.c_float(0.0)
        check(_lib.load().mv_ivfpq_plan_tune(self._h, n, _p(cfg), C.byref(ms)))
        return {"coarse_matrix": bool(cfg[0]), "scan_threads": int(cfg[1]),
                "scan_ctas_per_sm": int(cfg[2]), "best_ms": float(ms.value)}

    def run(self, n: int, use_graph: bool = True, stream: int = 0):
        check(_lib.load().mv_ivfpq_plan_run(self._h, n, 1 if use_graph else 0, stream or None))

    def results(self, n: int, distances=None, labels=None):
        """Copies the first n result rows to the host (synchronous), into the
        caller's (n, kmax) arrays when given (pinned memory copies fastest)."""
        dist = _out(distances, n, self.kmax, np.float32, "distances")
        lab = _out(labels, n, self.kmax, np.int64, "labels")
        check(_lib.load().mv_ivfpq_plan_results(self._h, n, _p(dist), _p(lab)))
        return dist, lab


class Server:
    """Continuous-batching serving loop over resident collections
    (mv_server_*). submit() returns a request id at once; wait() blocks and
    returns (distances, labels, latency_s)."""

    def __init__(self, ctx: Context | None = None, hbm_budget: int = 8 << 30, lanes: int = 4,
                 max_batch_queries: int = 4096):
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        check(_lib.load().mv_server_create(self.ctx.handle, int(hbm_budget), lanes,
                                           max_batch_queries, C.byref(h)))
        self._h = h
        _LIVE[_TIER_SERVER].add(self)
        self._dims = {}
        self._pending = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.mv_server_destroy(h)
        self._h = None

    _release = close

    def __del__(self):
        self.close()

    def add(self, index, form=None, nprobe: int = 0, rerank: int = 0, rerank_factor: int = 0):
        cid = C.c_int32(0)
        p = _params(form, nprobe, rerank)
        lib = _lib.load()
        if isinstance(index, IndexIVFPQ):
            check(lib.mv_server_add_ivfpq(self._h, index._h, C.byref(p), C.byref(cid)))
        elif isinstance(index, IndexFlat):
            check(lib.mv_server_add_flat(self._h, index._h, C.byref(p), C.byref(cid)))
        elif isinstance(index, IndexFlatSQ8):
            check(lib.mv_server_add_sq8(self._h, index._h, rerank_factor, C.byref(p),
                                        C.byref(cid)))
        else:
            raise TypeError("unsupported index type")
        self._dims[cid.value] = index.d
        return cid.value

    def submit(self, coll: int, x, k: int) -> int:
        x = _f32(x, self._dims[coll])
        n = x.shape[0]
        dist = np.empty((n, k), np.float32)
        lab = np.empty((n, k), np.int64)
        rid = C.c_int64(0)
        check(_lib.load().mv_server_submit(self._h, coll, _p(x), n, k, _p(dist), _p(lab),
                                           C.byref(rid)))
        self._pending[rid.value] = (dist, lab)
        return rid.value

    def wait(self, rid: int):
        lat = C.c_double(0.0)
        st = _lib.load().mv_server_wait(self._h, rid, C.byref(lat))
        dist, lab = self._pending.pop(rid)
        check(st)
        return dist, lab, lat.value

    def device_overlap(self):
        """(peak batches on the device at one instant, batches recorded)."""
        out = np.zeros(2, np.int64)
        check(_lib.load().mv_server_device_overlap(self._h, _p(out)))
        return int(out[0]), int(out[1])

    def stats(self):
        out = np.zeros(4, np.int64)
        check(_lib.load().mv_server_stats(self._h, _p(out)))
        return {"completed": int(out[0]), "batches": int(out[1]), "batched_queries": int(out[2]),
                "peak_inflight_bytes": int(out[3])}
