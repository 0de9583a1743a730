"""IVFPQCollection: the managed IVF-PQ collection facade on the GPU.

Mirrors python/mojovec/_ivfpq.py:28-218 (method names and arguments) and the
semantics of mojovec/api/collection_ivfpq.mojo:
  * validation and error messages (collection_ivfpq.mojo:37-49, :176-185,
    :197-204, :259-264);
  * cosine rows L2-normalised in FP64 (api/collection_vector_query.mojo:24-46)
    and searched with the inner-product index metric (collection_codec.mojo:42);
  * auto-train on the first add (collection_ivfpq.mojo:228-229);
  * internal sequential ids mapped to user ids, and 1 - d distances for
    cosine / ip (collection_ivfpq.mojo:307-326).
"""

from __future__ import annotations

import numpy as np

from . import index as _index
from ._lib import METRIC_IP, METRIC_L2

MAX_IVF_NLIST = 1_000_000
MAX_IVF_NPROBE = 65_536
MAX_QUERY_RESULTS = 2_048
PQ_CENTROIDS = 256
_METRICS = {"l2": METRIC_L2, "cosine": 2, "ip": METRIC_IP}


def _validate(dimension, nlist, M, nprobe):
    if dimension <= 0 or dimension > 65_536:
        raise ValueError("dimension must be between 1 and 65536.")
    if nlist <= 0 or nlist > MAX_IVF_NLIST:
        raise ValueError("nlist must be between 1 and 1000000.")
    if M <= 0 or M > dimension or dimension % M != 0:
        raise ValueError("M must divide dimension and be between 1 and dimension.")
    if nprobe <= 0 or nprobe > nlist or nprobe > MAX_IVF_NPROBE:
        raise ValueError("nprobe must be between 1 and nlist.")


def _flatten(embeddings, dimension):
    arr = np.asarray(embeddings, dtype=np.float32)
    if arr.ndim == 1:
        if arr.size % dimension != 0:
            raise ValueError(f"embeddings length must be a multiple of {dimension}")
        arr = arr.reshape(-1, dimension)
    if arr.ndim != 2 or arr.shape[1] != dimension:
        raise ValueError(f"embeddings rows have {arr.shape[-1]} values; expected {dimension}")
    return np.ascontiguousarray(arr)


class IVFPQCollection:
    """Compressed IVF-PQ vector collection served by libmojovec_gpu."""

    def __init__(self, dimension: int, nlist: int = 100, pq_subvectors: int = 16,
                 nprobe: int | None = None, metric: str = "l2", name: str = "",
                 ctx: _index.Context | None = None):
        eff = min(10, nlist) if not nprobe else nprobe  # collection_ivfpq.mojo:77
        _validate(dimension, nlist, pq_subvectors, eff)
        if metric not in _METRICS:
            raise ValueError('metric must be "l2", "cosine", or "ip".')
        self._name = name
        self._dimension = dimension
        self._metric = metric
        index_metric = METRIC_IP if metric in ("cosine", "ip") else METRIC_L2
        self._index = _index.IndexIVFPQ(dimension, nlist, pq_subvectors, index_metric, ctx)
        self._index.nprobe = eff
        self._user_ids: list[int] = []
        self._id_to_internal: dict[int, int] = {}
        self.search_options: dict = {}

    def __repr__(self) -> str:
        return (
            f"IVFPQCollection(name={self.name()!r}, dimension={self.dimension()}, "
            f"metric={self.metric()!r}, count={self.count()}, nlist={self.nlist()}, "
            f"pq_subvectors={self.pq_subvectors()}, nprobe={self.nprobe()}, "
            f"trained={self.is_trained()})"
        )

    def name(self) -> str:
        return self._name

    def dimension(self) -> int:
        return self._dimension

    def metric(self) -> str:
        return self._metric

    def count(self) -> int:
        return len(self._user_ids)

    def is_trained(self) -> bool:
        return self._index.is_trained

    def nlist(self) -> int:
        return self._index.nlist

    def pq_subvectors(self) -> int:
        return self._index.M

    def nprobe(self) -> int:
        return self._index.nprobe

    def set_nprobe(self, nprobe: int) -> None:
        if nprobe <= 0 or nprobe > self.nlist():
            raise ValueError("nprobe must be between 1 and nlist.")
        self._index.nprobe = nprobe

    def stats(self) -> dict:
        return {
            "count": self.count(),
            "dimension": self._dimension,
            "nlist": self.nlist(),
            "M": self.pq_subvectors(),
            "nprobe": self.nprobe(),
            "trained": self.is_trained(),
            "metric": self.metric(),
            "code_size_bytes": self.pq_subvectors(),
        }

    # -- preparation ------------------------------------------------------
    def _prepare(self, rows: np.ndarray) -> np.ndarray:
        if self._metric == "cosine":
            return _index.normalize(rows, self._index.ctx)
        if rows.size and not np.isfinite(rows).all():
            raise ValueError("Vector components must be finite.")
        return rows

    # -- training / ingest -------------------------------------------------
    def train(self, embeddings) -> None:
        self._train_rows(_flatten(embeddings, self._dimension))

    def train_numpy(self, embeddings) -> None:
        arr = np.asarray(embeddings)
        if (arr.dtype != np.float32 or arr.ndim != 2 or arr.shape[1] != self._dimension
                or not arr.flags.c_contiguous):
            raise TypeError("embeddings must be a contiguous (n, dimension) numpy.float32 array")
        self._train_rows(arr)

    def _train_rows(self, rows: np.ndarray) -> None:
        minimum = max(self.nlist(), PQ_CENTROIDS)
        if rows.shape[0] < minimum:
            raise ValueError("IVF-PQ training requires at least max(nlist, 256) vectors.")
        if self.is_trained():
            return
        self._index.train(self._prepare(rows))

    def add(self, ids, embeddings) -> None:
        rows = _flatten(embeddings, self._dimension)
        if len(ids) != rows.shape[0]:
            raise ValueError(
                f"embeddings contain {rows.size} values; expected {len(ids) * self._dimension}")
        self._add_rows(list(int(i) for i in ids), rows)

    def add_numpy(self, ids, embeddings) -> None:
        ids_arr = np.asarray(ids)
        if ids_arr.dtype != np.int64:
            raise TypeError("ids must be a numpy.int64 array")
        rows = np.asarray(embeddings)
        if rows.dtype != np.float32:
            raise TypeError("embeddings must have numpy.float32 dtype")
        rows = rows.reshape(-1, self._dimension)
        self._add_rows(ids_arr.tolist(), np.ascontiguousarray(rows))

    def _add_rows(self, ids: list[int], rows: np.ndarray) -> None:
        if rows.shape[0] != len(ids):
            raise ValueError("Embeddings length must equal len(ids) * dimension.")
        if not ids:
            return
        seen = set()
        for rid in ids:  # collection_ivfpq.mojo:197-204
            if rid in seen:
                raise ValueError("Duplicate IDs are not allowed within an add batch.")
            if rid in self._id_to_internal:
                raise ValueError("Cannot add an ID that already exists.")
            seen.add(rid)
        if not self.is_trained():
            self._train_rows(rows)
        self._index.add(self._prepare(rows))
        for rid in ids:
            self._id_to_internal[rid] = len(self._user_ids)
            self._user_ids.append(rid)

    # -- query ------------------------------------------------------------
    def query(self, query_embeddings, n_results: int = 10) -> dict:
        return self._query_rows(_flatten(query_embeddings, self._dimension), n_results)

    def query_numpy(self, query_embeddings, n_results: int = 10) -> dict:
        arr = np.asarray(query_embeddings)
        if arr.dtype != np.float32:
            raise TypeError("query_embeddings must have numpy.float32 dtype")
        if arr.ndim == 1:
            if arr.size % self._dimension != 0:
                raise ValueError("query embeddings length must be a multiple of dimension")
            arr = arr.reshape(-1, self._dimension)
        if arr.ndim != 2 or arr.shape[1] != self._dimension or not arr.flags.c_contiguous:
            raise ValueError("query_embeddings must be a contiguous (n, dimension) array")
        return self._query_rows(arr, n_results)

    def _query_rows(self, rows: np.ndarray, n_results: int) -> dict:
        if n_results <= 0 or n_results > MAX_QUERY_RESULTS:
            raise ValueError("n_results must be between 1 and 2048.")
        if rows.shape[0] == 0:
            return {"ids": [], "distances": [], "metadatas": [], "documents": [], "scores": []}
        dist, lab = self._index.search(self._prepare(rows), n_results, **self.search_options)
        user = np.asarray(self._user_ids + [-1], dtype=np.int64)
        valid = (lab >= 0) & (lab < len(self._user_ids))
        ids = np.where(valid, user[np.where(valid, lab, len(self._user_ids))], -1)
        if self._metric != "l2":
            dist = np.where(valid, np.float32(1.0) - dist, dist)
        return {
            "ids": ids.tolist(),
            "distances": dist.astype(np.float32).tolist(),
            "metadatas": [],
            "documents": [],
            "scores": [],
        }
