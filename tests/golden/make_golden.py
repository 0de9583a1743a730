"""Generates the golden fixtures in tests/golden/ from the oracle.

The reference (Mojo) cannot run in this image, so the fixtures are the
oracle's own outputs on small seeded inputs. They pin the oracle against
regressions (a change in the restated operation order changes these bits)
and are the expected values of the GPU parity tests at these sizes.

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from mojovec_gb300 import synth  # noqa: E402


def make():
    out = {}
    # Philox stream of the k-means seed (clustering/kmeans.mojo:70)
    out["philox_kmeans_seed_steps"] = orc.philox_steps(0x4D4F4A4F564543, 16)

    # Distance kernels on odd and exact dimensions (utils/distances.mojo)
    rng = np.random.default_rng(1234)
    for d in (1, 3, 4, 7, 8, 12, 31, 32, 33, 96, 128, 130, 257):
        x = rng.standard_normal(d).astype(np.float32) * 3
        y = rng.standard_normal(d).astype(np.float32) * 3
        out[f"dist_d{d}"] = np.array(
            [orc.l2_simd(x, y, 8), orc.ip_simd(x, y, 8), orc.l2_simd(x, y, 4),
             orc.ip_simd(x, y, 4), orc.l2_simd(x, y, 64), orc.ip_simd(x, y, 64)],
            np.float32)
        out[f"dist_d{d}_x"] = x
        out[f"dist_d{d}_y"] = y

    # IVF-PQ on the reference test grid (tests/test_ivf_pq.mojo:30-38)
    rows = synth.grid_vectors()
    ix = orc.IVFPQ(8, 8, 2)
    ix.train(rows, niter_coarse=15, niter_pq=15)
    ix.add(rows)
    cent, pq = ix.codebooks()
    off, ids, codes = ix.lists()
    d, lab = ix.search(rows[:16], 5, 4)
    out.update(grid_centroids=cent, grid_pq=pq, grid_offsets=off, grid_ids=ids, grid_codes=codes,
               grid_dist=d, grid_labels=lab)

    # SIFT-like IVF-PQ (integer data, many ties)
    base, q = synth.sift_like(4000, d=32, n_centers=40, nq=40, seed=3)
    ix2 = orc.IVFPQ(32, 16, 8)
    ix2.train(base, niter_coarse=6, niter_pq=6)
    ix2.add(base)
    d2, l2 = ix2.search(q, 10, 3)
    out.update(sift_queries=q, sift_dist=d2, sift_labels=l2)
    c2, p2 = ix2.codebooks()
    out.update(sift_centroids=c2, sift_pq=p2)

    # K-means (tests/test_kmeans.mojo:48-72 data)
    i = np.arange(257 * 8)
    x = (((i * 37 + (i // 8) * 11) % 101) / 50.0 - 1.0).astype(np.float32).reshape(257, 8)
    kc, ka = orc.kmeans_train(x, 17, niter=5)
    out.update(kmeans_x=x, kmeans_centroids=kc, kmeans_assign=ka)

    # SQ8 with a requantising second batch (index/index_flat_sq8.mojo:365-476)
    r = np.random.default_rng(99)
    a = (r.standard_normal((50, 16)) * 2).astype(np.float32)
    b = (r.standard_normal((40, 16)) * 3).astype(np.float32)
    for metric in (0, 1):
        s = orc.SQ8(16, metric)
        s.add(a)
        s.add(b)
        codes, norms = s.codes()
        dd, ll = s.search(a[:8], 5)
        out[f"sq8_m{metric}_params"] = np.array(s.params(), np.float32)
        out[f"sq8_m{metric}_codes"] = codes
        out[f"sq8_m{metric}_norms"] = norms
        out[f"sq8_m{metric}_dist"] = dd
        out[f"sq8_m{metric}_labels"] = ll
    out.update(sq8_a=a, sq8_b=b)
    return out


if __name__ == "__main__":
    data = make()
    path = os.path.join(HERE, "oracle_golden.npz")
    np.savez_compressed(path, **data)
    print(path, len(data), "arrays", os.path.getsize(path), "bytes")
