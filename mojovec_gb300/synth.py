"""Seeded synthetic workloads standing in for SIFT-like data.

No public dataset is read. The generators follow the shapes and value
distributions of the benchmark configurations:

* sift_like (G1): C centres uniform in [0, 128]^d; each row picks a centre
  uniformly, adds N(0, 20^2) per component, is clipped to [0, 255] and
  rounded to integers (stored as float32, like SIFT descriptors).
* cos_mixture (G2): C unit-norm centres; row = centre + N(0, std^2) per
  component, then L2-normalised.

Every stream derives from numpy PCG64 seeded with a SeedSequence and its
spawned children (centres / labels / noise / queries), so base rows and
queries are reproducible and independent.
"""

from __future__ import annotations

import numpy as np

BASE_SEED = 20261203


def _streams(seed: int, n: int):
    ss = np.random.SeedSequence(seed)
    return [np.random.Generator(np.random.PCG64(s)) for s in ss.spawn(n)]


def sift_like(n: int, d: int = 128, n_centers: int = 1024, seed: int = BASE_SEED,
              nq: int = 0, chunk: int = 1 << 18):
    """Returns (base (n, d) float32, queries (nq, d) float32)."""
    g_cent, g_lab, g_noise, g_q = _streams(seed, 4)
    centers = g_cent.uniform(0.0, 128.0, size=(n_centers, d)).astype(np.float32)

    def draw(g_l, g_n, count):
        out = np.empty((count, d), np.float32)
        for r0 in range(0, count, chunk):
            r1 = min(count, r0 + chunk)
            lab = g_l.integers(0, n_centers, size=r1 - r0)
            x = centers[lab] + g_n.standard_normal(size=(r1 - r0, d), dtype=np.float32) * np.float32(20.0)
            np.clip(x, 0.0, 255.0, out=x)
            np.rint(x, out=x)
            out[r0:r1] = x
        return out

    base = draw(g_lab, g_noise, n)
    queries = draw(g_q, g_q, nq) if nq else np.zeros((0, d), np.float32)
    return base, queries


def cos_mixture(n: int, d: int = 96, n_centers: int = 4096, std: float = 0.05,
                seed: int = BASE_SEED + 1, nq: int = 0, chunk: int = 1 << 18):
    g_cent, g_lab, g_noise, g_q = _streams(seed, 4)
    centers = g_cent.standard_normal(size=(n_centers, d)).astype(np.float32)
    centers /= np.linalg.norm(centers, axis=1, keepdims=True)

    def draw(g_l, g_n, count):
        out = np.empty((count, d), np.float32)
        for r0 in range(0, count, chunk):
            r1 = min(count, r0 + chunk)
            lab = g_l.integers(0, n_centers, size=r1 - r0)
            x = centers[lab] + g_n.standard_normal(size=(r1 - r0, d), dtype=np.float32) * np.float32(std)
            x /= np.linalg.norm(x, axis=1, keepdims=True)
            out[r0:r1] = x
        return out

    base = draw(g_lab, g_noise, n)
    queries = draw(g_q, g_q, nq) if nq else np.zeros((0, d), np.float32)
    return base, queries


def sample_rows(n: int, m: int, seed: int = BASE_SEED + 3) -> np.ndarray:
    """Row indices of a training sample: the first m of a seeded permutation
    of range(n), in permutation order."""
    g = np.random.Generator(np.random.PCG64(np.random.SeedSequence(seed)))
    return g.permutation(n)[:m]


def grid_vectors(count: int = 256, dimension: int = 8) -> np.ndarray:
    """The integer-pattern rows used by the reference's IVF-PQ tests
    (tests/test_ivf_pq.mojo:30-38): ((r*17 + c*29) % 251) / 251 + 2*[c == r % d]."""
    r = np.arange(count)[:, None]
    c = np.arange(dimension)[None, :]
    v = ((r * 17 + c * 29) % 251).astype(np.float32) / np.float32(251.0)
    v = v + np.where(c == r % dimension, np.float32(2.0), np.float32(0.0))
    return v.astype(np.float32)
