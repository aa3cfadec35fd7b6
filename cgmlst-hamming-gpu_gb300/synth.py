"""Seeded synthetic cgMLST allele-call matrices of the benchmark shapes.

The reference's headline numbers are on real Campylobacter chewBBACA calls
(63 005 x 1 142), which are not available here; these generators produce
profiles with the stated shapes and value distributions instead.  Every
matrix is n x L uint64 (0 = missing), a deterministic function of the seed.

* ``small``     2 000 x 1 142: per-locus distinct-allele count lognormal with
                mean 40 (capped at 500), calls Zipf(1.1) over those alleles,
                2% missing, 32-bit ids.
* ``longtail``  63 005 x 1 142: distinct counts lognormal with median 60 and
                a tail to 3 000, calls Zipf(1.2), 1-5% missing per locus, 5% of
                each locus's allele ids replaced by hashed 64-bit values.
* ``founders``  50 000 x 5 000: 50 founder alleles per locus drawn uniformly
                (so ~250 k frequent one-hot columns), 1% of calls mutated to
                fresh rare ids, 2% missing.
* ``zipf_big``  200 000 x 3 000: Zipf(1.1), the ``small`` distinct-count law.
"""
from __future__ import annotations

import numpy as np

CONFIGS = {
    "small": dict(n=2000, L=1142),
    "longtail": dict(n=63005, L=1142),
    "founders": dict(n=50000, L=5000),
    "zipf_big": dict(n=200000, L=3000),
}


def _ids(rng, k: int, hashed_frac: float = 0.0) -> np.ndarray:
    """k distinct non-zero allele ids: u32 values, a fraction of them
    replaced by 64-bit hash-like values (>= 2^32)."""
    ids = np.unique(rng.integers(1, 2**32, size=k + 16, dtype=np.uint64))
    while len(ids) < k:
        ids = np.unique(np.concatenate([ids, rng.integers(1, 2**32, size=k, dtype=np.uint64)]))
    ids = rng.permutation(ids)[:k]
    if hashed_frac > 0:
        h = rng.random(k) < hashed_frac
        ids[h] = rng.integers(2**32, 2**64 - 1, size=int(h.sum()), dtype=np.uint64)
    return ids


def zipf_profiles(n: int, L: int, seed: int, s: float, distinct, miss, hashed_frac: float = 0.0) -> np.ndarray:
    """distinct(rng, L) -> per-locus allele counts; miss(rng, L) -> per-locus
    missing rates.  Calls are Zipf(s) over each locus's alleles."""
    rng = np.random.default_rng(seed)
    k = distinct(rng, L)
    m = miss(rng, L)
    out = np.zeros((L, n), dtype=np.uint64)
    for l in range(L):
        w = np.arange(1, k[l] + 1, dtype=np.float64) ** (-s)
        cdf = np.cumsum(w)
        cdf /= cdf[-1]
        idx = np.minimum(np.searchsorted(cdf, rng.random(n), side="right"), k[l] - 1)
        col = _ids(rng, int(k[l]), hashed_frac)[idx]
        col[rng.random(n) < m[l]] = 0
        out[l] = col
    return np.ascontiguousarray(out.T)


def small(seed: int = 1, n: int = 2000, L: int = 1142) -> np.ndarray:
    def distinct(rng, L):
        # lognormal with mean 40: mu = ln 40 - sigma^2 / 2, sigma = 1
        return np.clip(np.rint(rng.lognormal(np.log(40.0) - 0.5, 1.0, L)), 2, 500).astype(np.int64)

    return zipf_profiles(n, L, seed, 1.1, distinct, lambda rng, L: np.full(L, 0.02))


def longtail(seed: int = 2, n: int = 63005, L: int = 1142) -> np.ndarray:
    def distinct(rng, L):
        # median 60; sigma 1.26 puts the largest of ~1 000 loci near 3 000
        return np.clip(np.rint(rng.lognormal(np.log(60.0), 1.26, L)), 2, 3000).astype(np.int64)

    return zipf_profiles(n, L, seed, 1.2, distinct, lambda rng, L: rng.uniform(0.01, 0.05, L), hashed_frac=0.05)


def founders(seed: int = 3, n: int = 50000, L: int = 5000, n_founders: int = 50) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.zeros((L, n), dtype=np.uint64)
    for l in range(L):
        f = _ids(rng, n_founders)
        col = f[rng.integers(0, n_founders, n)]
        mut = rng.random(n) < 0.01
        col[mut] = rng.integers(2**32, 2**64 - 1, size=int(mut.sum()), dtype=np.uint64)  # fresh ids
        col[rng.random(n) < 0.02] = 0
        out[l] = col
    return np.ascontiguousarray(out.T)


def zipf_big(seed: int = 4, n: int = 200000, L: int = 3000) -> np.ndarray:
    def distinct(rng, L):
        return np.clip(np.rint(rng.lognormal(np.log(40.0) - 0.5, 1.0, L)), 2, 500).astype(np.int64)

    return zipf_profiles(n, L, seed, 1.1, distinct, lambda rng, L: np.full(L, 0.02))


GENERATORS = {"small": small, "longtail": longtail, "founders": founders, "zipf_big": zipf_big}


def make(name: str, seed: int | None = None, **kw) -> np.ndarray:
    g = GENERATORS[name]
    return g(**kw) if seed is None else g(seed=seed, **kw)
