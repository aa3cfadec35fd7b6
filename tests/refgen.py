"""Seeded input generators of the reference, restated for the tests.

The reference's exactness check and its synthetic benchmark build their inputs
with numpy ``default_rng``; the same draws in the same order give the same
profiles, so these restatements let the tests rebuild the reference's inputs
without the reference present. ``tests/golden/`` holds the SHA-256 of what the
reference's own code produced, and ``test_refgen.py`` checks these
restatements against it.

* ``checkpy_make``  tensorcore/rs/check.py:17-36 (awkward cells: '-', '',
  'LNF', 'PLOT3', 'INF-' prefixes, optional 32-bit multiplicative hash)
* ``checkpy_tsv``   tensorcore/rs/check.py:63-66 (file layout)
* ``gen_profiles``  python/gen_profiles.py:3-12 (50 founders, ~3% mutated
  loci, 2% missing; the synthetic 30 000 x 5 000 set of the published checksum)
"""
from __future__ import annotations

import numpy as np


def checkpy_make(n: int, L: int, seed: int, hashed: bool):
    """Return (A, cells): A is the n x L int64 allele matrix (0 = missing) and
    cells the rendered strings, drawn in check.py's order."""
    rng = np.random.default_rng(seed)
    founders = rng.integers(1, 30, size=(8, L))
    A = founders[rng.integers(0, 8, n)]
    m = rng.random((n, L)) < 0.15
    A[m] = rng.integers(1, 2000, m.sum())
    A[rng.random((n, L)) < 0.05] = 0
    if hashed:
        A = np.where(A > 0, (A * 2654435761) % 4294967291 + 1, 0)
    # one uniform per cell, row-major, exactly as the nested loop draws them
    U = rng.random(n * L).reshape(n, L) if n * L else np.zeros((n, L))
    cells = []
    for r in range(n):
        row = []
        for k in range(L):
            v, u = int(A[r, k]), U[r, k]
            if v == 0:
                row.append("-" if u < 0.4 else "" if u < 0.6 else "LNF" if u < 0.8 else "PLOT3")
            else:
                row.append(f"INF-{v}" if u < 0.1 else str(v))
        cells.append(row)
    return A, cells


def checkpy_tsv(cells, L: int) -> str:
    out = ["FILE\t" + "\t".join(f"L{j}" for j in range(L)) + "\n"]
    for i, row in enumerate(cells):
        out.append(f"S{i}\t" + "\t".join(row) + "\n")
    return "".join(out)


CHECKPY_CASES = [(300, 97, 1, False), (700, 410, 2, True), (1500, 64, 3, False)]

# check.py:69-78: (extra CLI args, expected-matrix transform name)
CHECKPY_FLAGSETS = [
    ([], "full"),
    (["--tau", "2"], "full"),
    (["--tau", "100000"], "full"),
    (["--stripe", "64"], "full"),
    (["-m", "lower-tri"], "lower"),
    (["-m", "upper-tri"], "upper"),
    (["-X", "7"], "cap7"),
    (["-D", ","], "full"),
]


def checkpy_expected(H: np.ndarray, kind: str) -> np.ndarray:
    """check.py:69-78: the matrix the CLI must print for each flag set."""
    iu = np.triu(np.ones_like(H, dtype=bool))
    if kind == "full":
        return H
    if kind == "lower":
        return np.where(iu.T, H, 0)
    if kind == "upper":
        return np.where(iu, H, 0)
    if kind == "cap7":
        return np.minimum(H, 7)
    raise ValueError(kind)


def gen_profiles(n: int, L: int) -> np.ndarray:
    """python/gen_profiles.py:3-8 (seed 1): the n x L allele matrix."""
    rng = np.random.default_rng(1)
    F = rng.integers(1, 200, size=(50, L))
    P = F[rng.integers(0, 50, n)]
    m = rng.random((n, L)) < 0.03
    P[m] = rng.integers(1, 5000, m.sum())
    P[rng.random((n, L)) < 0.02] = 0
    return P


def gen_profiles_tsv(P: np.ndarray) -> str:
    """python/gen_profiles.py:9-12."""
    n, L = P.shape
    out = ["FILE\t" + "\t".join(f"L{j}" for j in range(L)) + "\n"]
    for i, r in enumerate(P):
        out.append(f"S{i}\t" + "\t".join("-" if v == 0 else str(v) for v in r) + "\n")
    return "".join(out)


def ranks_of(A: np.ndarray) -> np.ndarray:
    """Any injective per-locus map with 0 kept as missing gives the same
    distances; this one is the reference's sorted-unique rank (main.rs:135-165)."""
    n, L = A.shape
    x = np.zeros((n, L), dtype=np.uint16)
    for k in range(L):
        col = A[:, k]
        nz = col != 0
        u = np.unique(col[nz])
        assert len(u) <= 65535
        r = np.zeros(n, dtype=np.int64)
        r[nz] = np.searchsorted(u, col[nz]) + 1
        x[:, k] = r
    return x
