"""CPU oracle for the exact cgMLST Hamming distance path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, and only as the oracle
(the reference result a GPU result is compared with, or the CPU time measured).
The product library (``libtch``) and the CLI never call it.

It restates, function by function, what the reference computes on the host
and what its exactness check compares against (paths are relative to the
reference project):

* ``parse_allele``      tensorcore/rs/src/main.rs:95-113   (cell semantics)
* ``rust_lines``        main.rs:289-292 (``str::lines`` + blank-line filter)
* ``load_tsv``          main.rs:286-311 (header, ids, cells padded to L)
* ``completeness``      main.rs:313-348 (locus, then sample filters)
* ``dense_ranks``       main.rs:134-165 (sorted unique ids -> ranks 1..k)
* ``choose_tau``        main.rs:167-198 (analytic tau, reference L4 rates)
* ``encode``            main.rs:366-444 (frequent map, bit-pack, rare CSR)
* ``hamming``           tensorcore/rs/check.py:39-44 (brute-force count)
* ``write_matrix``      main.rs:224-265 (layouts, cap, separators)
* ``rollhash``          tensorcore/tc_hamming.cu:240-241 (upper-tri checksum)

and the consumers of the matrix that the reference's documentation names
(docs/index.html, "The problem": outbreak clustering, minimum spanning trees,
nearest-neighbour searches; the reference has no code for them), from their
definitions:

* ``mst``               Prim's algorithm, edges ordered by (distance, smaller
                        index, larger index), which makes the tree unique
* ``clusters``          single linkage: components of the graph of pairs at
                        distance <= t, straight from the matrix (not via a tree)
* ``neighbors``         the k smallest (distance, index) of every row

The heavy brute-force count is in ``oracle.c`` (OpenMP); everything else is
numpy or plain Python and is meant for sizes that finish in seconds.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")
LIBPATH = os.path.join(LIBDIR, "liborc.so")

U16_MAX = 65535


class OracleError(Exception):
    """Fatal condition of the reference host (its ``die``, main.rs:129-132)."""


# --------------------------------------------------------------------------------------
# build / load of the C part
# --------------------------------------------------------------------------------------

def build(force: bool = False) -> str:
    """Compile oracle.c into lib/liborc.so with gcc -O3 -fopenmp."""
    src = os.path.join(HERE, "oracle.c")
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= os.path.getmtime(src):
        return LIBPATH
    tmp = LIBPATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp])
    os.replace(tmp, LIBPATH)
    return LIBPATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIBPATH)
        i64, u16p, u64p = ctypes.c_int64, ctypes.POINTER(ctypes.c_uint16), ctypes.POINTER(ctypes.c_uint64)
        L.orc_hamming_block.argtypes = [u16p, i64, i64, i64, i64, i64, i64, u16p, i64, ctypes.c_int]
        L.orc_hamming_block.restype = None
        L.orc_upper_rows.argtypes = [u16p, i64, i64, i64, i64, u64p, ctypes.c_int]
        L.orc_upper_rows.restype = i64
        L.orc_hamming_block_u64.argtypes = [u64p, i64, i64, i64, i64, i64, i64, u16p, i64, ctypes.c_int]
        L.orc_hamming_block_u64.restype = None
        L.orc_upper_rows_step.argtypes = [u16p, i64, i64, i64, i64, u64p, ctypes.c_int]
        L.orc_upper_rows_step.restype = i64
        L.orc_rollhash_stripe.argtypes = [ctypes.c_uint64, u16p, i64, i64, i64]
        L.orc_rollhash_stripe.restype = ctypes.c_uint64
        L.orc_rollhash_ranks.argtypes = [u16p, i64, i64, ctypes.c_int]
        L.orc_rollhash_ranks.restype = ctypes.c_uint64
        L.orc_num_threads.argtypes = []
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _u16p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))


# --------------------------------------------------------------------------------------
# cell semantics and TSV loading (main.rs:95-113, 286-311)
# --------------------------------------------------------------------------------------

# Rust's char::is_whitespace (Unicode White_Space), used by str::trim.
_WHITE_SPACE = frozenset(
    [chr(c) for c in range(0x09, 0x0E)]
    + [chr(c) for c in (0x20, 0x85, 0xA0, 0x1680)]
    + [chr(c) for c in range(0x2000, 0x200B)]
    + [chr(c) for c in (0x2028, 0x2029, 0x202F, 0x205F, 0x3000)]
)


def rust_trim(s: str) -> str:
    a, b = 0, len(s)
    while a < b and s[a] in _WHITE_SPACE:
        a += 1
    while b > a and s[b - 1] in _WHITE_SPACE:
        b -= 1
    return s[a:b]


def parse_allele(cell: str, skip_repl: bool = False, missing: str = "-") -> int:
    """main.rs:98-113: trim, strip one leading ``INF-`` (unless -r), missing
    char or empty -> 0, all ASCII digits -> u64 (overflow is fatal), else 0."""
    s = rust_trim(cell)
    if not skip_repl and s.startswith("INF-"):
        s = s[4:]
    if s == missing or s == "":
        return 0
    if all("0" <= ch <= "9" for ch in s):
        v = int(s)
        if v > 0xFFFFFFFFFFFFFFFF:
            raise OracleError(f"allele '{rust_trim(cell)}' too large")
        return v
    return 0


def rust_lines(text: str) -> list[str]:
    """str::lines: split after each '\\n', drop the '\\n' and then one '\\r'
    before it; a final segment without '\\n' is a line if non-empty."""
    out = []
    for seg in text.split("\n"):
        out.append(seg)
    if out and out[-1] == "":
        out.pop()  # text ended with '\n' (or was empty)
        trailing_nl = True
    else:
        trailing_nl = False
    res = []
    for k, seg in enumerate(out):
        terminated = k < len(out) - 1 or trailing_nl
        if terminated and seg.endswith("\r"):
            seg = seg[:-1]
        res.append(seg)
    return res


@dataclass
class Table:
    ids: list
    calls: np.ndarray  # n x L uint64, 0 = missing
    L: int


def load_tsv(text: str, sep: str = "\t", skip_repl: bool = False, missing: str = "-") -> Table:
    """main.rs:286-311."""
    lines = rust_lines(text)
    if not lines:
        raise OracleError("empty input")
    header = lines[0]
    L = len(header.split(sep)) - 1
    data = [ln for ln in lines[1:] if ln != ""]
    ids = []
    calls = np.zeros((len(data), L), dtype=np.uint64)
    for i, line in enumerate(data):
        parts = line.split(sep)
        sid = parts[0]
        vals = []
        for cell in parts[1:]:
            try:
                vals.append(parse_allele(cell, skip_repl, missing))
            except OracleError:
                raise OracleError(f"sample {sid}: allele '{rust_trim(cell)}' too large")
        vals = vals[:L] + [0] * max(0, L - len(vals))
        ids.append(sid)
        if L:
            calls[i] = np.array(vals, dtype=np.uint64)
    return Table(ids, calls, L)


def completeness(tab: Table, locus_pct=None, sample_pct=None) -> Table:
    """main.rs:313-348: loci first (present fraction * 100 >= thr), then samples."""
    ids, calls = list(tab.ids), tab.calls
    n, L = calls.shape
    if locus_pct is not None:
        with np.errstate(invalid="ignore", divide="ignore"):
            frac = (calls != 0).sum(0).astype(np.float64) / float(n) * 100.0
        keep = np.nonzero(frac >= locus_pct)[0]
        if len(keep) != L:
            calls = calls[:, keep]
    n, L = calls.shape
    if sample_pct is not None:
        with np.errstate(invalid="ignore", divide="ignore"):
            frac = (calls != 0).sum(1).astype(np.float64) / float(L) * 100.0
        keep = np.nonzero(frac >= sample_pct)[0]
        if len(keep) != n:
            calls = calls[keep]
            ids = [ids[i] for i in keep]
    if calls.shape[1] > U16_MAX:
        raise OracleError("more than 65535 loci (u16 distances)")
    return Table(ids, calls, calls.shape[1])


# --------------------------------------------------------------------------------------
# encoding (main.rs:134-165, 167-198, 366-444)
# --------------------------------------------------------------------------------------

def dense_ranks(calls: np.ndarray):
    """main.rs:135-165: per locus, sorted unique non-zero ids -> rank = index+1,
    0 stays 0; counts per rank (index 0 = missing). Fatal above 65535 ids."""
    n, L = calls.shape
    x = np.zeros((n, L), dtype=np.uint16)
    cnt = []
    for k in range(L):
        col = calls[:, k]
        nz = col != 0
        uniq = np.unique(col[nz])
        if len(uniq) > U16_MAX:
            raise OracleError(f"locus {k} has {len(uniq)} distinct alleles (limit 65535)")
        r = np.zeros(n, dtype=np.int64)
        r[nz] = np.searchsorted(uniq, col[nz]) + 1
        x[:, k] = r.astype(np.uint16)
        cnt.append(np.bincount(r, minlength=len(uniq) + 1).astype(np.uint32))
    return x, cnt


def up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


# The reference's analytic model constants, measured on an L4 (main.rs:170-171).
REF_GEMM_RATE = 5.9e14  # pair-bits / s
REF_RARE_RATE = 3.5e9  # rare pairs / s


def choose_tau(cnt, n: int, stripe: int, free: int, gemm_rate=REF_GEMM_RATE, rare_rate=REF_RARE_RATE):
    """main.rs:169-198. Returns (tau, table) where table lists every candidate."""
    c = np.concatenate([v[1:][v[1:] > 0] for v in cnt]) if cnt else np.zeros(0, np.uint32)
    c = c.astype(np.float64)
    n_pad = up(n, 256)
    bufs = float(stripe * n_pad * 12 + (64 << 20))
    best = (0, float("inf"))
    table = []
    tau = 2
    while tau <= 4096:
        d = int((c >= tau).sum())
        rc = c[c < tau]
        r = float((rc * (rc - 1.0) / 2.0).sum())
        k1 = up(max(d, 1), 1024)
        mem = float(n_pad * k1 // 8) + 4.0 * (r + n + 1.0) + bufs
        t = float(n) * float(n) / 2.0 * k1 / gemm_rate + r / rare_rate
        fits = mem <= float(free) and r < 4.0e9
        table.append((tau, d, r, t, mem, fits))
        if fits and t < best[1]:
            best = (tau, t)
        tau *= 2
    if best[0] == 0:
        raise OracleError(f"no tau fits in {free / 1e9:.2f} GB of free VRAM")
    return best[0], table


@dataclass
class Encoding:
    tau: int
    col: list  # per locus: int32 array over ranks, -1 = not frequent
    base: np.ndarray  # L+1 prefix sums of frequent columns
    D: int
    n_pad: int
    K1: int
    K2: int
    O: np.ndarray  # n_pad * K1 / 8 bytes, LSB-first
    P: np.ndarray  # n_pad * K2 / 8 bytes, LSB-first
    start: np.ndarray  # n+1 uint32
    js: np.ndarray  # n_rare uint32, partners of row i sorted ascending


def encode(x: np.ndarray, cnt, tau: int) -> Encoding:
    """main.rs:366-444 (and tc_hamming.cu:138-190). The reference fills each
    row's partner list in a nondeterministic order; here it is sorted, which is
    the canonical form tests compare against (as a multiset per row)."""
    n, L = x.shape
    base = np.zeros(L + 1, dtype=np.int64)
    col = []
    for k in range(L):
        c = cnt[k]
        v = np.full(len(c), -1, dtype=np.int32)
        freq = np.nonzero(c[1:] >= tau)[0] + 1
        v[freq] = np.arange(len(freq), dtype=np.int32)
        base[k + 1] = len(freq)
        col.append(v)
    base = np.cumsum(base)
    D = int(base[L])
    n_pad = up(n, 256)
    K1, K2 = up(max(D, 1), 1024), up(L, 1024)
    Obits = np.zeros((n_pad, K1), dtype=np.uint8)
    Pbits = np.zeros((n_pad, K2), dtype=np.uint8)
    for k in range(L):
        a = x[:, k].astype(np.int64)
        called = a != 0
        Pbits[:n, k] = called
        c = col[k][a]
        f = called & (c >= 0)
        rows = np.nonzero(f)[0]
        Obits[rows, base[k] + c[rows]] = 1
    O = np.packbits(Obits, axis=1, bitorder="little").reshape(-1)
    P = np.packbits(Pbits, axis=1, bitorder="little").reshape(-1)
    # rare equal pairs (i < j), CSR by i
    pairs_i, pairs_j = [], []
    for k in range(L):
        a = x[:, k].astype(np.int64)
        rare = (a != 0) & (col[k][a] < 0) & (cnt[k][a] >= 2)
        rows = np.nonzero(rare)[0]
        if len(rows) < 2:
            continue
        order = np.argsort(a[rows], kind="stable")
        rows, vals = rows[order], a[rows][order]
        bounds = np.nonzero(np.diff(vals))[0] + 1
        for g in np.split(rows, bounds):
            if len(g) < 2:
                continue
            ii, jj = np.triu_indices(len(g), 1)
            pairs_i.append(g[ii])
            pairs_j.append(g[jj])
    if pairs_i:
        pi = np.concatenate(pairs_i)
        pj = np.concatenate(pairs_j)
    else:
        pi = pj = np.zeros(0, dtype=np.int64)
    if len(pi) >= (1 << 32):
        raise OracleError("too many rare pairs: raise --tau")
    order = np.lexsort((pj, pi))
    pi, pj = pi[order], pj[order]
    start = np.zeros(n + 1, dtype=np.uint32)
    np.cumsum(np.bincount(pi, minlength=n), out=start[1:]) if n else None
    return Encoding(tau, col, base, D, n_pad, K1, K2, O, P, start, pj.astype(np.uint32))


# --------------------------------------------------------------------------------------
# the brute-force count (check.py:39-44) and the output formats
# --------------------------------------------------------------------------------------

def hamming(x: np.ndarray, threads: int = 0) -> np.ndarray:
    """Full n x n distance matrix (u16) by the brute-force count of
    check.py:39-44, computed in oracle.c."""
    x = np.ascontiguousarray(x, dtype=np.uint16)
    n, L = x.shape
    H = np.zeros((n, n), dtype=np.uint16)
    if n and L:
        lib().orc_hamming_block(_u16p(x), n, L, 0, n, 0, n, _u16p(H), n, threads)
    return H


def hamming_numpy(A: np.ndarray) -> np.ndarray:
    """check.py:39-44 verbatim in meaning (int64 result), for tiny inputs."""
    P = A > 0
    H = np.zeros((len(A), len(A)), dtype=np.int64)
    for i in range(len(A)):
        H[i] = ((A[i] != A) & P[i] & P).sum(1)
    return H


def hamming_block(x: np.ndarray, i0: int, i1: int, j0: int, j1: int, threads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.uint16)
    n, L = x.shape
    out = np.zeros((i1 - i0, j1 - j0), dtype=np.uint16)
    if out.size and L:
        lib().orc_hamming_block(_u16p(x), n, L, i0, i1, j0, j1, _u16p(out), j1 - j0, threads)
    return out


def hamming_block_calls(calls: np.ndarray, i0: int, i1: int, j0: int, j1: int, threads: int = 0) -> np.ndarray:
    """hamming_block on raw u64 allele ids (0 = missing): the same count
    (check.py:39-44 compares ids for equality) without ranking them first."""
    c = np.ascontiguousarray(calls, dtype=np.uint64)
    n, L = c.shape
    out = np.zeros((i1 - i0, j1 - j0), dtype=np.uint16)
    if out.size and L:
        lib().orc_hamming_block_u64(c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n, L, i0, i1, j0, j1,
                                    _u16p(out), j1 - j0, threads)
    return out


def rollhash(H: np.ndarray) -> int:
    """tc_hamming.cu:240-241 over the upper triangle of a full matrix."""
    H = np.ascontiguousarray(H, dtype=np.uint16)
    n = H.shape[0]
    return int(lib().orc_rollhash_stripe(0, _u16p(H), n, n, n))


def rollhash_ranks(x: np.ndarray, threads: int = 0) -> int:
    x = np.ascontiguousarray(x, dtype=np.uint16)
    n, L = x.shape
    return int(lib().orc_rollhash_ranks(_u16p(x), n, L, threads))


def layout(H: np.ndarray, mode: str = "full", cap: int = 0) -> np.ndarray:
    """Values write_matrix prints (main.rs:245-253): layout mask, then cap."""
    n = H.shape[0]
    V = H.astype(np.int64).copy()
    np.fill_diagonal(V, 0)
    i, j = np.indices((n, n))
    if mode == "lower-tri":
        V[j > i] = 0
    elif mode == "upper-tri":
        V[j < i] = 0
    elif mode != "full":
        raise ValueError(mode)
    if cap > 0:
        V = np.minimum(V, cap)
    return V


def write_matrix(ids, H, osep="\t", index_name="cgmlst-hamming-gpu", mode="full", cap=0) -> str:
    """main.rs:225-265 as text."""
    V = layout(H, mode, cap)
    out = [index_name + "".join(osep + s for s in ids) + "\n"]
    for i, sid in enumerate(ids):
        out.append(sid + "".join(osep + str(int(v)) for v in V[i]) + "\n")
    return "".join(out)


def distances_from_text(text: str, **kw) -> tuple:
    """Whole host pipeline up to the matrix: load, filters, ranks, brute force."""
    tab = load_tsv(text, kw.get("sep", "\t"), kw.get("skip_repl", False), kw.get("missing", "-"))
    tab = completeness(tab, kw.get("locus_pct"), kw.get("sample_pct"))
    x, cnt = dense_ranks(tab.calls)
    return tab.ids, x, cnt, hamming(x)


# --------------------------------------------------------------------------------------
# consumers of the matrix: minimum spanning tree, single linkage, nearest neighbours
# --------------------------------------------------------------------------------------

EDGE_BITS = 21


def edge_keys(H: np.ndarray, v: int) -> np.ndarray:
    """Keys of the edges (v, x) for every x: distance, smaller index, larger index."""
    idx = np.arange(H.shape[0], dtype=np.uint64)
    a = np.minimum(idx, np.uint64(v))
    b = np.maximum(idx, np.uint64(v))
    return (H[v].astype(np.uint64) << np.uint64(2 * EDGE_BITS)) | (a << np.uint64(EDGE_BITS)) | b


def mst(H: np.ndarray):
    """Minimum spanning tree of the complete graph on a full symmetric matrix
    by Prim's algorithm under the strict edge order (distance, smaller index,
    larger index): (u, v, w) of its n - 1 edges in that order, u < v."""
    H = np.asarray(H)
    n = H.shape[0]
    if n < 2:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.uint16)
    none = np.uint64(np.iinfo(np.uint64).max)
    in_tree = np.zeros(n, dtype=bool)
    in_tree[0] = True
    best = edge_keys(H, 0)
    keys = []
    for _ in range(n - 1):
        cand = np.where(in_tree, none, best)
        x = int(cand.argmin())
        keys.append(int(cand[x]))
        in_tree[x] = True
        best = np.minimum(best, edge_keys(H, x))
    k = np.sort(np.array(keys, dtype=np.uint64))
    m = np.uint64((1 << EDGE_BITS) - 1)
    return (((k >> np.uint64(EDGE_BITS)) & m).astype(np.uint32), (k & m).astype(np.uint32),
            (k >> np.uint64(2 * EDGE_BITS)).astype(np.uint16))


def clusters(H: np.ndarray, thresholds) -> np.ndarray:
    """Single-linkage clusters: labels[t, i] = the smallest index of the
    component of i in the graph whose edges are the pairs i != j with
    H[i, j] <= thresholds[t]."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components

    H = np.asarray(H)
    n = H.shape[0]
    out = np.zeros((len(thresholds), n), dtype=np.uint32)
    for t, thr in enumerate(thresholds):
        adj = H.astype(np.int64) <= int(thr)
        np.fill_diagonal(adj, False)
        _, lab = connected_components(csr_matrix(adj), directed=False)
        first = np.full(lab.max() + 1 if n else 0, n, dtype=np.int64)
        np.minimum.at(first, lab, np.arange(n))
        out[t] = first[lab]
    return out


def neighbors(H: np.ndarray, k: int):
    """Every row's k nearest other rows by (distance, index): (idx, dist), n x k."""
    H = np.asarray(H)
    n = H.shape[0]
    keys = (H.astype(np.uint64) << np.uint64(32)) | np.arange(n, dtype=np.uint64)[None, :]
    np.fill_diagonal(keys, np.iinfo(np.uint64).max)
    keys = np.sort(keys, axis=1)[:, :k]
    return (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32), (keys >> np.uint64(32)).astype(np.uint16)
