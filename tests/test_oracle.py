"""The oracle, pinned against the reference's own outputs (CPU only).

The golden digests in tests/golden/golden.json were written by
tests/golden/make_golden.py from the reference's check.py (``make``/``ref``)
and python/gen_profiles.py.
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
import refgen

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(b):
    return hashlib.sha256(b).hexdigest()


def mat_sha(M):
    return sha(np.ascontiguousarray(M, dtype="<i8").tobytes())


@pytest.mark.parametrize("case_idx", [0, 1, 2])
def test_checkpy_generator_and_oracle_match_reference(golden, case_idx):
    c = golden["cases"][case_idx]
    A, cells = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    text = refgen.checkpy_tsv(cells, c["L"])
    assert sha(text.encode()) == c["tsv_sha256"]
    assert mat_sha(A) == c["A_sha256"]
    ids, x, cnt, H = oracle.distances_from_text(text)
    assert ids == [f"S{i}" for i in range(c["n"])]
    assert mat_sha(H) == c["H_sha256"]
    assert "%016x" % oracle.rollhash(H) == c["rollhash"]
    for kind in ("full", "lower", "upper", "cap7"):
        assert mat_sha(refgen.checkpy_expected(H.astype(np.int64), kind)) == c["expected"][kind]


def test_small_case_full_matrix():
    z = np.load(os.path.join(GOLDEN_DIR, "checkpy_300x97.npz"))
    A, H = z["A"], z["H"]
    x = refgen.ranks_of(A)
    np.testing.assert_array_equal(oracle.hamming(x), H)
    np.testing.assert_array_equal(oracle.hamming_numpy(x).astype(np.uint16), H)


def test_gen_profiles_restatement(golden):
    for k, v in golden["gen_profiles"].items():
        n, L = map(int, k.split("x"))
        assert sha(refgen.gen_profiles_tsv(refgen.gen_profiles(n, L)).encode()) == v


@pytest.mark.parametrize(
    "cell,expect",
    [
        ("5", 5), ("  7 ", 7), ("\t12\r", 12), ("INF-5", 5), (" INF-5", 5), ("INF- 5", 0),
        ("INF-INF-5", 0), ("-", 0), ("", 0), ("   ", 0), ("LNF", 0), ("PLOT3", 0), ("0", 0),
        ("007", 7), ("+5", 0), ("5a", 0), ("INF--", 0), (" 9　", 9), ("\x1c9", 0),
        ("18446744073709551615", 18446744073709551615),
    ],
)
def test_parse_allele(cell, expect):
    assert oracle.parse_allele(cell) == expect


def test_parse_allele_options():
    assert oracle.parse_allele("INF-5", skip_repl=True) == 0
    assert oracle.parse_allele("LNF", missing="LNF") == 0
    assert oracle.parse_allele("INF-LNF", missing="LNF") == 0
    with pytest.raises(oracle.OracleError):
        oracle.parse_allele("18446744073709551616")


def test_rust_lines():
    assert oracle.rust_lines("") == []
    assert oracle.rust_lines("a") == ["a"]
    assert oracle.rust_lines("a\n") == ["a"]
    assert oracle.rust_lines("a\r\nb\r\n") == ["a", "b"]
    assert oracle.rust_lines("a\n\nb") == ["a", "", "b"]
    assert oracle.rust_lines("a\r") == ["a\r"]
    assert oracle.rust_lines("\n") == [""]


def test_load_pads_and_truncates_rows():
    t = oracle.load_tsv("FILE\tL0\tL1\tL2\nA\t1\t2\nB\t1\t2\t3\t4\n\nC\n")
    assert t.ids == ["A", "B", "C"] and t.L == 3
    np.testing.assert_array_equal(t.calls, np.array([[1, 2, 0], [1, 2, 3], [0, 0, 0]], np.uint64))


def test_completeness_filters():
    t = oracle.load_tsv("F\ta\tb\tc\nA\t1\t-\t1\nB\t2\t-\t5\nC\t1\t3\t-\n")
    f = oracle.completeness(t, locus_pct=50.0)
    assert f.L == 2  # locus b has 1/3 calls
    g = oracle.completeness(f, sample_pct=100.0)
    assert g.ids == ["A", "B"]


def random_profiles(rng, n, L, max_alleles=40, miss=0.1):
    A = rng.integers(1, rng.integers(2, max_alleles + 1, size=L) + 1, size=(n, L))
    A[rng.random((n, L)) < miss] = 0
    return A


@pytest.mark.parametrize("tau", [1, 2, 3, 5, 8, 1 << 30])
def test_encoding_identity(tau):
    """P Pt - (O Ot + R) from the restated encoder equals the brute force for
    every tau (main.rs:366-444 against check.py:39-44)."""
    rng = np.random.default_rng(11 + tau % 97)
    A = random_profiles(rng, 97, 45)
    x, cnt = oracle.dense_ranks(A.astype(np.uint64))
    e = oracle.encode(x, cnt, tau)
    n = x.shape[0]
    P = np.unpackbits(e.P.reshape(e.n_pad, -1), axis=1, bitorder="little")[:n].astype(np.int64)
    O = np.unpackbits(e.O.reshape(e.n_pad, -1), axis=1, bitorder="little")[:n].astype(np.int64)
    R = np.zeros((n, n), np.int64)
    for i in range(n):
        js = e.js[e.start[i]:e.start[i + 1]]
        assert np.all(np.diff(js.astype(np.int64)) >= 0) and np.all(js > i)
        np.add.at(R[i], js.astype(np.int64), 1)
    R = R + R.T
    H = P @ P.T - O @ O.T - R
    Hb = oracle.hamming(x).astype(np.int64)
    iu = np.triu_indices(n, 1)
    np.testing.assert_array_equal(H[iu], Hb[iu])
    assert e.K1 % 1024 == 0 and e.K2 % 1024 == 0 and e.n_pad % 256 == 0


def test_choose_tau_reference_constants():
    rng = np.random.default_rng(5)
    A = random_profiles(rng, 500, 30, max_alleles=200)
    x, cnt = oracle.dense_ranks(A.astype(np.uint64))
    tau, table = oracle.choose_tau(cnt, 500, 512, 1 << 34)
    assert tau in [t[0] for t in table] and len(table) == 12
    best = min((t for t in table if t[5]), key=lambda t: t[3])
    assert best[0] == tau
    with pytest.raises(oracle.OracleError):
        oracle.choose_tau(cnt, 500, 512, 1 << 10)


def test_rollhash_and_blocks():
    rng = np.random.default_rng(3)
    x = refgen.ranks_of(random_profiles(rng, 130, 17))
    H = oracle.hamming(x)
    assert oracle.rollhash(H) == oracle.rollhash_ranks(x)
    np.testing.assert_array_equal(oracle.hamming_block(x, 7, 70, 33, 129), H[7:70, 33:129])
    h = 0
    for i in range(130):
        for j in range(i + 1, 130):
            h = (h * 1000003 + int(H[i, j])) % (1 << 64)
    assert h == oracle.rollhash(H)


def test_write_matrix_text():
    H = np.array([[0, 3], [3, 0]], np.uint16)
    assert oracle.write_matrix(["a", "b"], H) == "cgmlst-hamming-gpu\ta\tb\na\t0\t3\nb\t3\t0\n"
    assert oracle.write_matrix(["a", "b"], H, mode="lower-tri", osep=",") == "cgmlst-hamming-gpu,a,b\na,0,0\nb,3,0\n"
    assert oracle.write_matrix(["a", "b"], H, mode="upper-tri", cap=2, index_name="x") == "x\ta\tb\na\t0\t2\nb\t0\t0\n"


def test_block_on_raw_ids_equals_block_on_ranks():
    """The oracle's count on raw 64-bit ids (used where ranking a large matrix
    first would cost more than the check) equals its count on the ranks."""
    rng = np.random.default_rng(12)
    A = rng.integers(0, 7, size=(260, 33)).astype(np.uint64) * np.uint64(2**40 + 3)
    A[:, 5] = rng.integers(2**62, 2**63, size=260, dtype=np.uint64)
    x = oracle.dense_ranks(A)[0]
    for i0, i1, j0, j1 in [(0, 260, 0, 260), (7, 19, 100, 259), (259, 260, 0, 1)]:
        np.testing.assert_array_equal(oracle.hamming_block_calls(A, i0, i1, j0, j1),
                                      oracle.hamming_block(x, i0, i1, j0, j1))
