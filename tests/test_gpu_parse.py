"""The allele table parsed on the GPU (tch_tsv_*) against the oracle's restated
load (main.rs:286-311, parse_allele main.rs:95-113) and completeness filters
(main.rs:313-348): calls and sample ids equal cell for cell, on the reference's
own check-case texts (check.py's generator, every cell option), on edge texts
(CRLF and bare '\\r', blank lines, a last line without '\\n', short and long
rows, Unicode white space, 'INF-', missing tokens, values at and past 2^64 - 1,
lines longer than the GPU's 64 KB newline chunks), and as the input of a solver
whose distances equal the brute-force count."""
import numpy as np
import pytest

import oracle
import refgen

pytestmark = pytest.mark.gpu


def same(pkg, text, sep="\t", skip_repl=False, missing="-"):
    want = oracle.load_tsv(text, sep=sep, skip_repl=skip_repl, missing=missing)
    with pkg.Tsv(text.encode(), sep=sep, skip_repl=skip_repl, missing=missing) as t:
        assert t.shape() == want.calls.shape
        np.testing.assert_array_equal(t.calls(), want.calls)
        assert t.ids() == list(want.ids)
    return want


@pytest.mark.parametrize("flags", [(False, "-"), (True, "-"), (False, "LNF"), (True, "")])
def test_checkpy_cases(pkg, golden, flags):
    skip, missing = flags
    for c in golden["cases"]:
        _, cells = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
        same(pkg, refgen.checkpy_tsv(cells, c["L"]), skip_repl=skip, missing=missing)


EDGE = [
    "FILE\ta\tb\tc\ns1\t1\t2\t3\ns2\t4\t5\t6\n",
    "FILE\ta\tb\tc\r\ns1\t1\t2\t3\r\ns2\t4\t5\t6\r\n",
    "FILE\ta\tb\n\n\ns1\t1\t2\n\n",
    "FILE\ta\tb\ns1\t1\t2",                  # last line without '\n'
    "FILE\ta\tb\ns1\t1\t2\r",                # ... keeps its '\r' (trimmed from the cell)
    "FILE\ta\tb\tc\ns1\t1\ns2\t1\t2\t3\t4\t5\n",   # short and long rows
    "FILE\ta\tb\ns1\n",                      # no cells at all
    "FILE\ta\tb\n",                          # header only
    "FILE\ta\tb",                            # header only, no newline
    "FILE\ta\tb\tc\ns1\t\u00a0 12\u2003\t\u3000\t\u2028 7\u0085\n",   # Unicode white space around values
    "FILE\ta\tb\tc\ns1\tINF-7\t INF-8 \tINF- 9\n",
    "FILE\ta\tb\tc\td\ns1\t-\t\tN/A\t+5\n",
    "FILE\ta\tb\tc\ns1\t007\t12a\t18446744073709551615\n",
    "FILE\ta\tb\nséß\t1\t2\ns 2 \t3\t4\n",   # ids as written
    "FILE\ta\tb\ns1\tÉ12\t12É\n",
]


@pytest.mark.parametrize("text", EDGE)
@pytest.mark.parametrize("flags", [(False, "-"), (True, "N/A")])
def test_edge_texts(pkg, text, flags):
    same(pkg, text, skip_repl=flags[0], missing=flags[1])


def test_other_separator(pkg):
    same(pkg, "FILE,a,b\ns1,1,2\ns2,3,-\n", sep=",")


def test_overflow_is_an_error(pkg):
    text = "FILE\ta\tb\ns1\t1\t2\nbad one\t 18446744073709551616 \t3\n"
    with pytest.raises(pkg.TchError, match="sample bad one: allele '18446744073709551616' too large"):
        pkg.Tsv(text.encode())
    with pytest.raises(oracle.OracleError):
        oracle.load_tsv(text)


def test_long_lines_and_many_chunks(pkg):
    """Lines longer than one 64 KB newline chunk and a text of many chunks."""
    rng = np.random.default_rng(4)
    L = 12000
    A = rng.integers(0, 1000000, size=(40, L))
    head = "FILE\t" + "\t".join(f"l{k}" for k in range(L)) + "\n"
    rows = []
    for i in range(40):
        cells = [("-" if v == 0 else str(v)) for v in A[i]]
        rows.append(f"s{i}\t" + "\t".join(cells) + ("\r\n" if i % 3 == 0 else "\n"))
        if i % 7 == 0:
            rows.append("\n")
    same(pkg, head + "".join(rows))


@pytest.mark.parametrize("thr", [(None, 90.0), (95.0, None), (97.0, 99.0), (100.0, 0.0)])
def test_completeness_filters(pkg, thr):
    rng = np.random.default_rng(9)
    n, L = 300, 80
    A = rng.integers(1, 9, size=(n, L))
    A[rng.random((n, L)) < rng.uniform(0, 0.12, size=L)] = 0
    text = "FILE\t" + "\t".join(f"l{k}" for k in range(L)) + "\n" + "".join(
        f"s{i}\t" + "\t".join("-" if v == 0 else str(v) for v in A[i]) + "\n" for i in range(n))
    want = oracle.completeness(oracle.load_tsv(text), locus_pct=thr[0], sample_pct=thr[1])
    with pkg.Tsv(text.encode()) as t:
        t.filter(locus_pct=thr[0], sample_pct=thr[1])
        assert t.shape() == want.calls.shape
        np.testing.assert_array_equal(t.calls(), want.calls)
        assert t.ids() == list(want.ids)


def test_solver_from_parsed_table(pkg, golden):
    c = golden["cases"][0]
    _, cells = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    text = refgen.checkpy_tsv(cells, c["L"])
    tab = oracle.load_tsv(text)
    ref = oracle.hamming(oracle.dense_ranks(tab.calls)[0])
    with pkg.Tsv(text.encode()) as t, t.solver() as s:
        H, _ = s.run(64)
    n = len(tab.ids)
    iu = np.triu_indices(n, 1)
    np.testing.assert_array_equal(H[iu], ref[iu])
