"""The command-line host, driven the way the reference's exactness check drives
its binary (tensorcore/rs/check.py:47-83): same generator, same 3 cases x 8 flag
sets, output parsed the same way and compared cell for cell — here against the
golden digests of the matrices check.py expects, and against the oracle."""
import gzip
import hashlib
import os
import subprocess

import numpy as np
import pytest

import oracle
import refgen


def cli(pkg):
    assert os.path.exists(pkg.CLI_PATH), "CLI not built"
    return pkg.CLI_PATH


def run(pkg, args, stdin=None):
    return subprocess.run([cli(pkg), *args], capture_output=True, text=True, input=stdin, timeout=600)


def parse(stdout, sep="\t"):
    """check.py:51-53."""
    lines = stdout.rstrip("\n").split("\n")
    return np.array([[int(x) for x in ln.split(sep)[1:]] for ln in lines[1:]])


def mat_sha(M):
    return hashlib.sha256(np.ascontiguousarray(M, dtype="<i8").tobytes()).hexdigest()


# ------------------------------------------------------------------ CPU: host-side semantics

def test_usage_errors(pkg):
    r = run(pkg, [])
    assert r.returncode == 2 and "--input <INPUT>" in r.stderr
    r = run(pkg, ["-i", "x", "-m", "diagonal"])
    assert r.returncode == 2 and "possible values: full, lower-tri, upper-tri" in r.stderr
    r = run(pkg, ["-i", "x", "--tau", "-3"])
    assert r.returncode == 2
    r = run(pkg, ["--help"])
    assert r.returncode == 0 and "--stripe" in r.stdout and "--matrix-format" in r.stdout


def test_separator_checked_before_device(pkg):
    r = run(pkg, ["-i", "x", "-d", "ab"])
    assert r.returncode == 1 and r.stderr.strip() == "error: input separator must be a single character"


def test_missing_device_is_fatal(pkg):
    if pkg.device_count() > 0:
        pytest.skip("a GPU is present")
    r = run(pkg, ["-i", "x", "--device", "0"])
    assert r.returncode == 1 and "CUDA device 0 not available" in r.stderr


# ------------------------------------------------------------------ GPU: the check.py matrix

@pytest.fixture(scope="module")
def case_files(tmp_path_factory, golden):
    d = tmp_path_factory.mktemp("checkpy")
    out = []
    for c in golden["cases"]:
        A, cells = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
        p = d / f"c{c['seed']}.tsv"
        p.write_text(refgen.checkpy_tsv(cells, c["L"]))
        out.append((c, str(p), A))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("encoder", ["device", "device-hostformat", "device-hostparse", "host"])
@pytest.mark.parametrize("case_idx", [0, 1, 2])
@pytest.mark.parametrize("flags_idx", range(len(refgen.CHECKPY_FLAGSETS)))
def test_checkpy_matrix(pkg, case_files, encoder, case_idx, flags_idx):
    """device: table parsed on the GPU, device encoder, text formatted on the
    GPU; device-hostformat: the CPU writer; device-hostparse: the table parsed
    on the CPU; host: the reference's path (host parse and encode, tch_run)."""
    c, path, A = case_files[case_idx]
    args, kind = refgen.CHECKPY_FLAGSETS[flags_idx]
    if encoder == "host":
        args = args + ["--host-encode"]
    elif encoder == "device-hostformat":
        args = args + ["--host-format"]
    elif encoder == "device-hostparse":
        args = args + ["--host-parse"]
    r = run(pkg, ["-s", "-i", path, *args])
    assert r.returncode == 0, r.stderr
    got = parse(r.stdout, "," if "-D" in args else "\t")
    assert mat_sha(got) == c["expected"][kind]  # the matrix the reference's check.py expects


@pytest.mark.gpu
def test_full_text_equals_oracle(pkg, tmp_path):
    text = ("FILE\tL0\tL1\tL2\tL3\n"
            "a\t1\t2\tINF-3\t-\n"
            "b\t 1\t5\t3\tLNF\r\n"
            "\n"
            "c\t1\t\t3\t4\textra\n"
            "d\tINF-INF-1\t2\n"
            "e\t7\t2\t3\t4\n")
    p = tmp_path / "t.tsv"
    p.write_text(text)
    ids, x, cnt, H = oracle.distances_from_text(text)
    for args, kw in [([], {}), (["-m", "lower-tri", "-D", ";"], dict(mode="lower-tri", osep=";")),
                     (["-m", "upper-tri", "-X", "1", "-x", "ID"], dict(mode="upper-tri", cap=1, index_name="ID")),
                     (["-D", "::"], dict(osep="::"))]:
        for fmt in ([], ["--host-format"], ["--host-parse"], ["--host-encode"]):
            r = run(pkg, ["-s", "-i", str(p), *args, *fmt])
            assert r.returncode == 0, r.stderr
            assert r.stdout == oracle.write_matrix(ids, H, **kw), fmt


@pytest.mark.gpu
def test_options_and_streams(pkg, tmp_path, case_files):
    c, path, A = case_files[0]
    with open(path) as f:
        text = f.read()
    ids, x, cnt, H = oracle.distances_from_text(text)
    want = oracle.write_matrix(ids, H)
    # stdin, output file, gzip by flag and by extension, threads, stripe
    r = run(pkg, ["-s", "-i", "-", "-t", "3", "--stripe", "40"], stdin=text)
    assert r.returncode == 0 and r.stdout == want
    out = tmp_path / "o.tsv"
    assert run(pkg, ["-s", "-i", path, "-o", str(out)]).returncode == 0
    assert out.read_text() == want
    gz = tmp_path / "o.tsv.gz"
    assert run(pkg, ["-s", "-i", path, "-o", str(gz)]).returncode == 0
    assert gzip.decompress(gz.read_bytes()).decode() == want
    z = tmp_path / "o2"
    assert run(pkg, ["-s", "-i", path, "-o", str(z), "-z"]).returncode == 0
    assert gzip.decompress(z.read_bytes()).decode() == want
    # logging on stderr without -s
    for extra in ([], ["--host-encode"]):
        r = run(pkg, ["-i", path, "--tau", "4", *extra])
        assert r.returncode == 0 and "Loaded 300 samples x 97 loci" in r.stderr and "tau=4" in r.stderr
        assert r.stdout == want


@pytest.mark.gpu
def test_large_file_read_in_parts(pkg, tmp_path):
    """A regular file is read by parallel preads, one part per 4 MB (here 7
    threads over ~27 MB: uneven parts, cells across part boundaries): the same
    output as the same text through a pipe, and the oracle's distances."""
    rng = np.random.default_rng(31)
    n, L = 1800, 1500
    A = (np.arange(L, dtype=np.uint64)[None, :] << np.uint64(20)) + rng.integers(1, 30, size=(n, L)).astype(np.uint64)
    A[rng.random((n, L)) < 0.03] = 0
    lines = ["FILE\t" + "\t".join(f"L{k}" for k in range(L))]
    lines += [f"s{i}\t" + "\t".join("-" if v == 0 else str(v) for v in A[i].tolist()) for i in range(n)]
    text = "\n".join(lines) + "\n"
    p = tmp_path / "big.tsv"
    p.write_text(text)
    assert p.stat().st_size > 6 * (4 << 20)
    r_file = run(pkg, ["-s", "-i", str(p), "-t", "7"])
    assert r_file.returncode == 0, r_file.stderr
    r_pipe = run(pkg, ["-s", "-i", "-", "-t", "7"], stdin=text)
    assert r_pipe.returncode == 0, r_pipe.stderr
    assert r_file.stdout == r_pipe.stdout
    x, _ = oracle.dense_ranks(A)
    np.testing.assert_array_equal(parse(r_file.stdout), oracle.hamming(x).astype(np.int64))


@pytest.mark.gpu
def test_filters_and_cell_options(pkg, tmp_path):
    text = ("F\ta\tb\tc\td\n"
            "A\t1\tX\t1\tINF-2\n"
            "B\t2\tX\t-\t2\n"
            "C\t1\t3\tX\tINF-2\n"
            "D\t-\t-\t-\t5\n")
    p = tmp_path / "f.tsv"
    p.write_text(text)
    for args, kw in [(["-L", "70"], dict(locus_pct=70.0)), (["-S", "60"], dict(sample_pct=60.0)),
                     (["-L", "50", "-S", "50"], dict(locus_pct=50.0, sample_pct=50.0)),
                     (["-n", "X"], dict(missing="X")), (["-r"], dict(skip_repl=True))]:
        ids, x, cnt, H = oracle.distances_from_text(text, **kw)
        for parse_on in ([], ["--host-parse"]):
            r = run(pkg, ["-s", "-i", str(p), *args, *parse_on])
            assert r.returncode == 0, (args, parse_on, r.stderr)
            assert r.stdout == oracle.write_matrix(ids, H), (args, parse_on)


@pytest.mark.gpu
def test_edge_inputs(pkg, tmp_path):
    def go(text, *args):
        p = tmp_path / "e.tsv"
        p.write_bytes(text.encode() if isinstance(text, str) else text)
        return run(pkg, ["-s", "-i", str(p), *args])

    r = go("")
    assert r.returncode == 1 and "empty input" in r.stderr
    for parse_on in ([], ["--host-parse"]):
        r = go("F\tL0\nA\t18446744073709551616\n", *parse_on)
        assert r.returncode == 1 and "sample A: allele '18446744073709551616' too large" in r.stderr
    r = go(b"F\tL0\nA\t\xff\n")
    assert r.returncode == 1 and "valid UTF-8" in r.stderr
    r = go("F\tL0\tL1\nA\t1\t2\n")  # one sample: no GPU work, 1x1 matrix
    assert r.returncode == 0 and r.stdout == "cgmlst-hamming-gpu\tA\nA\t0\n"
    r = go("F\nA\nB\n")  # no loci
    assert r.returncode == 0 and r.stdout == "cgmlst-hamming-gpu\tA\tB\nA\t0\t0\nB\t0\t0\n"
    r = go("F\tL0\n")  # header only
    assert r.returncode == 0 and r.stdout == "cgmlst-hamming-gpu\n"


@pytest.mark.gpu
@pytest.mark.parametrize("layout,osep,cap,block", [("full", "\t", 0, 7), ("lower-tri", ",", 3, 64),
                                                   ("upper-tri", "\t", 0, 1), ("full", " | ", 40, 0)])
def test_gpu_tsv_writer_blocks(pkg, layout, osep, cap, block):
    """tch_solver_write_tsv over several blocks of rows equals the oracle's text."""
    rng = np.random.default_rng(11)
    n, L = 300, 120
    A = rng.integers(0, 30, size=(n, L)).astype(np.uint64)
    A[:, :10] = rng.integers(0, 2000, size=(n, 10))
    x = oracle.dense_ranks(A)[0]
    H = oracle.hamming(x)
    ids = [f"s{i}" * (1 + i % 3) for i in range(n)]
    with pkg.Solver.from_calls(A) as s:
        text = s.write_tsv(ids, osep=osep, index_name="IDX", layout=layout, cap=cap, block_rows=block)
    assert text == oracle.write_matrix(ids, H, osep=osep, index_name="IDX", mode=layout, cap=cap)
