"""Host code under AddressSanitizer and UBSan, on the CPU: the library's host
encoder (csrc/encode_host.cpp), the CLI's input path (parallel preads, UTF-8
check, line split, cell parse, the fused row parser), its CPU TSV writer and its
gzip writer, compiled here with -fsanitize and run
on generated inputs.  A sanitizer report makes the program exit non-zero."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "cgmlst-hamming-gpu_gb300")
FLAGS = ["-O1", "-g", "-std=c++17", "-pthread", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
         "-fno-omit-frame-pointer"]


def build(tmp_path, name, srcs, extra=()):
    exe = str(tmp_path / name)
    r = subprocess.run(["g++", *FLAGS, "-I", os.path.join(ROOT, "include"), *srcs, "-o", exe, *extra],
                       capture_output=True, text=True)
    if r.returncode:
        if "asan" in r.stderr.lower() or "ubsan" in r.stderr.lower():
            pytest.skip("no sanitizer runtime for g++ here")
        if "zlib.h" in r.stderr or "-lz" in r.stderr:
            pytest.skip("no zlib for g++ here")
        raise AssertionError(r.stderr[-3000:])
    return exe


def test_host_encoder_under_sanitizers(tmp_path):
    exe = build(tmp_path, "encode_check", [os.path.join(ROOT, "tests", "sanitize", "encode_host_check.cpp"),
                                           os.path.join(PKG_DIR, "csrc", "encode_host.cpp")])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "encode_host ok" in r.stdout, r.stdout + r.stderr[-3000:]


# Unicode White_Space, the set Rust's str::trim removes
WHITE_SPACE = ("\t\n\x0b\x0c\r \x85\xa0\u1680" + "".join(chr(c) for c in range(0x2000, 0x200B))
               + "\u2028\u2029\u202f\u205f\u3000")


def expected(text: str):
    """bytes, lines (str::lines), fields before each line's end, and the sum
    of the parsed ids, for inputs of digits, '-', 'INF-' ids and white space."""
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    lines = [ln[:-1] if ln.endswith("\r") else ln for ln in lines]
    cells, total = 0, 0
    for ln in lines:
        fields = ln.split("\t")
        if ln.endswith("\t"):
            fields.pop()
        if ln == "":
            fields = []
        cells += len(fields)
        for f in fields:
            f = f.strip(WHITE_SPACE)
            if f.startswith("INF-"):
                f = f[4:]
            if f and f != "-" and f.isdigit():
                total += int(f)
    return len(text.encode()), len(lines), cells, total


def test_cli_input_path_under_sanitizers(tmp_path, pkg):
    lib_dir = os.path.join(PKG_DIR, "lib")
    exe = build(tmp_path, "cli_read_check", [os.path.join(ROOT, "tests", "sanitize", "cli_read_check.cpp")],
                extra=["-I", os.path.join(PKG_DIR, "host"), "-L", lib_dir, "-ltch", "-ldl",
                       f"-Wl,-rpath,{lib_dir}"])
    rng = np.random.default_rng(3)
    n, L = 2500, 700
    ids = rng.integers(1, 10**9, size=(n, L))
    rows = []
    for i in range(n):
        cells = [str(v) for v in ids[i].tolist()]
        for k in rng.integers(0, L, size=20).tolist():
            cells[k] = "-"
        cells[i % L] = f"INF-{ids[i, 0]}"
        cells[(i * 7) % L] = f" {ids[i, 1]} "
        if i % 97 == 0:
            cells = cells[: L // 2]  # a short row
        rows.append(f"s{i}\t" + "\t".join(cells) + ("\r\n" if i % 5 == 0 else "\n"))
    big = "FILE\t" + "\t".join(f"L{k}" for k in range(L)) + "\n" + "".join(rows)
    files = {"big.tsv": big, "small.tsv": "FILE\tA\nx\t1\n\n y \tINF-3", "empty.tsv": "",
             "utf8.tsv": "FILE\tA\u00e9\n\u3000s\u00e9\t\u00a012\u2003\n\U0001F600\t7\n" * 5000}
    for name, text in files.items():
        (tmp_path / name).write_text(text, encoding="utf-8")
    assert len(big) > 12 * (1 << 20)  # at least three read parts
    r = subprocess.run([exe, *[str(tmp_path / f) for f in files]], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr[-3000:]
    out = r.stdout.strip().split("\n")
    assert len(out) == 4 * len(files)
    for k, (name, text) in enumerate(files.items()):
        got = out[4 * k: 4 * k + 4]
        assert len(set(got)) == 1, (name, got)  # every thread count reads the same
        assert tuple(int(v) for v in got[0].split()) == expected(text), name
    # invalid UTF-8 anywhere (also past the first 8-byte ASCII runs) is an error,
    # as Rust's str::from_utf8 (and Python's decoder) has it
    ascii_run = b"FILE\tA\n" + b"s1\t123\n" * 3
    bad = {"lone_continuation": b"\x80", "truncated": b"\xe3\x80", "overlong": b"\xc0\xaf",
           "surrogate": b"\xed\xa0\x80", "too_large": b"\xf4\x90\x80\x80", "bad_lead": b"\xff"}
    good = {"two_byte": "\u00e9".encode(), "three_byte": "\u3000".encode(), "four_byte": "\U0001F600".encode()}
    for name, seq in {**bad, **good}.items():
        for where in (0, 5, len(ascii_run)):
            data = ascii_run[:where] + seq + ascii_run[where:]
            (tmp_path / "u.tsv").write_bytes(data)
            r = subprocess.run([exe, str(tmp_path / "u.tsv")], capture_output=True, text=True, timeout=60)
            assert r.returncode == 0, r.stderr[-3000:]
            try:
                data.decode("utf-8")
                valid = True
            except UnicodeDecodeError:
                valid = False
            assert valid == (name in good)
            lines = r.stdout.strip().split("\n")
            assert all(("error" not in ln) == valid for ln in lines), (name, where, lines)


@pytest.mark.parametrize("zlib", [True, False])
def test_gzip_writer_under_sanitizers(tmp_path, zlib):
    """Stored blocks and zlib deflate both decompress to the bytes written."""
    import gzip

    extra = ["-I", os.path.join(PKG_DIR, "host")] + (["-DTCH_HAVE_ZLIB", "-lz"] if zlib else [])
    exe = build(tmp_path, f"gzip_check_{int(zlib)}", [os.path.join(ROOT, "tests", "sanitize", "gzip_check.cpp")],
                extra=extra)
    rng = np.random.default_rng(4)
    data = b"".join([rng.integers(0, 10, 3_000_000, dtype=np.uint8).astype(np.uint8).tobytes() + b"\t",
                     b"", bytes(range(256)) * 9000, b"x" * 2_500_000])
    for payload in (data, b"", b"a"):
        r = subprocess.run([exe], input=payload, capture_output=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        assert gzip.decompress(r.stdout) == payload


def test_cpu_writer_under_sanitizers(tmp_path, pkg):
    """The --host-format writer's text equals the oracle's (main.rs:224-265)
    for every layout, a cap and a multi-byte separator, over more than one
    1 024-row chunk."""
    import oracle

    lib_dir = os.path.join(PKG_DIR, "lib")
    exe = build(tmp_path, "writer_check", [os.path.join(ROOT, "tests", "sanitize", "writer_check.cpp")],
                extra=["-I", os.path.join(PKG_DIR, "host"), "-L", lib_dir, "-ltch", "-ldl",
                       f"-Wl,-rpath,{lib_dir}"])
    rng = np.random.default_rng(6)
    n = 1100
    U = np.triu(rng.integers(0, 70000, size=(n, n)) % 65536, 1).astype(np.int64)
    H = U + U.T
    text_in = f"{n}\n" + "\n".join(" ".join(map(str, row)) for row in H.tolist()) + "\n"
    ids = [f"s{i}" for i in range(n)]
    for osep, index_name, mode, cap, threads in [("\t", "cgmlst-hamming-gpu", "full", 0, 7),
                                                  (";", "ID", "lower-tri", 0, 3),
                                                  ("::", "x", "upper-tri", 1000, 16)]:
        r = subprocess.run([exe, osep, index_name, mode, str(cap), str(threads)], input=text_in,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        assert r.stdout == oracle.write_matrix(ids, H, osep=osep, index_name=index_name, mode=mode, cap=cap), mode


def test_row_parser_matches_the_per_cell_parse(tmp_path, pkg):
    """The CLI's fused row parser (a fast path for plain digit cells) gives the
    values, verdict and first bad cell of the per-cell parse on 36 000 random
    rows of adversarial cells, for two separators, three missing tokens (one
    all digits) and both INF- settings."""
    lib_dir = os.path.join(PKG_DIR, "lib")
    exe = build(tmp_path, "parse_row_check", [os.path.join(ROOT, "tests", "sanitize", "parse_row_check.cpp")],
                extra=["-I", os.path.join(PKG_DIR, "host"), "-L", lib_dir, "-ltch", "-ldl",
                       f"-Wl,-rpath,{lib_dir}"])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "parse_row ok" in r.stdout, r.stdout + r.stderr[-3000:]

