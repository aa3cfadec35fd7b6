"""Ranks files (tensorcore/to_ranks.py format: int32 n, int32 L, n x L u16,
0 = missing) and the prototype-compatible front end bin/tch-ranks
(tensorcore/tc_hamming.cu:12-13, 105-117, 240-253): rolling checksum of the
upper triangle against the golden fixtures and the oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
import refgen


def test_ranks_file_roundtrip(pkg, tmp_path):
    rng = np.random.default_rng(0)
    x = rng.integers(0, 500, size=(37, 11)).astype(np.uint16)
    p = str(tmp_path / "r.bin")
    pkg.write_ranks(p, x)
    raw = open(p, "rb").read()
    assert raw[:8] == np.array([37, 11], "<i4").tobytes() and len(raw) == 8 + 37 * 11 * 2
    np.testing.assert_array_equal(pkg.read_ranks(p), x)
    open(p, "wb").write(raw[:-2])
    with pytest.raises(pkg.TchError, match="truncated"):
        pkg.read_ranks(p)


def test_ranks_tool_usage(pkg, tmp_path):
    r = subprocess.run([pkg.RANKS_TOOL_PATH], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
    r = subprocess.run([pkg.RANKS_TOOL_PATH, str(tmp_path / "missing.bin")], capture_output=True, text=True)
    assert r.returncode == 1


def factorized(A):
    """to_ranks.py's ranks: per locus, order of first appearance (not sorted)."""
    x = np.zeros(A.shape, np.uint16)
    for k in range(A.shape[1]):
        seen = {}
        for i, v in enumerate(A[:, k]):
            if v == 0:
                continue
            x[i, k] = seen.setdefault(int(v), len(seen) + 1)
    return x


@pytest.mark.gpu
@pytest.mark.parametrize("case_idx", [0, 1, 2])
def test_ranks_tool_checksum_matches_golden(pkg, golden, tmp_path, case_idx):
    c = golden["cases"][case_idx]
    A, _ = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    p = str(tmp_path / "case.bin")
    pkg.write_ranks(p, factorized(A.astype(np.uint64)))
    for args in ([], ["0", "64"], ["2", "8"]):
        r = subprocess.run([pkg.RANKS_TOOL_PATH, p, *args], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        h = int(re.search(r"checksum=([0-9a-f]+)", r.stdout).group(1), 16)
        assert h == int(c["rollhash"], 16)
    r = subprocess.run([pkg.RANKS_TOOL_PATH, p, "0", "512", "noverify"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "checksum=0" in r.stdout


@pytest.mark.gpu
def test_solver_from_ranks_exact(pkg):
    rng = np.random.default_rng(5)
    x = rng.integers(0, 40, size=(700, 90)).astype(np.uint16)
    x[:, :5] = rng.integers(0, 65535, size=(700, 5))
    ref = oracle.hamming(x)
    with pkg.Solver.from_ranks(x, tau=0) as s:
        H, _ = s.run(256)
    iu = np.triu_indices(700, 1)
    np.testing.assert_array_equal(H[iu], ref[iu])
