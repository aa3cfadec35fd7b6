"""Host-side parts of libtch on the CPU: the C ABI loads and exports what
include/tch.h declares, and the C++ host encoder equals the oracle's
restatement of the reference host (main.rs:134-198, 366-444)."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
import refgen
from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "tch.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tch_\w+)\s*\(", text)) - {"tch_cb"})


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.lib()
    syms = declared_symbols()
    assert "tch_run" in syms and "tch_device_count" in syms and "tch_free_vram" in syms
    for s in syms:
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", pkg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (tch_\w+)", out))
    assert set(syms) <= exported


def test_bindings_check_shapes_before_the_library(pkg):
    """Arrays whose shapes disagree with one another are rejected in Python,
    before a pointer reaches C (which would read or write past them).  The
    serving calls are made on stand-ins for a database and a server, which
    are never reached."""
    from types import SimpleNamespace

    w = np.zeros(pkg.MLP_PARAMS, np.float32)
    X = np.zeros((5, pkg.TAU_FEATURES), np.float32)
    with pytest.raises(pkg.TchError, match="parameters"):
        pkg.mlp_predict(w[:-1], X)
    with pytest.raises(pkg.TchError, match="samples must be"):
        pkg.mlp_predict(w, X[:, :-1])
    with pytest.raises(pkg.TchError, match="samples must be"):
        pkg.mlp_predict(w, X.ravel())
    with pytest.raises(pkg.TchError, match="one target per sample"):
        pkg.mlp_loss_grad(w, X, np.zeros(4, np.float32))
    with pytest.raises(pkg.TchError, match="one target per sample"):
        pkg.mlp_train(w, X, np.zeros(6, np.float32), steps=1, lr=1e-3)
    db = SimpleNamespace(n=10, L=7, _h=None)
    q = np.ones((3, 7), np.uint64)
    with pytest.raises(pkg.TchError, match="loci"):
        pkg.Database.query(db, np.ones((3, 6), np.uint64))
    with pytest.raises(pkg.TchError, match="out must be"):
        pkg.Database.query(db, q, out=np.zeros((3, 9), np.uint16))
    with pytest.raises(pkg.TchError, match="out_qq must be"):
        pkg.Database.query(db, q, out_qq=np.zeros((3, 3), np.uint32))
    sv = SimpleNamespace(db=db, _h=None, _live={})
    with pytest.raises(pkg.TchError, match="queries must be"):
        pkg.Server.submit(sv, np.ones((3, 6), np.uint64))
    with pytest.raises(pkg.TchError, match="out must be"):
        pkg.Server.submit(sv, q, out=np.zeros((10, 3), np.uint16))
    with pytest.raises(pkg.TchError, match="out_qq must be"):
        pkg.Server.submit(sv, q, out_qq=np.zeros((3, 6), np.uint16)[:, ::2])  # not contiguous


def test_encoder_rejects_ranks_above_their_counts(pkg):
    """The host encoder and the tau model count ranks per (locus, rank): a rank
    above its locus's distinct count, a count above 65 535 or counts of the
    wrong length are errors (a C caller could otherwise index past the
    counters)."""
    rng = np.random.default_rng(5)
    A = rng.integers(0, 9, size=(50, 12)).astype(np.uint64)
    x, nd = pkg.dense_ranks(A)
    bad = nd.copy()
    bad[7] = max(int(x[:, 7].max()) - 1, 0)
    with pytest.raises(pkg.TchError, match="locus 7: rank"):
        pkg.encode_host(x, bad, tau=4)
    with pytest.raises(pkg.TchError, match="locus 7: rank"):
        pkg.choose_tau(x, bad, free_bytes=1 << 40)
    big = nd.copy()
    big[3] = 70000
    with pytest.raises(pkg.TchError, match="locus 3: 70000 distinct"):
        pkg.encode_host(x, big, tau=4)
    with pytest.raises(pkg.TchError, match="one distinct count per locus"):
        pkg.encode_host(x, nd[:-1], tau=4)
    enc = pkg.encode_host(x, nd, tau=4)  # the consistent pair still encodes
    assert enc.n == 50 and enc.L == 12


def test_kernel_names(pkg):
    assert pkg.kernel_name(1) == "popc" and pkg.kernel_name(99) == "?"
    assert pkg.kernel_available("popc")


@pytest.mark.parametrize("seed", [0, 1])
def test_dense_ranks_matches_oracle(pkg, seed):
    rng = np.random.default_rng(seed)
    calls = rng.integers(0, 2**64 - 1, size=(50, 9), dtype=np.uint64, endpoint=True)
    calls[rng.random(calls.shape) < 0.3] = 0
    calls[:, 3] = calls[rng.integers(0, 50, 50), 3]  # repeats
    x, nd = pkg.dense_ranks(calls, threads=3)
    xo, cnt = oracle.dense_ranks(calls)
    np.testing.assert_array_equal(x, xo)
    np.testing.assert_array_equal(nd, [len(c) - 1 for c in cnt])


def test_dense_ranks_limit(pkg):
    calls = np.arange(1, 70001, dtype=np.uint64).reshape(-1, 1)
    with pytest.raises(pkg.TchError, match="65535"):
        pkg.dense_ranks(calls)


@pytest.mark.parametrize("case_idx", [0, 1])
@pytest.mark.parametrize("tau", [1, 2, 8, 100000])
def test_encode_host_matches_oracle(pkg, golden, case_idx, tau):
    c = golden["cases"][case_idx]
    A, _ = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    x, nd = pkg.dense_ranks(A.astype(np.uint64))
    xo, cnt = oracle.dense_ranks(A.astype(np.uint64))
    enc = pkg.encode_host(x, nd, tau, threads=4)
    ref = oracle.encode(xo, cnt, tau)
    assert (enc.D, enc.n_pad, enc.K1, enc.K2, enc.n_rare) == (ref.D, ref.n_pad, ref.K1, ref.K2, len(ref.js))
    np.testing.assert_array_equal(enc.O, ref.O)
    np.testing.assert_array_equal(enc.P, ref.P)
    np.testing.assert_array_equal(enc.start, ref.start)
    np.testing.assert_array_equal(enc.js, ref.js)


@pytest.mark.parametrize("free", [1 << 24, 1 << 30, 1 << 40])
def test_choose_tau_matches_oracle(pkg, golden, free):
    c = golden["cases"][1]
    A, _ = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    x, nd = pkg.dense_ranks(A.astype(np.uint64))
    xo, cnt = oracle.dense_ranks(A.astype(np.uint64))
    try:
        want = oracle.choose_tau(cnt, c["n"], 512, free)[0]
    except oracle.OracleError:
        with pytest.raises(pkg.TchError, match="no tau fits"):
            pkg.choose_tau(x, nd, 512, free)
        return
    assert pkg.choose_tau(x, nd, 512, free) == want
