"""The device encoder (allele calls -> ranks, operands, rare CSR on the GPU)
against the oracle: every cell of the upper triangle, and the encoder's sizes
(one-hot columns, rare pairs) against the restated reference host encoder."""
import numpy as np
import pytest

import oracle
import refgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["dense", "lists"])
def tch(pkg, request):
    """Every test runs for both holdings of the rare term: per-stripe dense
    counts from the rare groups, and the reference's pair lists."""
    assert pkg.device_count() > 0, "no CUDA device visible"
    pkg.set_rare_term(request.param == "dense")
    yield pkg
    pkg.set_rare_term(True)


def upper_equal(H, ref):
    iu = np.triu_indices(ref.shape[0], 1)
    bad = np.nonzero(H[iu] != ref[iu])[0]
    assert len(bad) == 0, f"{len(bad)} cells differ"


@pytest.mark.parametrize("case_idx", [0, 1, 2])
@pytest.mark.parametrize("tau", [0, 1, 2, 8, 100000])
def test_checkpy_cases_device_encoder(tch, golden, case_idx, tau):
    c = golden["cases"][case_idx]
    A, _ = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
    calls = A.astype(np.uint64)
    with tch.Solver.from_calls(calls, tau=tau) as s:
        info = s.info()
        H, _ = s.run(128)
    assert "%016x" % oracle.rollhash(H) == c["rollhash"]
    if tau > 0:  # same encoding sizes as the reference host (main.rs:366-444)
        x, cnt = oracle.dense_ranks(calls)
        e = oracle.encode(x, cnt, tau)
        assert info["d_onehot"] == e.D and info["n_rare"] == len(e.js) and info["tau"] == tau


def test_run_calls_contract(tch):
    rng = np.random.default_rng(9)
    A = rng.integers(0, 2**64 - 1, size=(333, 77), dtype=np.uint64, endpoint=True) % np.uint64(13)
    A[A == 0] = 0
    A[:, :5] = rng.integers(1, 2**63, size=(333, 5), dtype=np.uint64)  # 64-bit ids, all distinct
    A[::7, 5] = A[0, 5]
    H, secs, tau, sink = tch.run_calls(A, stripe=40)
    assert tau >= 2
    assert [c[0] for c in sink.calls] == list(range(0, 333, 40))
    upper_equal(H, oracle.hamming(oracle.dense_ranks(A)[0]))


@pytest.mark.parametrize("n,L", [(1, 1), (2, 1), (9, 3), (129, 64), (257, 65), (300, 0), (5, 200)])
def test_edge_shapes_device_encoder(tch, n, L):
    rng = np.random.default_rng(n + 7 * L)
    A = rng.integers(0, 5, size=(n, L)).astype(np.uint64)
    with tch.Solver.from_calls(A, tau=3) as s:
        H, _ = s.run(64)
    x = oracle.dense_ranks(A)[0] if L else np.zeros((n, 1), np.uint16)
    upper_equal(H, oracle.hamming(x))


def test_many_alleles_per_locus(tch):
    """A locus near the 65 535-allele limit and one above it."""
    n = 70000
    rng = np.random.default_rng(1)
    A = np.zeros((n, 2), np.uint64)
    A[:, 0] = rng.permutation(n).astype(np.uint64) % np.uint64(65535) + np.uint64(1)
    A[:, 1] = rng.integers(1, 4, n)
    with tch.Solver.from_calls(A, tau=2) as s:
        info = s.info()
    assert info["n"] == n
    A[:, 0] = np.arange(1, n + 1, dtype=np.uint64)  # 70 000 distinct ids
    with pytest.raises(tch.TchError, match="65535"):
        tch.Solver.from_calls(A, tau=2)


def test_longtail_sample_device_vs_host_encoder(tch):
    synth = __import__("importlib").import_module("cgmlst-hamming-gpu_gb300.synth")
    A = synth.longtail(n=3000, L=400, seed=5)
    x, nd = tch.dense_ranks(A)
    for tau in (32, 128):
        enc = tch.encode_host(x, nd, tau)
        with tch.Solver.from_calls(A, tau=tau) as s:
            info = s.info()
            Hd, _ = s.run(512)
        assert info["d_onehot"] == enc.D and info["n_rare"] == enc.n_rare
        Hh, _, _, _ = tch.run(enc, stripe=512)
        iu = np.triu_indices(3000, 1)
        np.testing.assert_array_equal(Hd[iu], Hh[iu])
    upper_equal(Hd, oracle.hamming(x))


def test_rare_term_mode_reported(tch, pkg):
    rng = np.random.default_rng(12)
    A = rng.integers(1, 30, size=(200, 40)).astype(np.uint64)
    with tch.Solver.from_calls(A, tau=8) as s:
        info = s.info()
        H, _ = s.run(64)
    upper_equal(H, oracle.hamming(oracle.dense_ranks(A)[0]))
    x, cnt = oracle.dense_ranks(A)
    assert info["n_rare"] == len(oracle.encode(x, cnt, 8).js)
    assert info["rare_dense"] in (0, 1)


def test_more_loci_than_threads(tch):
    """More loci than one CTA pass of the rare-count kernel covers (1024)."""
    rng = np.random.default_rng(21)
    n, L = 400, 2500
    A = rng.integers(1, 12, size=(n, L)).astype(np.uint64)
    A[rng.random((n, L)) < 0.02] = 0
    x = oracle.dense_ranks(A)[0]
    ref = oracle.hamming(x)
    for tau in (4, 64, 1000):
        with tch.Solver.from_calls(A, tau=tau) as s:
            H, _ = s.run(96)
        upper_equal(H, ref)


def test_wide_stripe_blocks(tch):
    """n above 65 536 columns: the rare counts of a row take several passes
    of the shared-memory counters.  Rows checked against the oracle's block."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(33)
    n, L = 70001, 12
    A = rng.integers(1, 3000, size=(n, L)).astype(np.uint64)  # ~23 rows per allele: rare at tau 64
    A[:, :3] = rng.integers(1, 4, size=(n, 3))  # frequent loci
    x = oracle.dense_ranks(A)[0]
    with tch.Solver.from_calls(A, tau=64) as s:
        assert s.info()["n_rare"] > 0
        for r0, rows in ((0, 200), (4097, 131), (n - 300, 300)):
            ldo = (n - r0 + 7) // 8 * 8
            out = torch.zeros((rows, ldo), dtype=torch.int16, device="cuda")
            s.stripe(r0, rows, out.data_ptr(), ldo, torch.cuda.current_stream().cuda_stream)
            s.check()
            got = out.cpu().numpy().view(np.uint16)
            ref = oracle.hamming_block(x, r0, r0 + rows, r0, n)
            for r in range(rows):
                np.testing.assert_array_equal(got[r, r + 1: n - r0], ref[r, r + 1:])
