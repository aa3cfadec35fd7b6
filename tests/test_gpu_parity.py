"""GPU parity: every cell of the upper triangle, through the C ABI, against
the oracle's brute-force count (check.py:39-44), on the reference's own test
inputs (check.py's generator and flag space) and on edge shapes."""
import os

import numpy as np
import pytest

import oracle
import refgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tch(pkg):
    assert pkg.device_count() > 0, "no CUDA device visible"
    return pkg


def kernels(tch):
    return [k for k in ("popc", "tc_f4", "tc_f8", "tc_i8", "tc_f16", "mma_b1") if tch.kernel_available(k)]


def upper_equal(H, ref):
    n = ref.shape[0]
    iu = np.triu_indices(n, 1)
    bad = np.nonzero(H[iu] != ref[iu])[0]
    if len(bad):
        i, j = iu[0][bad[0]], iu[1][bad[0]]
        raise AssertionError(f"{len(bad)} cells differ; first H[{i},{j}] = {H[i, j]}, oracle {ref[i, j]}")


@pytest.fixture(scope="module")
def checkpy_inputs(golden):
    out = []
    for c in golden["cases"]:
        A, _ = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
        x = refgen.ranks_of(A)
        out.append((c, A, x, oracle.hamming(x)))
    return out


@pytest.mark.parametrize("case_idx", [0, 1, 2])
@pytest.mark.parametrize("tau,stripe", [(None, 512), (2, 512), (100000, 512), (None, 64), (1, 8), (4, 200)])
def test_tch_run_checkpy_cases(tch, checkpy_inputs, golden, case_idx, tau, stripe):
    c, A, x, ref = checkpy_inputs[case_idx]
    xr, nd = tch.dense_ranks(A.astype(np.uint64))
    if tau is None:
        tau = tch.choose_tau(xr, nd, stripe)
    enc = tch.encode_host(xr, nd, tau)
    for k in kernels(tch):
        tch.set_kernel(k)
        try:
            H, secs, rare_gpu, sink = tch.run(enc, stripe=stripe)
        finally:
            tch.set_kernel("auto")
        upper_equal(H, ref)
        assert "%016x" % oracle.rollhash(H) == c["rollhash"], k
        assert rare_gpu == 1


def test_callback_contract(tch):
    rng = np.random.default_rng(1)
    A = rng.integers(0, 9, size=(203, 33)).astype(np.uint64)
    x, nd = tch.dense_ranks(A)
    enc = tch.encode_host(x, nd, 3)
    sink = tch.StripeSink(203, keep_raw=True)
    tch.run(enc, stripe=48, sink=sink)
    assert [c[0] for c in sink.calls] == list(range(0, 203, 48))
    for r0, rows, w in sink.calls:
        assert rows == min(48, 203 - r0) and w == 203 - r0
    ref = oracle.hamming(x)
    for (r0, rows, w), s in zip(sink.calls, sink.raw):
        for r in range(rows):
            np.testing.assert_array_equal(s[r, r + 1:], ref[r0 + r, r0 + r + 1:])


def test_host_rare_fallback(tch, checkpy_inputs):
    """tch.cu:105, 140-144: rare pairs applied on the host when they do not fit."""
    c, A, x, ref = checkpy_inputs[0]
    xr, nd = tch.dense_ranks(A.astype(np.uint64))
    enc = tch.encode_host(xr, nd, 64)
    assert enc.n_rare > 0
    os.environ["TCH_FORCE_HOST_RARE"] = "1"
    try:
        H, secs, rare_gpu, _ = tch.run(enc, stripe=64)
    finally:
        del os.environ["TCH_FORCE_HOST_RARE"]
    assert rare_gpu == 0
    upper_equal(H, ref)


@pytest.mark.parametrize("stripe", [136, 1024, 1030])
@pytest.mark.parametrize("pull", ["1", "0"])
def test_tch_run_partner_upload_paths(tch, checkpy_inputs, pull, stripe):
    """tch_run uploads the partner lists ahead of the stripes that use them:
    copied by cudaMemcpyAsync, or read by the GPU from host memory
    (TCH_HOST_PULL=1, where the platform allows it).  Both in any order.
    Stripes of 1 024 rows and more start with their first stripe in
    sub-stripes of a quarter (multiples of 128 rows): 1 024 -> 4 x 256,
    1 030 -> 384 + 384 + 262, then 1 024 + 476 / 470 rows."""
    c, A, x, ref = checkpy_inputs[2]
    xr, nd = tch.dense_ranks(A.astype(np.uint64))
    enc = tch.encode_host(xr, nd, 64)
    rng = np.random.default_rng(5)
    for i in range(0, enc.n, 3):  # every third row unsorted
        seg = enc.js[enc.start[i]:enc.start[i + 1]]
        rng.shuffle(seg)
    os.environ["TCH_HOST_PULL"] = pull
    try:
        H, _, rare_gpu, sink = tch.run(enc, stripe=stripe)
    finally:
        del os.environ["TCH_HOST_PULL"]
    assert rare_gpu == 1
    assert [c[0] for c in sink.calls] == list(range(0, enc.n, stripe))
    upper_equal(H, ref)


@pytest.mark.parametrize("row", [300, 700, 1200])
def test_invalid_rare_pair_in_a_sub_stripe(tch, row):
    """An invalid partner in a sub-stripe of the first stripe (rows 256-511,
    512-767 of a 1 024-row stripe) or in a later stripe is still an error."""
    rng = np.random.default_rng(8)
    A = rng.integers(0, 400, size=(1400, 12)).astype(np.uint64)
    x, nd = tch.dense_ranks(A)
    enc = tch.encode_host(x, nd, 1000)
    a, b = int(enc.start[row]), int(enc.start[row + 1])
    assert b > a
    enc.js = enc.js.copy()
    enc.js[a] = row  # j == i
    with pytest.raises(tch.TchError, match="rare"):
        tch.run(enc, stripe=1024)


def test_unsorted_partner_lists(tch, checkpy_inputs):
    """The reference host fills partner lists in any order (main.rs:436-442)."""
    c, A, x, ref = checkpy_inputs[1]
    xr, nd = tch.dense_ranks(A.astype(np.uint64))
    enc = tch.encode_host(xr, nd, 16)
    rng = np.random.default_rng(0)
    for i in range(enc.n):
        seg = enc.js[enc.start[i]:enc.start[i + 1]]
        rng.shuffle(seg)
    for k in kernels(tch):
        with tch.Solver.from_encoding(enc, kernel=k) as s:
            assert s.info()["rare_sorted"] == 0 or enc.n_rare == 0
            H, _ = s.run(100)
        upper_equal(H, ref)


@pytest.mark.parametrize("n", [1, 2, 7, 8, 9, 127, 128, 129, 255, 257])
@pytest.mark.parametrize("L", [1, 63, 64, 65])
def test_edge_shapes(tch, n, L):
    rng = np.random.default_rng(n * 1000 + L)
    A = rng.integers(0, 6, size=(n, L)).astype(np.uint64)
    A[:, : max(1, L // 3)] = rng.integers(0, 300, size=(n, max(1, L // 3)))
    x, nd = tch.dense_ranks(A)
    ref = oracle.hamming(x)
    for tau in (2, 5):
        enc = tch.encode_host(x, nd, tau)
        for k in kernels(tch):
            with tch.Solver.from_encoding(enc, kernel=k) as s:
                H, _ = s.run(8 if n > 50 else 3)
            upper_equal(H, ref)


def test_all_equal_and_all_missing(tch):
    n, L = 300, 200
    for A in (np.full((n, L), 7, np.uint64), np.zeros((n, L), np.uint64),
              np.tile(np.arange(1, L + 1, dtype=np.uint64), (n, 1))):
        x, nd = tch.dense_ranks(A)
        enc = tch.encode_host(x, nd, 2)
        for k in kernels(tch):
            with tch.Solver.from_encoding(enc, kernel=k) as s:
                H, _ = s.run(128)
            upper_equal(H, oracle.hamming(x))


def test_max_distance_65535_loci(tch):
    """Distances up to L = 65535 (the u16 limit, main.rs:349-351) stay exact."""
    n, L = 40, 65535
    rng = np.random.default_rng(3)
    A = np.tile(np.arange(1, n + 1, dtype=np.uint64)[:, None], (1, L))  # every pair differs everywhere
    A[5] = A[6]  # one identical pair
    A[7, : L // 2] = 0  # half missing
    x, nd = tch.dense_ranks(A)
    enc = tch.encode_host(x, nd, 1 << 20)  # all rare: pure GEMM P Pt - R
    ref = oracle.hamming(x)
    assert ref.max() == 65535
    for k in kernels(tch):
        with tch.Solver.from_encoding(enc, kernel=k) as s:
            H, _ = s.run(16)
        upper_equal(H, ref)
    enc = tch.encode_host(x, nd, 1)  # all frequent: one-hot GEMM
    for k in kernels(tch):
        with tch.Solver.from_encoding(enc, kernel=k) as s:
            H, _ = s.run(16)
        upper_equal(H, ref)


def test_invalid_rare_pair_is_an_error(tch):
    rng = np.random.default_rng(2)
    A = rng.integers(0, 50, size=(60, 10)).astype(np.uint64)
    x, nd = tch.dense_ranks(A)
    enc = tch.encode_host(x, nd, 1000)
    assert enc.n_rare > 0
    bad = enc.js.copy()
    bad[0] = 60  # j == n
    enc.js = bad
    with pytest.raises(tch.TchError, match="rare"):
        tch.run(enc, stripe=16)
    enc.js[0] = 0  # j <= i
    with pytest.raises(tch.TchError, match="rare"):
        tch.run(enc, stripe=16)


def test_device_stripe_api(tch):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    n, L = 700, 120
    A = rng.integers(0, 40, size=(n, L)).astype(np.uint64)
    x, nd = tch.dense_ranks(A)
    enc = tch.encode_host(x, nd, 8)
    ref = oracle.hamming(x)
    for k in kernels(tch):
        with tch.Solver.from_encoding(enc, kernel=k) as s:
            r0, rows = 130, 300
            ldo = n - r0 + 24
            out = torch.zeros((rows, ldo), dtype=torch.int16, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            s.stripe(r0, rows, out.data_ptr(), ldo, stream)
            s.check()
            got = out.cpu().numpy().view(np.uint16)
            for r in range(rows):
                i = r0 + r
                np.testing.assert_array_equal(got[r, i - r0 + 1: n - r0], ref[i, i + 1:])


def test_k_chunked_operand(tch):
    """The operand rows split along K into several allocations (K tiling of
    the one-hot matrix): same distances as one allocation, for both solver
    builds."""
    rng = np.random.default_rng(17)
    n, L = 900, 300
    A = rng.integers(1, 60, size=(n, L)).astype(np.uint64)
    A[rng.random((n, L)) < 0.03] = 0
    x, nd = tch.dense_ranks(A)
    ref = oracle.hamming(x)
    enc = tch.encode_host(x, nd, 4)
    try:
        # rows are ~18.4 KB long and padded to 1024 rows: chunks of 2.5 KB / 8 KB of K
        for limit in (1024 * 2560, 1024 * 8192):
            tch.set_max_chunk_bytes(limit)
            with tch.Solver.from_encoding(enc, kernel="tc_f4") as s:
                info = s.info()
                H, _ = s.run(256)
            assert 1 < info["k_chunks"] <= 8
            upper_equal(H, ref)
            with tch.Solver.from_calls(A, tau=4) as s:
                info = s.info()
                H, _ = s.run(300)
            assert 1 < info["k_chunks"] <= 8
            upper_equal(H, ref)
        tch.set_max_chunk_bytes(1024)  # would need far more than 8 chunks
        with pytest.raises(tch.TchError, match="chunks"):
            tch.Solver.from_encoding(enc, kernel="tc_f4")
    finally:
        tch.set_max_chunk_bytes(0)
