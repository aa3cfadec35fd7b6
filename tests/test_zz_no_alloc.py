"""tch_stripe_noalloc, the entry point for callers that may not allocate
device memory: its stripes must equal the oracle's brute-force count and the
allocating path's (tch_solver_from_bits + tch_solver_stripe) cell for cell,
on two calls in a row through the C ABI.  The distances are integers, so the
tolerance is zero.  A partner list with an invalid entry must fail with the
rare-CSR message, and the next valid call must succeed (the error word in the
shared array is cleared per call).

Collected last on purpose (file name), so a failure here never hides the
results of the other tests."""
import ctypes

import numpy as np
import oracle
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20


def bind(lib):
    f = lib.tch_stripe_noalloc
    v, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    f.argtypes = [i, i, v, sz, v, sz, v, v, sz, i, i, v, sz, v, ctypes.c_char_p, i]
    f.restype = i
    return f


def upper_rows(out, r0, rows, n):
    """The meaningful cells of a stripe: row r, columns c > r (j > i)."""
    return [out[r, r + 1: n - r0].copy() for r in range(rows)]


def test_noalloc_matches_allocating_path(pkg):
    torch = pytest.importorskip("torch")
    assert pkg.device_count() > 0
    f = bind(pkg.lib())
    rng = np.random.default_rng(2024)
    n, L = 1500, 400
    A = rng.integers(1, 40, size=(n, L)).astype(np.uint64)
    A[:, :60] = rng.integers(1, 3000, size=(n, 60))  # rare alleles -> many rare pairs
    A[rng.random((n, L)) < 0.04] = 0
    x, nd = pkg.dense_ranks(A)
    enc = pkg.encode_host(x, nd, 6)
    assert enc.n_rare > 0
    # callers may hand partner lists in any order
    for i in range(enc.n):
        seg = enc.js[enc.start[i]:enc.start[i + 1]]
        rng.shuffle(seg)

    dev = torch.device("cuda:0")
    dO = torch.from_numpy(enc.O).to(dev)
    dP = torch.from_numpy(enc.P).to(dev)
    dS = torch.from_numpy(enc.start.view(np.int32)).to(dev)
    dJ = torch.from_numpy(enc.js.view(np.int32)).to(dev)
    stream = torch.cuda.current_stream().cuda_stream
    err = ctypes.create_string_buffer(512)

    H = oracle.hamming(x)
    with pkg.Solver.from_encoding(enc) as s:
        for r0, rows in [(0, 640), (512, 700)]:  # two calls in a row, overlapping rows
            ldo = (n - r0 + 7) // 8 * 8
            ref = torch.full((rows, ldo), -1, dtype=torch.int16, device=dev)
            got = torch.full((rows, ldo), -1, dtype=torch.int16, device=dev)
            s.stripe(r0, rows, ref.data_ptr(), ldo, stream)
            s.check()
            rc = f(0, n, dO.data_ptr(), enc.K1, dP.data_ptr(), enc.K2, dS.data_ptr(), dJ.data_ptr(), enc.n_rare,
                   r0, rows, got.data_ptr(), ldo, stream, err, len(err))
            assert rc == 0, err.value.decode()
            torch.cuda.synchronize()
            a = ref.cpu().numpy().view(np.uint16)
            b = got.cpu().numpy().view(np.uint16)
            for r, (ra, rb) in enumerate(zip(upper_rows(a, r0, rows, n), upper_rows(b, r0, rows, n))):
                i = r0 + r
                np.testing.assert_array_equal(rb, H[i, i + 1:n])
                np.testing.assert_array_equal(ra, H[i, i + 1:n])


def test_noalloc_reports_an_invalid_partner_then_recovers(pkg):
    torch = pytest.importorskip("torch")
    f = bind(pkg.lib())
    rng = np.random.default_rng(77)
    n, L = 700, 200
    A = rng.integers(1, 30, size=(n, L)).astype(np.uint64)
    A[:, :40] = rng.integers(1, 900, size=(n, 40))
    x, nd = pkg.dense_ranks(A)
    enc = pkg.encode_host(x, nd, 5)
    assert enc.n_rare > 2
    dev = torch.device("cuda:0")
    dO = torch.from_numpy(enc.O).to(dev)
    dP = torch.from_numpy(enc.P).to(dev)
    dS = torch.from_numpy(enc.start.view(np.int32)).to(dev)
    stream = torch.cuda.current_stream().cuda_stream
    err = ctypes.create_string_buffer(512)
    ldo = (n + 7) // 8 * 8
    out = torch.zeros((n, ldo), dtype=torch.int16, device=dev)
    row = int(np.nonzero(np.diff(enc.start.astype(np.int64)))[0][0])  # a row with partners
    for bad in (n + 5, row):  # j >= n, then j == i (not in (i, n))
        js = enc.js.copy()
        js[enc.start[row]] = bad
        dJ = torch.from_numpy(js.view(np.int32)).to(dev)
        rc = f(0, n, dO.data_ptr(), enc.K1, dP.data_ptr(), enc.K2, dS.data_ptr(), dJ.data_ptr(), enc.n_rare, 0, n,
               out.data_ptr(), ldo, stream, err, len(err))
        assert rc != 0 and "rare CSR" in err.value.decode()
    dJ = torch.from_numpy(enc.js.view(np.int32)).to(dev)
    rc = f(0, n, dO.data_ptr(), enc.K1, dP.data_ptr(), enc.K2, dS.data_ptr(), dJ.data_ptr(), enc.n_rare, 0, n,
           out.data_ptr(), ldo, stream, err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint16)
    H = oracle.hamming(x)
    for i in range(n - 1):
        np.testing.assert_array_equal(got[i, i + 1:n], H[i, i + 1:n])


def test_noalloc_rejects_sizes_beyond_the_scratch(pkg):
    f = bind(pkg.lib())
    err = ctypes.create_string_buffer(512)
    n, K1, K2 = 4096, 1 << 15, 1024  # 4096 rows x 33792 bytes > 64 MiB
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = f(0, n, dummy, K1, dummy, K2, dummy, dummy, 0, 0, 128, dummy, n, None, err, len(err))
    assert rc != 0
    msg = err.value.decode()
    assert "scratch" in msg and str(SCRATCH_BYTES) in msg
