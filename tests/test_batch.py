"""Batched solves under a CUDA graph (tch_batch_*): every set's upper triangle
against the oracle's brute-force count, on the first run, on graph replays,
after the autotuner has picked another schedule, and under the persistent
schedule (two launches for the whole batch)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tch(pkg):
    assert pkg.device_count() > 0, "no CUDA device visible"
    return pkg


def uneven_sets(seed, count):
    rng = np.random.default_rng(seed)
    sets = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(0, np.log(900))))
        L = int(rng.choice([13, 64, 150, 333]))
        A = rng.integers(1, int(rng.integers(3, 200)), size=(n, L)).astype(np.uint64)
        A[rng.random((n, L)) < rng.uniform(0, 0.08)] = 0
        sets.append(A)
    return sets


def check_all(sets, buf, off, ld):
    for s, A in enumerate(sets):
        n = len(A)
        if n < 2:
            continue
        H = buf[off[s]:off[s] + n * ld[s]].reshape(n, ld[s])[:, :n]
        ref = oracle.hamming(oracle.dense_ranks(A)[0])
        iu = np.triu_indices(n, 1)
        np.testing.assert_array_equal(H[iu], ref[iu], err_msg=f"set {s} (n={n}, L={A.shape[1]})")


def upper_cells(sets, buf, off, ld):
    parts = []
    for s, A in enumerate(sets):
        n = len(A)
        H = buf[off[s]:off[s] + n * ld[s]].reshape(n, ld[s])[:, :n]
        parts.append(H[np.triu_indices(n, 1)])
    return np.concatenate(parts)


def test_batch_graph_runs_and_replays(tch):
    torch = pytest.importorskip("torch")
    sets = uneven_sets(1, 40)
    with tch.Batch(sets) as b:
        off, ld = b.layout()
        out = torch.zeros(int(off[-1]) + 8, dtype=torch.int16, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        b.run(out.data_ptr(), stream)
        b.check()
        first = out.cpu().numpy().view(np.uint16)[: int(off[-1])].copy()
        check_all(sets, first, off, ld)
        out.zero_()
        for _ in range(3):  # graph replays
            b.run(out.data_ptr(), stream)
        b.check()
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16)[: int(off[-1])], first)
        info = b.info()
        assert info["count"] == 40 and len(info["taus"]) == 40


def test_batch_autotune_keeps_results(tch):
    torch = pytest.importorskip("torch")
    sets = uneven_sets(2, 24)
    with tch.Batch(sets, taus=[0 if k % 2 else 4 for k in range(24)]) as b:
        off, ld = b.layout()
        out = torch.zeros(int(off[-1]) + 8, dtype=torch.int16, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        res = b.tune(out.data_ptr(), stream, reps=2)
        assert res["branches"] in (0, 1, 4, 8, 16, 32) and res["ms"] > 0
        out.zero_()
        b.run(out.data_ptr(), stream)
        b.check()
        check_all(sets, out.cpu().numpy().view(np.uint16), off, ld)
        b.set_schedule(3)
        out.zero_()
        b.run(out.data_ptr(), stream)
        b.check()
        check_all(sets, out.cpu().numpy().view(np.uint16), off, ld)


def test_batch_persistent_schedule(tch):
    """branches = 0: the rare counts of every set's rows in one launch, every
    set's tiles in one persistent tile pass; same distances, replayable, and
    switching back to streams keeps them."""
    torch = pytest.importorskip("torch")
    sets = uneven_sets(3, 48)
    sets.append(np.zeros((1, 5), np.uint64) + 1)  # a one-row set has no pairs
    with tch.Batch(sets, taus=[[0, 2, 1 << 20][k % 3] for k in range(len(sets))]) as b:
        off, ld = b.layout()
        out = torch.zeros(int(off[-1]) + 8, dtype=torch.int16, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        b.set_schedule(0)
        assert b.info()["branches"] == 0
        b.run(out.data_ptr(), stream)
        b.check()
        first = out.cpu().numpy().view(np.uint16)[: int(off[-1])].copy()
        check_all(sets, first, off, ld)
        out.zero_()
        for _ in range(2):
            b.run(out.data_ptr(), stream)
        b.check()
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16)[: int(off[-1])], first)
        b.set_schedule(4)  # cells on and below the diagonal are unspecified: compare the triangles
        out.zero_()
        b.run(out.data_ptr(), stream)
        b.check()
        np.testing.assert_array_equal(upper_cells(sets, out.cpu().numpy().view(np.uint16), off, ld),
                                      upper_cells(sets, first, off, ld))


def test_batch_persistent_wide_sets(tch):
    """Persistent schedule on sets wider than one tile column and row block,
    with K chunks of the operand (chunk limit 4 MB): job tables, per-set
    tensor maps and the K chunk boundaries inside one launch."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    sets = []
    for n, L in [(1500, 3016), (700, 1142), (257, 64), (2, 13), (129, 2794)]:
        A = rng.zipf(1.2, size=(n, L)).astype(np.uint64) % 4000 + 1
        A[rng.random((n, L)) < 0.03] = 0
        sets.append(A)
    try:
        tch.set_max_chunk_bytes(4 << 20)
        b = tch.Batch(sets)
    finally:
        tch.set_max_chunk_bytes(0)
    with b:
        off, ld = b.layout()
        out = torch.zeros(int(off[-1]) + 8, dtype=torch.int16, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        b.set_schedule(0)
        b.run(out.data_ptr(), stream)
        b.check()
        check_all(sets, out.cpu().numpy().view(np.uint16), off, ld)
