"""Serving: new profiles against a resident database, through the C ABI
(tch_db_query, tch_server_*), every distance against the oracle's brute-force
count of the joint profile set (check.py:39-44)."""
import importlib
import threading

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
PKG = "cgmlst-hamming-gpu_gb300"


@pytest.fixture(scope="module")
def tch(pkg):
    assert pkg.device_count() > 0, "no CUDA device visible"
    return pkg


def expected(db_calls, q):
    """(q x db, q x q) distances by the oracle on the joint set."""
    n = len(db_calls)
    x = oracle.dense_ranks(np.concatenate([db_calls, q]))[0]
    m = len(q)
    qdb = oracle.hamming_block(x, n, n + m, 0, n)
    qq = oracle.hamming_block(x, n, n + m, n, n + m)
    return qdb, qq


def check(qdb, qq, exp_qdb, exp_qq):
    np.testing.assert_array_equal(qdb, exp_qdb)
    if qq is not None and len(qq) > 1:
        iu = np.triu_indices(len(qq), 1)
        np.testing.assert_array_equal(qq[iu], exp_qq[iu])


def profiles(n, L, seed, alleles=40):
    synth = importlib.import_module(PKG + ".synth")
    return synth.zipf_profiles(n, L, seed, 1.2, lambda rng, L: rng.integers(2, alleles, L),
                               lambda rng, L: rng.uniform(0.0, 0.05, L), hashed_frac=0.05)


@pytest.mark.parametrize("tau", [0, 2, 16, 100000])
def test_query_against_database(tch, tau):
    A = profiles(900, 150, seed=1)
    db_calls, q = A[:700], A[700:]
    q = q.copy()
    q[0, :20] = np.arange(1, 21, dtype=np.uint64) + np.uint64(2**62)  # ids the database has never seen
    q[1] = 0                                                          # all missing
    q[2] = db_calls[5]                                                # a database row again
    exp_qdb, exp_qq = expected(db_calls, q)
    with tch.Database(db_calls, tau=tau) as db:
        for m in (1, 3, 57, 200):
            qdb, qq = db.query(q[:m])
            check(qdb, qq, exp_qdb[:m], exp_qq[:m, :m])
    assert exp_qdb[2, 5] == 0


def test_query_wide_database(tch):
    """More database rows than one pass of the shared-memory counters (65 536)."""
    rng = np.random.default_rng(3)
    n, L = 70001, 10
    A = rng.integers(1, 4000, size=(n + 40, L)).astype(np.uint64)  # mostly rare alleles
    A[:, :2] = rng.integers(1, 5, size=(n + 40, 2))
    with tch.Database(A[:n], tau=64) as db:
        qdb, qq = db.query(A[n:])
    exp_qdb, exp_qq = expected(A[:n], A[n:])
    check(qdb, qq, exp_qdb, exp_qq)


def test_server_results_same_alone_and_in_the_mix(tch):
    A = profiles(1500, 200, seed=4)
    db_calls = A[:1000]
    rng = np.random.default_rng(5)
    batches = []
    for _ in range(14):
        m = int(rng.integers(1, 120))
        idx = rng.integers(1000, 1500, size=m)
        batches.append(A[idx].copy())
    with tch.Database(db_calls) as db:
        alone = [db.query(b) for b in batches]
        with tch.Server(db, slots=4) as sv:
            # submitted from several threads at once: they run concurrently
            ids = [None] * len(batches)

            def put(k):
                ids[k] = sv.submit(batches[k])

            ts = [threading.Thread(target=put, args=(k,)) for k in range(len(batches))]
            for t in ts:
                t.start()
            for t in ts:
                t.join()
            mixed = [sv.wait(i) for i in ids]
    for b, (qa, qqa), (qm, qqm, queued, lat) in zip(batches, alone, mixed):
        np.testing.assert_array_equal(qm, qa)
        if len(b) > 1:
            iu = np.triu_indices(len(b), 1)
            np.testing.assert_array_equal(qqm[iu], qqa[iu])
        assert lat >= queued >= 0
        exp_qdb, exp_qq = expected(db_calls, b)
        check(qm, qqm, exp_qdb, exp_qq)


def test_server_admission_by_memory(tch):
    """A budget below two requests runs them one at a time, still exact."""
    A = profiles(800, 120, seed=6)
    with tch.Database(A[:600]) as db:
        budget = db.query_bytes(100) + db.query_bytes(100) // 2
        with tch.Server(db, slots=3, budget=budget) as sv:
            ids = [sv.submit(A[600 + 50 * k: 700 + 50 * k]) for k in range(3)]
            res = [sv.wait(i) for i in ids]
    for k, (qdb, qq, queued, lat) in enumerate(res):
        exp_qdb, exp_qq = expected(A[:600], A[600 + 50 * k: 700 + 50 * k])
        check(qdb, qq, exp_qdb, exp_qq)


def test_query_errors(tch):
    A = profiles(300, 50, seed=7)
    with tch.Database(A[:200]) as db:
        with pytest.raises(tch.TchError):
            db.query(A[200:, :40])  # wrong locus count


def test_query_against_k_chunked_database(tch):
    """A database whose operand rows are split along K into several
    allocations: the new profiles' rows follow the same split."""
    A = profiles(600, 300, seed=9, alleles=120)
    try:
        tch.set_max_chunk_bytes(1024 * 512)  # rows padded to 512 -> chunks of 1 KB of K
        with tch.Database(A[:500], tau=8) as db:
            assert db.info()["k_chunks"] > 1
            qdb, qq = db.query(A[500:])
    finally:
        tch.set_max_chunk_bytes(0)
    exp_qdb, exp_qq = expected(A[:500], A[500:])
    check(qdb, qq, exp_qdb, exp_qq)
