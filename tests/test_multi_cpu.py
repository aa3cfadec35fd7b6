"""The N > 1 path of bench.py on CPU: row shares of the upper triangle (no
data-path collective), every rank's share of the distances computed by the
oracle and gathered, the max-over-ranks time, with world_size 2 gloo ranks
(the host logic the GPU ranks run around their solves)."""
import importlib.util
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("n,ws", [(1000, 2), (63005, 2), (63005, 4), (63005, 8), (130, 3), (5, 2)])
def test_row_shares_cover_and_balance(n, ws):
    shares = load_bench().row_shares(n, ws)
    assert shares[0][0] == 0 and shares[-1][1] == n
    for (a, b), (c, d) in zip(shares, shares[1:]):
        assert b == c and a <= b
    pairs = [sum(n - 1 - i for i in range(a, b)) for a, b in shares]
    assert sum(pairs) == n * (n - 1) // 2
    if n >= 1000 * ws:  # equal pair counts up to one row
        assert max(pairs) / min(pairs) < 1.01


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, x, out_path):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    bench = load_bench()
    n = x.shape[0]
    a, b = bench.row_shares(n, ws)[rank]
    part = oracle.hamming_block(x, a, b, 0, n)  # this rank's rows, no exchange on the data path
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)  # the bench's max-over-ranks time
    parts = [None] * ws
    dist.all_gather_object(parts, (a, b, part))  # test only: gather to check the union
    if rank == 0:
        H = np.zeros((n, n), np.uint16)
        for a_, b_, p_ in parts:
            H[a_:b_] = p_
        np.save(out_path, H)
        with open(out_path + ".max", "w") as f:
            f.write(str(float(t.item())))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_shard_the_triangle(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    rng = np.random.default_rng(3)
    x = rng.integers(0, 7, size=(300, 40)).astype(np.uint16)
    out = str(tmp_path / "H.npy")
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, x, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    H = np.load(out)
    ref = oracle.hamming(x)
    iu = np.triu_indices(300, 1)
    np.testing.assert_array_equal(H[iu], ref[iu])
    assert open(out + ".max").read() == "2.0"
