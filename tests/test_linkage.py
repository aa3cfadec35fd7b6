"""Consumers of the distance matrix: the minimum spanning tree, single-linkage
clusters and nearest neighbours (the uses the reference's documentation names
for the matrix, docs/index.html "The problem"; the reference has no code for
them).

CPU: the oracle's Prim tree equals a plain Kruskal under the same strict edge
order and has the weight of scipy's tree, its threshold components equal the
cut of that tree by the library's host cut (tch_mst_clusters) and scipy's
single-linkage clusters, and its neighbours equal a sort of every row.
GPU: the device MST, clusters and neighbours equal the oracle's exactly, on
the check.py cases, on the 2 000 x 1 142 synthetic set, on profile sets full
of ties, and on arbitrary symmetric matrices in device memory (values over the
whole u16 range, diagonal and padding set to 0 so that reading them would
show)."""
import numpy as np
import pytest

import oracle
import refgen

M21 = (1 << 21) - 1


def kruskal(H):
    n = H.shape[0]
    keys = sorted((int(H[i, j]) << 42) | (i << 21) | j for i in range(n) for j in range(i + 1, n))
    p = list(range(n))

    def find(x):
        while p[x] != x:
            p[x] = p[p[x]]
            x = p[x]
        return x

    out = []
    for k in keys:
        a, b = find((k >> 21) & M21), find(k & M21)
        if a != b:
            p[max(a, b)] = min(a, b)
            out.append(k)
    return [((k >> 21) & M21, k & M21, k >> 42) for k in out]


def tie_heavy(rng, n, L=6, alleles=3):
    A = rng.integers(0, alleles + 1, size=(n, L))
    return oracle.hamming_numpy(A)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_mst_is_kruskal(seed):
    rng = np.random.default_rng(seed)
    H = tie_heavy(rng, int(rng.integers(2, 60)))
    u, v, w = oracle.mst(H)
    assert list(zip(u.tolist(), v.tolist(), w.tolist())) == kruskal(H)


@pytest.mark.parametrize("seed", range(6))
def test_tree_cut_equals_threshold_components(pkg, seed):
    """The library's host cut of the oracle's tree against the oracle's
    components of the threshold graph (computed without any tree)."""
    rng = np.random.default_rng(10 + seed)
    H = tie_heavy(rng, int(rng.integers(1, 80)), L=int(rng.integers(1, 9)))
    u, v, w = oracle.mst(H)
    thr = [0, 1, 2, 3, 7, 65535, 2, 0]
    np.testing.assert_array_equal(pkg.mst_clusters(H.shape[0], u, v, w, thr), oracle.clusters(H, thr))
    # edges in any order give the same labels
    perm = rng.permutation(len(u))
    np.testing.assert_array_equal(pkg.mst_clusters(H.shape[0], u[perm], v[perm], w[perm], thr),
                                  oracle.clusters(H, thr))


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_scipy(seed):
    """An independent pin of the oracle: scipy's minimum spanning tree has the
    same total weight (ties may pick other edges, never another weight; the
    weights are shifted by 1 because scipy reads a 0 as no edge), and scipy's
    single-linkage hierarchy cut at each threshold gives the same partition as
    the oracle's threshold components."""
    from scipy.cluster.hierarchy import fcluster, linkage
    from scipy.sparse.csgraph import minimum_spanning_tree
    from scipy.spatial.distance import squareform

    rng = np.random.default_rng(20 + seed)
    n = int(rng.integers(2, 70))
    H = tie_heavy(rng, n, L=int(rng.integers(1, 9)))
    _, _, w = oracle.mst(H)
    T = minimum_spanning_tree(np.triu(H.astype(np.float64) + 1, 1))
    assert T.nnz == n - 1
    assert round(T.sum()) - (n - 1) == int(w.astype(np.int64).sum())
    Z = linkage(squareform(H.astype(np.float64), checks=False), method="single")
    thr = [0, 1, 2, 3, 5, 8]
    lab = oracle.clusters(H, thr)
    for t, th in enumerate(thr):
        f = fcluster(Z, th, criterion="distance")
        first = {}
        for i, c in enumerate(f.tolist()):
            first.setdefault(c, i)  # a cluster's label: its smallest member
        np.testing.assert_array_equal(lab[t], [first[c] for c in f.tolist()])


def test_tree_cut_rejects_bad_edges(pkg):
    with pytest.raises(pkg.TchError, match="not between"):
        pkg.mst_clusters(3, [0], [3], [1], [1])
    with pytest.raises(pkg.TchError, match="not between"):
        pkg.mst_clusters(3, [1], [1], [1], [1])
    with pytest.raises(pkg.TchError, match="one entry per edge"):
        pkg.mst_clusters(3, [0, 1], [1, 2], [1], [1])
    assert pkg.mst_clusters(0, [], [], [], [4]).shape == (1, 0)
    np.testing.assert_array_equal(pkg.mst_clusters(1, [], [], [], [0, 9]), [[0], [0]])


def test_oracle_neighbors_by_sort():
    rng = np.random.default_rng(3)
    H = tie_heavy(rng, 40)
    idx, dist = oracle.neighbors(H, 5)
    for i in range(40):
        want = sorted((int(H[i, j]), j) for j in range(40) if j != i)[:5]
        assert list(zip(dist[i].tolist(), idx[i].tolist())) == want


# ---------------------------------------------------------------------------------------------
# on the GPU
# ---------------------------------------------------------------------------------------------

def same_tree(got, H):
    want = oracle.mst(H)
    for g, w_ in zip(got, want):
        np.testing.assert_array_equal(g, w_)


def check_solver(pkg, calls, H, ks=(1, 5, 32), thr=(0, 1, 3, 10, 100, 65535)):
    n = H.shape[0]
    with pkg.Solver.from_calls(calls) as s:
        same_tree(s.mst(), H)
        np.testing.assert_array_equal(s.clusters(list(thr)), oracle.clusters(H, thr))
        for k in ks:
            if k < n:
                idx, dist = s.neighbors(k)
                wi, wd = oracle.neighbors(H, k)
                np.testing.assert_array_equal(dist, wd)
                np.testing.assert_array_equal(idx, wi)


@pytest.mark.gpu
def test_checkpy_cases(pkg, golden):
    for c in golden["cases"]:
        _, cells = refgen.checkpy_make(c["n"], c["L"], c["seed"], c["hashed"])
        tab = oracle.load_tsv(refgen.checkpy_tsv(cells, c["L"]))
        x, _ = oracle.dense_ranks(tab.calls)
        check_solver(pkg, tab.calls, oracle.hamming(x))


@pytest.mark.gpu
def test_small_config_2000x1142(pkg):
    import importlib

    synth = importlib.import_module(pkg.__name__ + ".synth")
    A = synth.small()
    x, _ = oracle.dense_ranks(A)
    check_solver(pkg, A, oracle.hamming(x), ks=(1, 10, 32), thr=(0, 5, 10, 50, 200, 1142))


@pytest.mark.gpu
@pytest.mark.parametrize("n,L,alleles", [(2, 3, 2), (3, 1, 1), (70, 6, 2), (300, 4, 3), (513, 12, 1)])
def test_tie_heavy_sets(pkg, n, L, alleles):
    rng = np.random.default_rng(n)
    A = rng.integers(0, alleles + 1, size=(n, L)).astype(np.uint64)
    check_solver(pkg, A, oracle.hamming_numpy(A).astype(np.uint16))


@pytest.mark.gpu
def test_identical_and_empty_profiles(pkg):
    """Every distance 0: the tree is the star (0, x) and the neighbours are the
    lowest other indices."""
    A = np.zeros((90, 20), np.uint64)
    A[:45] = 7  # identical profiles; the rest have no calls at all
    H = np.zeros((90, 90), np.uint16)
    check_solver(pkg, A, H)
    with pkg.Solver.from_calls(A) as s:
        u, v, w = s.mst()
    assert (u == 0).all() and (v == np.arange(1, 90)).all() and (w == 0).all()


@pytest.mark.gpu
def test_one_profile_and_bad_k(pkg):
    torch = pytest.importorskip("torch")
    d = torch.zeros((1, 8), dtype=torch.int16, device="cuda:0")
    torch.cuda.synchronize()
    assert all(len(a) == 0 for a in pkg.mst_device(d.data_ptr(), 8, 1))
    with pytest.raises(pkg.TchError, match="below n"):
        pkg.neighbors_device(d.data_ptr(), 8, 1, 1)
    with pkg.Solver.from_calls(np.arange(1, 41, dtype=np.uint64).reshape(8, 5)) as s:
        for k in (0, 33, 8):
            with pytest.raises(pkg.TchError):
                s.neighbors(k)


def device_matrix(torch, H, pad=0):
    n = H.shape[0]
    ld = (n + 7) // 8 * 8 + pad
    Hp = np.zeros((n, ld), np.uint16)  # padding columns and the diagonal read as 0 if touched
    Hp[:, :n] = H
    np.fill_diagonal(Hp[:, :n], 0)
    d = torch.from_numpy(Hp.view(np.int16)).to("cuda:0")
    torch.cuda.synchronize()  # the consumers run on a stream of their own
    return d, ld


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 3, 9, 64, 257, 1500])
def test_device_matrix_any_values(pkg, n):
    """Arbitrary symmetric matrices: values over the whole u16 range (high
    bytes included), many ties, the row stride wider than the row."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    for scale in (3, 257, 65535):
        M = rng.integers(0, scale + 1, size=(n, n)).astype(np.uint16)
        H = np.triu(M, 1)
        H = H + H.T
        d, ld = device_matrix(torch, H, pad=8 * (n % 3))
        stream = torch.cuda.current_stream().cuda_stream
        same_tree(pkg.mst_device(d.data_ptr(), ld, n, stream), H)
        for k in (1, 7, 32):
            if k < n:
                idx, dist = pkg.neighbors_device(d.data_ptr(), ld, n, k, stream)
                wi, wd = oracle.neighbors(H, k)
                np.testing.assert_array_equal(dist, wd)
                np.testing.assert_array_equal(idx, wi)


@pytest.mark.gpu
def test_device_matrix_rejects_bad_layout(pkg):
    torch = pytest.importorskip("torch")
    d = torch.zeros((16, 16), dtype=torch.int16, device="cuda:0")
    with pytest.raises(pkg.TchError, match="multiple of 8"):
        pkg.mst_device(d.data_ptr(), 12, 10)
    with pytest.raises(pkg.TchError, match="aligned"):
        pkg.neighbors_device(d.data_ptr() + 2, 16, 10, 3)
