"""The benchmark's workload shapes against the oracle, on the GPU.

* small: 2 000 profiles x 1 142 loci (lognormal distinct counts, mean 40,
  Zipf 1.1, 2 % missing): the whole upper triangle, bit-exact against the
  brute-force count (tensorcore/rs/check.py:39-44), for the analytic tau, the
  learned tau, tau = 2 (every allele seen twice or more is frequent) and a
  tau above every count (every shared allele is rare), through the device
  encoder, and through the reference's C ABI (tch_run with host-encoded bits
  and pair lists).
* founders: all-frequent loci at the full 5 000 loci (50 founder alleles per
  locus, ~250 k one-hot columns) with fewer profiles, in one K chunk and in
  the K-chunked operand, spread rows against the oracle.
* zipf_big's law (Zipf 1.1, 3 000 loci) at reduced n, spread rows.

The distances are integers: the tolerance is zero."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def synth(pkg):
    import importlib

    return importlib.import_module(pkg.__name__ + ".synth")


@pytest.fixture(scope="module")
def small(synth):
    A = synth.small()
    x = oracle.dense_ranks(A)[0]
    return A, x, oracle.hamming(x)


def upper_equal(H, ref):
    iu = np.triu_indices(ref.shape[0], 1)
    bad = int((H[iu] != ref[iu]).sum())
    assert bad == 0, f"{bad} of {len(iu[0])} cells differ from the oracle"


def spread_rows_equal(H, x, rows=48):
    n = x.shape[0]
    for i in sorted(set(np.linspace(0, n - 2, rows).astype(int).tolist())):
        want = oracle.hamming_block(x, i, i + 1, i + 1, n)[0]
        got = H[i, i + 1:n]
        bad = int((got != want).sum())
        assert bad == 0, f"row {i}: {bad} cells differ from the oracle"


@pytest.mark.parametrize("tau", ["analytic", "learned", 2, 1 << 20])
def test_small_config_whole_triangle(pkg, small, tau):
    A, x, ref = small
    if tau == "learned":
        if not os.path.exists(pkg.TAU_MLP_PATH):
            pytest.skip("no shipped tau model")
        pkg.set_tau_mlp(pkg.load_tau_mlp())
        t = 0
    else:
        t = 0 if tau == "analytic" else tau
    try:
        with pkg.Solver.from_calls(A, tau=t) as s:
            info = s.info()
            H, _ = s.run(512)
    finally:
        pkg.set_tau_mlp(None)
    assert info["n"] == 2000
    upper_equal(H, ref)


def test_small_config_reference_abi(pkg, small):
    """tch_run, the reference's entry point, with the reference host's encoding
    at the reference's own tau choice (main.rs:167-198)."""
    A, x, ref = small
    xp, nd = pkg.dense_ranks(A)
    tau = pkg.choose_tau(xp, nd, 512)
    enc = pkg.encode_host(xp, nd, tau)
    H, _, rare_gpu, _ = pkg.run(enc, stripe=512)
    assert rare_gpu == 1
    upper_equal(H, ref)


@pytest.mark.parametrize("chunk_mb", [0, 96])
def test_founders_full_loci(pkg, synth, chunk_mb):
    n = 3000
    A = synth.founders(n=n)
    x = oracle.dense_ranks(A)[0]
    try:
        pkg.set_max_chunk_bytes(chunk_mb << 20)
        with pkg.Solver.from_calls(A, tau=16) as s:
            info = s.info()
            H, _ = s.run(1024)
    finally:
        pkg.set_max_chunk_bytes(0)
    assert info["d_onehot"] > 200_000, info  # every founder allele is a one-hot column
    if chunk_mb:
        assert info["k_chunks"] > 1, info
    spread_rows_equal(H, x)


def test_zipf_big_law_reduced(pkg, synth):
    A = synth.zipf_big(n=6000)
    x = oracle.dense_ranks(A)[0]
    with pkg.Solver.from_calls(A) as s:
        H, _ = s.run(2048)
    spread_rows_equal(H, x)


@pytest.mark.parametrize("sub_rows,group", [(0, 1), (256, 4), (1024, 16), (128, 8)])
def test_schedules_give_the_same_distances(pkg, small, sub_rows, group):
    """Sub-stripes of the rare counts and tile pass, and raster groups of the
    tile pass, change the order of the work, never a distance."""
    A, x, ref = small
    with pkg.Solver.from_calls(A, tau=256) as s:
        s.set_schedule(sub_rows, group)
        info = s.info()
        H, _ = s.run(2000)
    assert info["sub_rows"] == sub_rows and info["tile_group"] == group
    upper_equal(H, ref)
