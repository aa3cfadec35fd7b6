"""bench.py's reference arm (the reference's CPU path for the matrix, timed on
the host cores) on the CPU: one JSON line with the benchmark contract's keys,
the GPU arm's workload dict, a measured (not extrapolated) time per step, and
no part of the package loaded into the process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUNNER = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3", "--ref-stride", "97"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("LIBTCH_LOADED" if "libtch" in maps else "LIBTCH_ABSENT", file=sys.stderr)
"""


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "-c", RUNNER], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "LIBTCH_ABSENT" in r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "exact_pairs_per_s" and d["unit"] == "pairs/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["warmup"] >= 3 and d["steps"] == 2
    sys.path.insert(0, ROOT)
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert d["config"] == bench.workload_config(63005, 1142)
    # each step is about 1/97 of the triangle: its measured time, not an extrapolation to the whole
    assert d["ms_per_step"] < 60_000
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]


def test_strided_rows_cover_the_triangle():
    """s consecutive steps of the reference arm count every upper-triangle pair once."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ctypes

    import oracle

    rng = np.random.default_rng(3)
    x = rng.integers(0, 5, size=(301, 40)).astype(np.uint16)
    lib = oracle.lib()
    xp = x.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
    full = ctypes.c_uint64(0)
    pairs_full = lib.orc_upper_rows(xp, 301, 40, 0, 301, ctypes.byref(full), 0)
    tot_pairs, tot = 0, 0
    for k in range(7):
        acc = ctypes.c_uint64(0)
        tot_pairs += lib.orc_upper_rows_step(xp, 301, 40, k, 7, ctypes.byref(acc), 0)
        tot += acc.value
    assert tot_pairs == pairs_full == 301 * 300 // 2
    assert tot == full.value == int(np.triu(oracle.hamming(x), 1).astype(np.int64).sum())


def test_parity_rows_counts_planted_mismatches():
    """The bench's check of its timed output (the line's `parity`): the
    oracle's own matrix gives 0 mismatches, and one wrong cell planted in a
    sampled row (in a CPU tensor) is counted once."""
    import importlib.util

    import numpy as np
    import pytest

    torch = pytest.importorskip("torch")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    rng = np.random.default_rng(8)
    x = rng.integers(0, 6, size=(211, 37)).astype(np.uint16)
    H = oracle.hamming(x)
    out = torch.from_numpy(H.view(np.int16).copy())
    r = bench.parity_rows(x, out, rows=16)
    assert r["mismatches"] == 0 and r["rows"] >= 16 and r["cells"] > 0
    out[0, 5] += 1  # row 0 is always sampled
    assert bench.parity_rows(x, out, rows=16)["mismatches"] == 1
