#!/usr/bin/env python3
"""Writes the golden fixtures of tests/golden/ from the reference's own code.

Run once, with the path of a checkout of the reference project:

    python tests/golden/make_golden.py <reference checkout> [--kat]

It imports the reference's exactness check (tensorcore/rs/check.py) and calls
its ``make`` and ``ref`` functions, and it runs the reference's synthetic
generator (python/gen_profiles.py) as a subprocess. Nothing else of the
reference is used. The outputs are small: SHA-256 digests of the generated
TSV text, of the allele matrices and of every expected output matrix, the
rolling checksums, and the full 300 x 97 case as an .npz file.

``--kat`` also rebuilds the 30 000 x 5 000 profiles of the reference's
published checksum (tensorcore/README.md:52, ``85724a9d7d090f9f``) with the
restated generator, after checking the restatement against gen_profiles.py on
a small shape, and computes the oracle's checksum of their distance matrix.
"""
import hashlib
import importlib.util
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import refgen  # noqa: E402
import oracle  # noqa: E402


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def mat_sha(M) -> str:
    return sha(np.ascontiguousarray(M, dtype="<i8").tobytes())


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if len(args) != 1:
        sys.exit("usage: make_golden.py <reference checkout> [--kat]")
    ref_root = args[0]
    kat = "--kat" in sys.argv
    spec = importlib.util.spec_from_file_location("ref_check", os.path.join(ref_root, "tensorcore/rs/check.py"))
    check = importlib.util.module_from_spec(spec)
    saved = sys.argv
    sys.argv = ["check.py", "/nonexistent"]  # its module-level TC default reads argv
    spec.loader.exec_module(check)
    sys.argv = saved

    out = {"generated_by": "tests/golden/make_golden.py", "cases": [], "gen_profiles": {}}
    for n, L, seed, hashed in refgen.CHECKPY_CASES:
        A, cells = check.make(n, L, seed, hashed)
        text = "FILE\t" + "\t".join(f"L{j}" for j in range(L)) + "\n"
        text += "".join(f"S{i}\t" + "\t".join(row) + "\n" for i, row in enumerate(cells))
        H = check.ref(A)
        case = {
            "n": n, "L": L, "seed": seed, "hashed": hashed,
            "tsv_sha256": sha(text.encode()),
            "A_sha256": mat_sha(A),
            "H_sha256": mat_sha(H),
            "rollhash": "%016x" % oracle.rollhash(H.astype(np.uint16)),
            "H_max": int(H.max()),
            "expected": {},
        }
        iu = np.triu(np.ones_like(H, dtype=bool))
        for name, want in [("full", H), ("lower", np.where(iu.T, H, 0)), ("upper", np.where(iu, H, 0)),
                           ("cap7", np.minimum(H, 7))]:
            case["expected"][name] = mat_sha(want)
        out["cases"].append(case)
        if (n, L) == (300, 97):
            np.savez_compressed(os.path.join(HERE, "checkpy_300x97.npz"), A=A.astype(np.int64),
                                H=H.astype(np.uint16))

    # gen_profiles.py on a small shape: pins the restated generator
    with tempfile.TemporaryDirectory() as d:
        for n, L in [(257, 131), (64, 1)]:
            p = os.path.join(d, "g.tsv")
            subprocess.check_call([sys.executable, os.path.join(ref_root, "python/gen_profiles.py"), str(n), str(L), p])
            with open(p, "rb") as f:
                out["gen_profiles"][f"{n}x{L}"] = sha(f.read())

    if kat:
        n, L = 30000, 5000
        P = refgen.gen_profiles(n, L)
        x = refgen.ranks_of(P)
        h = oracle.rollhash_ranks(x)
        out["kat_30000x5000"] = {
            "published": "85724a9d7d090f9f",
            "published_at": "tensorcore/README.md:52",
            "oracle": "%016x" % h,
            "profiles_sha256": mat_sha(P),
        }
    else:
        old = os.path.join(HERE, "golden.json")
        if os.path.exists(old):
            with open(old) as f:
                prev = json.load(f)
            if "kat_30000x5000" in prev:
                out["kat_30000x5000"] = prev["kat_30000x5000"]

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
