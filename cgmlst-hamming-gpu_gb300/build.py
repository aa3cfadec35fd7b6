"""In-tree build of libtch.so (CUDA, sm_103a) and the command-line host.

    python -m build            (from this directory)   or   build.build()

nvcc compiles each translation unit in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; the objects are
linked into ``lib/libtch.so`` (static CUDA runtime, so the library needs only
the driver).  The CLI (``host/cgmlst_hamming_gpu.cpp``) is compiled with g++
into ``bin/cgmlst-hamming-gpu`` and linked against ``lib/libtch.so``, and the
ranks-file front end (``host/ranks_tool.cpp``) into ``bin/tch-ranks``.
Nothing is installed outside this directory.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
LIB = os.path.join(HERE, "lib")
BIN = os.path.join(HERE, "bin")
OBJ = os.path.join(LIB, "obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["tch_solver.cu", "k_popc.cu", "k_expand.cu", "k_tc.cu", "k_encode.cu", "k_rare.cu", "k_mlp.cu",
              "serve.cu", "batch.cu", "format.cu", "encode_host.cpp", "noalloc.cu", "k_parse.cu",
              "k_linkage.cu"]
LIBNAME = "libtch.so"
CLI_NAME = "cgmlst-hamming-gpu"


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, "tch.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def compile_unit(src: str, extra=()) -> str:
    os.makedirs(OBJ, exist_ok=True)
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _newer(obj, [src] + _headers()):
        return obj
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "-I", INCLUDE, "-I", CSRC,
           "-c", src, "-o", obj + ".tmp", *extra]
    _run(cmd)
    os.replace(obj + ".tmp", obj)
    return obj


def build_lib(verbose: bool = False) -> str:
    os.makedirs(LIB, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_unit, srcs))
    out = os.path.join(LIB, LIBNAME)
    if not _newer(out, objs):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", out + ".tmp", "-lpthread"])
        os.replace(out + ".tmp", out)
    if verbose:
        print("built", out)
    return out


def build_cli(verbose: bool = False) -> str | None:
    src = os.path.join(HOST, "cgmlst_hamming_gpu.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(BIN, exist_ok=True)
    out = os.path.join(BIN, CLI_NAME)
    lib = os.path.join(LIB, LIBNAME)
    deps = [src, lib, os.path.join(INCLUDE, "tch.h")] + [
        os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".h", ".hpp"))]
    if not _newer(out, deps):
        cmd = ["g++", "-O3", "-std=c++17", "-pthread", "-I", INCLUDE, "-I", HOST, src, "-o", out + ".tmp",
               "-L", LIB, "-ltch", "-Wl,-rpath,$ORIGIN/../lib", "-ldl"]
        try:  # deflate through zlib when its header and library are present
            _run(cmd + ["-DTCH_HAVE_ZLIB", "-lz"])
        except RuntimeError:  # stored-block gzip (valid, uncompressed)
            _run(cmd)
        os.replace(out + ".tmp", out)
    if verbose:
        print("built", out)
    return out


def build_ranks_tool(verbose: bool = False) -> str | None:
    """bin/tch-ranks: the ranks-file front end (host/ranks_tool.cpp)."""
    src = os.path.join(HOST, "ranks_tool.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(BIN, exist_ok=True)
    out = os.path.join(BIN, "tch-ranks")
    lib = os.path.join(LIB, LIBNAME)
    if not _newer(out, [src, lib, os.path.join(INCLUDE, "tch.h")]):
        _run(["g++", "-O3", "-std=c++17", "-I", INCLUDE, src, "-o", out + ".tmp", "-L", LIB, "-ltch",
              "-Wl,-rpath,$ORIGIN/../lib"])
        os.replace(out + ".tmp", out)
    if verbose:
        print("built", out)
    return out


def build_peak(verbose: bool = False) -> str:
    """bin/tch-peak: the instruction-throughput probe (csrc/peak.cu)."""
    src = os.path.join(CSRC, "peak.cu")
    os.makedirs(BIN, exist_ok=True)
    out = os.path.join(BIN, "tch-peak")
    if not _newer(out, [src] + _headers()):
        _run([nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-I", INCLUDE, "-I", CSRC, src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    if verbose:
        print("built", out)
    return out


def build(verbose: bool = False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        fpeak = ex.submit(build_peak, verbose)
        lib = build_lib(verbose)
        cli = build_cli(verbose)
        build_ranks_tool(verbose)
        fpeak.result()
    return lib, cli


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
