"""cgmlst-hamming-gpu for GB300: Python bindings of libtch (ctypes).

The library is the product; this module only binds its C ABI (include/tch.h)
for Python callers, the tests and the benchmark.  It never computes a
distance itself and has no CPU fallback: if ``lib/libtch.so`` is missing the
import of any entry point raises.

    import importlib
    tch = importlib.import_module("cgmlst-hamming-gpu_gb300")
    x, nd = tch.dense_ranks(calls)                  # u64 ids -> u16 ranks
    enc = tch.encode_host(x, nd, tau=64)            # O, P bits + rare CSR
    H = tch.run(enc, stripe=512)                    # tch_run: full u16 matrix
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libtch.so")
CLI_PATH = os.path.join(HERE, "bin", "cgmlst-hamming-gpu")
RANKS_TOOL_PATH = os.path.join(HERE, "bin", "tch-ranks")

KERNELS = {"auto": 0, "popc": 1, "mma_b1": 2, "tc_f8": 3, "tc_i8": 4, "tc_f16": 5, "tc_f4": 6}

# The reference host's analytic-model rates, measured on an L4 (main.rs:170-171).
REF_GEMM_RATE = 5.9e14
REF_RARE_RATE = 3.5e9

CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                      ctypes.POINTER(ctypes.c_uint16))


TEXT_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_char), ctypes.c_size_t)
LAYOUTS = {"full": 0, "lower-tri": 1, "upper-tri": 2}


class TchError(RuntimeError):
    pass


class Info(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("L", ctypes.c_int), ("tau", ctypes.c_int), ("kernel", ctypes.c_int),
                ("n_pad", ctypes.c_size_t), ("k_presence", ctypes.c_size_t), ("k_onehot", ctypes.c_size_t),
                ("d_onehot", ctypes.c_size_t), ("n_rare", ctypes.c_size_t), ("rare_sorted", ctypes.c_int),
                ("device_bytes", ctypes.c_size_t), ("k_chunks", ctypes.c_int),
                ("rare_dense", ctypes.c_int), ("sub_rows", ctypes.c_int), ("tile_group", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HostEncoding(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("L", ctypes.c_int), ("tau", ctypes.c_int), ("D", ctypes.c_size_t),
                ("n_pad", ctypes.c_size_t), ("K1", ctypes.c_size_t), ("K2", ctypes.c_size_t),
                ("n_rare", ctypes.c_size_t), ("O", ctypes.POINTER(ctypes.c_uint8)),
                ("P", ctypes.POINTER(ctypes.c_uint8)), ("start", ctypes.POINTER(ctypes.c_uint32)),
                ("js", ctypes.POINTER(ctypes.c_uint32))]


_lib = None


def compile_native(verbose: bool = False):
    """Compile libtch.so and the CLI in-tree (nvcc for sm_103a, g++)."""
    from .build import build as _build

    return _build(verbose)


def lib():
    """The loaded libtch.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise TchError(f"{LIB_PATH} is missing: build it first (build.py / __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        c_int, c_size, c_void, c_char_p, c_double = (ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                                     ctypes.c_char_p, ctypes.c_double)
        P = ctypes.POINTER
        L.tch_device_count.argtypes, L.tch_device_count.restype = [], c_int
        L.tch_free_vram.argtypes, L.tch_free_vram.restype = [c_int], c_size
        L.tch_run.argtypes = [c_int, c_int, c_size, c_void, c_size, c_void, c_size, c_void, c_void, c_size, c_int,
                              CB, c_void, P(c_double), P(c_int), c_char_p, c_int]
        L.tch_run.restype = c_int
        L.tch_version.argtypes, L.tch_version.restype = [], c_int
        L.tch_kernel_name.argtypes, L.tch_kernel_name.restype = [c_int], c_char_p
        L.tch_kernel_available.argtypes, L.tch_kernel_available.restype = [c_int], c_int
        L.tch_set_kernel.argtypes, L.tch_set_kernel.restype = [c_int], c_int
        L.tch_get_kernel.argtypes, L.tch_get_kernel.restype = [], c_int
        L.tch_solver_from_bits.argtypes = [c_int, c_int, c_size, c_void, c_size, c_void, c_size, c_void, c_void,
                                           c_size, c_int, P(c_void), c_char_p, c_int]
        L.tch_solver_from_bits.restype = c_int
        L.tch_solver_info.argtypes, L.tch_solver_info.restype = [c_void, P(Info)], c_int
        L.tch_solver_set_schedule.argtypes, L.tch_solver_set_schedule.restype = [c_void, c_int, c_int], c_int
        L.tch_solver_stripe.argtypes = [c_void, c_int, c_int, c_void, c_size, c_void, c_char_p, c_int]
        L.tch_solver_stripe.restype = c_int
        L.tch_solver_check.argtypes, L.tch_solver_check.restype = [c_void, c_char_p, c_int], c_int
        L.tch_solver_rare_counts.argtypes = [c_void, c_int, c_int, c_void, c_size, c_void, c_char_p, c_int]
        L.tch_solver_rare_counts.restype = c_int
        L.tch_solver_stripe_counts.argtypes = [c_void, c_int, c_int, c_void, c_size, c_void, c_size, c_void,
                                               c_char_p, c_int]
        L.tch_solver_stripe_counts.restype = c_int
        L.tch_solver_run.argtypes = [c_void, c_int, CB, c_void, P(c_double), c_char_p, c_int]
        L.tch_solver_run.restype = c_int
        L.tch_solver_destroy.argtypes, L.tch_solver_destroy.restype = [c_void], None
        L.tch_dense_ranks.argtypes = [c_void, c_int, c_int, c_void, c_void, c_int, c_char_p, c_int]
        L.tch_dense_ranks.restype = c_int
        L.tch_choose_tau.argtypes = [c_void, c_void, c_int, c_int, c_int, c_size, c_double, c_double, c_int, P(c_int),
                                     c_char_p, c_int]
        L.tch_choose_tau.restype = c_int
        L.tch_encode_host.argtypes = [c_void, c_void, c_int, c_int, c_int, c_int, P(HostEncoding), c_char_p, c_int]
        L.tch_encode_host.restype = c_int
        L.tch_host_encoding_free.argtypes, L.tch_host_encoding_free.restype = [P(HostEncoding)], None
        L.tch_solver_from_calls.argtypes = [c_int, c_int, c_int, c_void, c_int, c_int, P(c_void), c_char_p, c_int]
        L.tch_solver_from_calls.restype = c_int
        L.tch_tsv_parse.argtypes = [c_int, c_void, c_size, ctypes.c_char, c_int, c_char_p, P(c_void), c_char_p,
                                    c_int]
        L.tch_tsv_parse.restype = c_int
        L.tch_tsv_shape.argtypes, L.tch_tsv_shape.restype = [c_void, P(c_int), P(c_int)], c_int
        L.tch_tsv_ids.argtypes, L.tch_tsv_ids.restype = [c_void, c_void, c_void], c_int
        L.tch_tsv_filter.argtypes = [c_void, c_double, c_double, c_char_p, c_int]
        L.tch_tsv_filter.restype = c_int
        L.tch_tsv_calls.argtypes, L.tch_tsv_calls.restype = [c_void, c_void], c_int
        L.tch_solver_from_tsv.argtypes = [c_void, c_int, P(c_void), c_char_p, c_int]
        L.tch_solver_from_tsv.restype = c_int
        L.tch_tsv_free.argtypes, L.tch_tsv_free.restype = [c_void], None
        L.tch_run_calls.argtypes = [c_int, c_int, c_int, c_void, c_int, c_int, CB, c_void, P(c_double), P(c_int),
                                    c_char_p, c_int]
        L.tch_run_calls.restype = c_int
        L.tch_set_tau_model.argtypes, L.tch_set_tau_model.restype = [c_double, c_double], c_int
        L.tch_set_max_chunk_bytes.argtypes, L.tch_set_max_chunk_bytes.restype = [c_size], c_int
        L.tch_set_dense_rare_rate.argtypes, L.tch_set_dense_rare_rate.restype = [c_double], c_int
        L.tch_set_rare_term.argtypes, L.tch_set_rare_term.restype = [c_int], c_int
        L.tch_tau_features.argtypes = [c_int, c_int, c_int, c_void, c_int, c_void, c_void, c_void, c_void, c_void,
                                       P(c_int),
                                       c_char_p, c_int]
        L.tch_tau_features.restype = c_int
        L.tch_mlp_init.argtypes, L.tch_mlp_init.restype = [c_void, ctypes.c_uint64], c_int
        L.tch_mlp_train.argtypes = [c_int, c_void, c_void, c_void, c_int, c_int, ctypes.c_float,
                                    P(ctypes.c_float), c_char_p, c_int]
        L.tch_mlp_train.restype = c_int
        L.tch_mlp_predict.argtypes = [c_int, c_void, c_void, c_int, c_void, c_char_p, c_int]
        L.tch_mlp_predict.restype = c_int
        L.tch_mlp_loss_grad.argtypes = [c_int, c_void, c_void, c_void, c_int, P(ctypes.c_float), c_void, c_char_p,
                                        c_int]
        L.tch_mlp_loss_grad.restype = c_int
        L.tch_set_tau_mlp.argtypes, L.tch_set_tau_mlp.restype = [c_void], c_int
        L.tch_db_create.argtypes = [c_int, c_int, c_int, c_void, c_int, P(c_void), c_char_p, c_int]
        L.tch_db_create.restype = c_int
        L.tch_db_destroy.argtypes, L.tch_db_destroy.restype = [c_void], None
        L.tch_db_info.argtypes = [c_void, P(c_int), P(c_int), P(c_int), P(c_size), P(c_size), P(c_int)]
        L.tch_db_info.restype = c_int
        L.tch_db_query_bytes.argtypes, L.tch_db_query_bytes.restype = [c_void, c_int], c_size
        L.tch_host_alloc.argtypes, L.tch_host_alloc.restype = [c_size], c_void
        L.tch_host_free.argtypes, L.tch_host_free.restype = [c_void], None
        L.tch_db_query.argtypes = [c_void, c_int, c_void, c_void, c_void, c_void, c_char_p, c_int]
        L.tch_db_query.restype = c_int
        L.tch_server_create.argtypes = [c_void, c_int, c_size, P(c_void), c_char_p, c_int]
        L.tch_server_create.restype = c_int
        L.tch_server_submit.argtypes = [c_void, c_int, c_void, c_void, c_void]
        L.tch_server_submit.restype = ctypes.c_int64
        L.tch_server_wait.argtypes = [c_void, ctypes.c_int64, P(c_double), P(c_double), c_char_p, c_int]
        L.tch_server_wait.restype = c_int
        L.tch_server_destroy.argtypes, L.tch_server_destroy.restype = [c_void], None
        L.tch_batch_create.argtypes = [c_int, c_int, c_void, c_void, c_void, c_void, P(c_void), c_char_p, c_int]
        L.tch_batch_create.restype = c_int
        L.tch_batch_add.argtypes = [c_void, c_int, c_int, c_void, c_int, c_char_p, c_int]
        L.tch_batch_add.restype = c_int
        L.tch_batch_layout.argtypes, L.tch_batch_layout.restype = [c_void, c_void, c_void], c_int
        L.tch_batch_run.argtypes = [c_void, c_void, c_void, c_char_p, c_int]
        L.tch_batch_run.restype = c_int
        L.tch_batch_check.argtypes, L.tch_batch_check.restype = [c_void, c_char_p, c_int], c_int
        L.tch_batch_tune.argtypes = [c_void, c_void, c_void, c_int, P(c_double), P(c_int), c_char_p, c_int]
        L.tch_batch_tune.restype = c_int
        L.tch_batch_set_schedule.argtypes = [c_void, c_int]
        L.tch_batch_set_schedule.restype = c_int
        L.tch_batch_info.argtypes = [c_void, P(c_int), c_void, P(c_int)]
        L.tch_batch_info.restype = c_int
        L.tch_batch_destroy.argtypes, L.tch_batch_destroy.restype = [c_void], None
        L.tch_solver_from_ranks.argtypes = [c_int, c_int, c_int, c_void, c_int, c_int, P(c_void), c_char_p, c_int]
        L.tch_solver_from_ranks.restype = c_int
        L.tch_solver_write_tsv.argtypes = [c_void, P(c_char_p), c_char_p, c_char_p, c_int, c_int, c_int, TEXT_CB,
                                           c_void, c_char_p, c_int]
        L.tch_solver_write_tsv.restype = c_int
        L.tch_solver_mst.argtypes = [c_void, c_void, c_void, c_void, P(ctypes.c_uint64), c_char_p, c_int]
        L.tch_solver_mst.restype = c_int
        L.tch_solver_clusters.argtypes = [c_void, c_void, c_int, c_void, c_char_p, c_int]
        L.tch_solver_clusters.restype = c_int
        L.tch_solver_neighbors.argtypes = [c_void, c_int, c_void, c_void, c_char_p, c_int]
        L.tch_solver_neighbors.restype = c_int
        L.tch_mst_device.argtypes = [c_void, c_size, c_int, c_void, c_void, c_void, c_void, P(ctypes.c_uint64),
                                     c_char_p, c_int]
        L.tch_mst_device.restype = c_int
        L.tch_neighbors_device.argtypes = [c_void, c_size, c_int, c_int, c_void, c_void, c_void, c_char_p, c_int]
        L.tch_neighbors_device.restype = c_int
        L.tch_mst_clusters.argtypes = [c_int, c_void, c_void, c_void, c_size, c_void, c_int, c_void, c_char_p,
                                       c_int]
        L.tch_mst_clusters.restype = c_int
        _lib = L
    return _lib


def _errbuf():
    return ctypes.create_string_buffer(1024)


def _check(rc, err):
    if rc:
        raise TchError(err.value.decode(errors="replace"))


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def device_count() -> int:
    return lib().tch_device_count()


def free_vram(device: int = 0) -> int:
    return lib().tch_free_vram(device)


def kernel_id(kernel) -> int:
    if isinstance(kernel, str):
        return KERNELS[kernel]
    return int(kernel)


def kernel_name(k: int) -> str:
    return lib().tch_kernel_name(k).decode()


def kernel_available(kernel) -> bool:
    return bool(lib().tch_kernel_available(kernel_id(kernel)))


def set_kernel(kernel) -> None:
    if lib().tch_set_kernel(kernel_id(kernel)):
        raise TchError(f"kernel {kernel!r} not available")


# ---------------------------------------------------------------------------------------
# host encoder (main.rs:134-198, 366-444)
# ---------------------------------------------------------------------------------------

def dense_ranks(calls: np.ndarray, threads: int = 0):
    calls = np.ascontiguousarray(calls, dtype=np.uint64)
    n, L = calls.shape
    x = np.zeros((n, L), dtype=np.uint16)
    nd = np.zeros(L, dtype=np.uint32)
    err = _errbuf()
    _check(lib().tch_dense_ranks(_ptr(calls), n, L, _ptr(x), _ptr(nd), threads, err, len(err)), err)
    return x, nd


def _ranks_args(x, nd):
    """Ranks (n x L u16) and per-locus distinct counts (L u32), as dense_ranks
    returns them; the library checks every rank against its locus's count."""
    x = np.ascontiguousarray(x, dtype=np.uint16)
    nd = np.ascontiguousarray(nd, dtype=np.uint32)
    if x.ndim != 2 or nd.shape != (x.shape[1],):
        raise TchError(f"ranks must be n x L with one distinct count per locus (got {x.shape} and {nd.shape})")
    return x, nd


def choose_tau(x, nd, stripe=512, free_bytes=None, gemm_rate=REF_GEMM_RATE, rare_rate=REF_RARE_RATE,
               verbose=False, device=0) -> int:
    x, nd = _ranks_args(x, nd)
    n, L = x.shape
    if free_bytes is None:
        free_bytes = free_vram(device)
    tau = ctypes.c_int(0)
    err = _errbuf()
    _check(lib().tch_choose_tau(_ptr(x), _ptr(nd), n, L, stripe, free_bytes, gemm_rate, rare_rate, int(verbose),
                                ctypes.byref(tau), err, len(err)), err)
    return tau.value


class Encoding:
    """The reference's tch_run operands, copied out of the C encoder."""

    def __init__(self, h: HostEncoding):
        self.n, self.L, self.tau, self.D = h.n, h.L, h.tau, h.D
        self.n_pad, self.K1, self.K2, self.n_rare = h.n_pad, h.K1, h.K2, h.n_rare
        self.O = np.ctypeslib.as_array(h.O, shape=(max(h.n_pad * h.K1 // 8, 1),))[: h.n_pad * h.K1 // 8].copy()
        self.P = np.ctypeslib.as_array(h.P, shape=(max(h.n_pad * h.K2 // 8, 1),))[: h.n_pad * h.K2 // 8].copy()
        self.start = np.ctypeslib.as_array(h.start, shape=(h.n + 1,)).copy()
        self.js = np.ctypeslib.as_array(h.js, shape=(max(h.n_rare, 1),))[: h.n_rare].copy()


def encode_host(x, nd, tau: int, threads: int = 0) -> Encoding:
    x, nd = _ranks_args(x, nd)
    n, L = x.shape
    h = HostEncoding()
    err = _errbuf()
    _check(lib().tch_encode_host(_ptr(x), _ptr(nd), n, L, tau, threads, ctypes.byref(h), err, len(err)), err)
    try:
        return Encoding(h)
    finally:
        lib().tch_host_encoding_free(ctypes.byref(h))


# ---------------------------------------------------------------------------------------
# the reference ABI: tch_run
# ---------------------------------------------------------------------------------------

class StripeSink:
    """Collects tch_run's stripes into a full n x n u16 matrix (upper triangle
    filled, the rest zero), the way the reference host's on_stripe callback
    copies each row's columns r+1.. (main.rs:204-211)."""

    def __init__(self, n: int, keep_raw: bool = False):
        self.n = n
        self.H = np.zeros((n, n), dtype=np.uint16)
        self.calls = []
        self.keep_raw = keep_raw
        self.raw = []

    def __call__(self, ctx, r0, rows, w, ptr):
        s = np.ctypeslib.as_array(ptr, shape=(rows * w,)).reshape(rows, w)
        self.calls.append((r0, rows, w))
        for r in range(rows):
            self.H[r0 + r, r0 + r + 1:] = s[r, r + 1:]
        if self.keep_raw:
            self.raw.append(s.copy())


def run(enc: Encoding, stripe: int = 512, device: int = 0, sink: StripeSink | None = None):
    """tch_run on an Encoding; returns (H upper-triangle matrix, gpu_secs, rare_on_gpu, sink)."""
    sink = sink or StripeSink(enc.n)
    cb = CB(sink)
    secs = ctypes.c_double(0)
    rare_gpu = ctypes.c_int(-1)
    err = _errbuf()
    rc = lib().tch_run(device, enc.n, enc.n_pad, _ptr(enc.O), enc.K1, _ptr(enc.P), enc.K2, _ptr(enc.start),
                       _ptr(enc.js), enc.n_rare, stripe, cb, None, ctypes.byref(secs), ctypes.byref(rare_gpu), err,
                       len(err))
    _check(rc, err)
    return sink.H, secs.value, rare_gpu.value, sink


def run_calls(calls: np.ndarray, stripe: int = 512, tau: int = 0, device: int = 0, sink: StripeSink | None = None):
    """tch_run_calls: device encoding + stripes; returns (H, gpu_secs, tau_used, sink)."""
    calls = np.ascontiguousarray(calls, dtype=np.uint64)
    n, L = calls.shape
    sink = sink or StripeSink(n)
    cb = CB(sink)
    secs = ctypes.c_double(0)
    tau_used = ctypes.c_int(0)
    err = _errbuf()
    _check(lib().tch_run_calls(device, n, L, _ptr(calls), tau, stripe, cb, None, ctypes.byref(secs),
                               ctypes.byref(tau_used), err, len(err)), err)
    return sink.H, secs.value, tau_used.value, sink


def set_max_chunk_bytes(nbytes: int) -> None:
    """Split solver operands along K into allocations of at most nbytes (0 = one)."""
    lib().tch_set_max_chunk_bytes(int(nbytes))


def set_tau_model(gemm_rate: float, rare_rate: float, dense_rare_rate: float | None = None) -> None:
    if lib().tch_set_tau_model(gemm_rate, rare_rate):
        raise TchError("rates must be positive")
    if dense_rare_rate is not None and lib().tch_set_dense_rare_rate(dense_rare_rate):
        raise TchError("rates must be positive")


# ---------------------------------------------------------------------------------------
# learned tau (no reference counterpart)
# ---------------------------------------------------------------------------------------

TAU_FEATURES = 14
MLP_HIDDEN = 32
MLP_PARAMS = TAU_FEATURES * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN + 1
TAU_MLP_PATH = os.path.join(HERE, "tau_mlp_gb300.f32")


MAX_CANDIDATES = 512


def tau_features(calls: np.ndarray, device: int = 0):
    """Candidates (tau x schedule) whose encoding fits on the device:
    dict(taus, subs, groups, feats [rows x TAU_FEATURES] f32, est: the
    analytic estimate of the candidate's tau in s)."""
    calls = np.ascontiguousarray(calls, dtype=np.uint64)
    n, L = calls.shape
    M = MAX_CANDIDATES
    taus, subs, groups = np.zeros(M, np.int32), np.zeros(M, np.int32), np.zeros(M, np.int32)
    feats = np.zeros((M, TAU_FEATURES), np.float32)
    est = np.zeros(M, np.float64)
    rows = ctypes.c_int(0)
    err = _errbuf()
    _check(lib().tch_tau_features(device, n, L, _ptr(calls), M, _ptr(taus), _ptr(subs), _ptr(groups), _ptr(feats),
                                  _ptr(est), ctypes.byref(rows), err, len(err)), err)
    r = rows.value
    return dict(taus=taus[:r].copy(), subs=subs[:r].copy(), groups=groups[:r].copy(), feats=feats[:r].copy(),
                est=est[:r].copy())


def _mlp_args(w, X, y=None):
    """Weights, samples (m x TAU_FEATURES) and targets (m) as the kernels read
    them, checked against one another before any pointer reaches C."""
    w = np.ascontiguousarray(w, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    if w.size != MLP_PARAMS:
        raise TchError(f"the model has {MLP_PARAMS} parameters (got {w.size})")
    if X.ndim != 2 or X.shape[1] != TAU_FEATURES:
        raise TchError(f"samples must be m x {TAU_FEATURES} (got shape {X.shape})")
    if y is None:
        return w, X
    y = np.ascontiguousarray(y, dtype=np.float32)
    if y.shape != (X.shape[0],):
        raise TchError(f"one target per sample: {X.shape[0]} samples, targets of shape {y.shape}")
    return w, X, y


def mlp_init(seed: int) -> np.ndarray:
    w = np.zeros(MLP_PARAMS, np.float32)
    lib().tch_mlp_init(_ptr(w), seed)
    return w


def mlp_train(w: np.ndarray, X: np.ndarray, y: np.ndarray, steps: int, lr: float, device: int = 0):
    """Adam on the GPU (the library's kernels); returns (new weights, final loss)."""
    w, X, y = _mlp_args(w, X, y)
    w = w.copy()
    loss = ctypes.c_float(0)
    err = _errbuf()
    _check(lib().tch_mlp_train(device, _ptr(w), _ptr(X), _ptr(y), len(y), steps, lr, ctypes.byref(loss), err,
                               len(err)), err)
    return w, loss.value


def mlp_predict(w: np.ndarray, X: np.ndarray, device: int = 0) -> np.ndarray:
    w, X = _mlp_args(w, X)
    out = np.zeros(len(X), np.float32)
    err = _errbuf()
    _check(lib().tch_mlp_predict(device, _ptr(w), _ptr(X), len(X), _ptr(out), err, len(err)), err)
    return out


def mlp_loss_grad(w: np.ndarray, X: np.ndarray, y: np.ndarray, device: int = 0):
    w, X, y = _mlp_args(w, X, y)
    g = np.zeros(MLP_PARAMS, np.float32)
    loss = ctypes.c_float(0)
    err = _errbuf()
    _check(lib().tch_mlp_loss_grad(device, _ptr(w), _ptr(X), _ptr(y), len(y), ctypes.byref(loss), _ptr(g), err,
                                   len(err)), err)
    return loss.value, g


def set_tau_mlp(w: np.ndarray | None) -> None:
    """Model used by tau <= 0 (None: the analytic model)."""
    if w is None:
        lib().tch_set_tau_mlp(None)
        return
    w = np.ascontiguousarray(w, dtype=np.float32)
    if w.size != MLP_PARAMS or lib().tch_set_tau_mlp(_ptr(w)):
        raise TchError("invalid tau model parameters")


def load_tau_mlp(path: str = TAU_MLP_PATH) -> np.ndarray:
    """The trained model shipped with the package (little-endian f32), set
    as the solver's tau model; returns its parameters."""
    w = np.fromfile(path, dtype="<f4")
    set_tau_mlp(w)
    return w


def set_rare_term(dense: bool) -> None:
    """Rare term of solvers built from calls: dense per-stripe counts from the
    rare groups (True, default) or per-row pair lists (False)."""
    lib().tch_set_rare_term(1 if dense else 0)


# ---------------------------------------------------------------------------------------
# solver (device-resident operands)
# ---------------------------------------------------------------------------------------

class Tsv:
    """The allele table parsed on the GPU (tch_tsv_*): `text` is the whole
    input (bytes, UTF-8); the calls stay in device memory."""

    def __init__(self, text: bytes, sep: str = "\t", skip_repl: bool = False, missing: str = "-",
                 device: int = 0):
        self._text = bytes(text)
        self._h = ctypes.c_void_p()
        err = _errbuf()
        buf = ctypes.create_string_buffer(self._text, len(self._text))
        _check(lib().tch_tsv_parse(device, ctypes.cast(buf, ctypes.c_void_p), len(self._text),
                                   sep.encode()[:1], 1 if skip_repl else 0, missing.encode(), ctypes.byref(self._h),
                                   err, len(err)), err)

    def shape(self):
        n, L = ctypes.c_int(), ctypes.c_int()
        lib().tch_tsv_shape(self._h, ctypes.byref(n), ctypes.byref(L))
        return n.value, L.value

    def ids(self) -> list:
        n, _ = self.shape()
        b = np.zeros(max(n, 1), np.uint64)
        e = np.zeros(max(n, 1), np.uint64)
        lib().tch_tsv_ids(self._h, _ptr(b), _ptr(e))
        return [self._text[int(b[i]):int(e[i])].decode() for i in range(n)]

    def filter(self, locus_pct=None, sample_pct=None):
        err = _errbuf()
        _check(lib().tch_tsv_filter(self._h, -1.0 if locus_pct is None else float(locus_pct),
                                    -1.0 if sample_pct is None else float(sample_pct), err, len(err)), err)

    def calls(self) -> np.ndarray:
        n, L = self.shape()
        out = np.zeros((n, L), np.uint64)
        if lib().tch_tsv_calls(self._h, _ptr(out)):
            raise TchError("copying the parsed calls failed")
        return out

    def solver(self, tau: int = 0) -> "Solver":
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_solver_from_tsv(self._h, tau, ctypes.byref(h), err, len(err)), err)
        return Solver(h)

    def close(self):
        if self._h:
            lib().tch_tsv_free(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_encoding(cls, enc: Encoding, kernel="auto", device: int = 0):
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_solver_from_bits(device, enc.n, enc.n_pad, _ptr(enc.O), enc.K1, _ptr(enc.P), enc.K2,
                                          _ptr(enc.start), _ptr(enc.js), enc.n_rare, kernel_id(kernel),
                                          ctypes.byref(h), err, len(err)), err)
        return cls(h)

    @classmethod
    def from_ranks(cls, ranks: np.ndarray, tau: int = 0, kernel="auto", device: int = 0):
        """Device encoding of dense per-locus ranks (n x L u16, 0 = missing)."""
        ranks = np.ascontiguousarray(ranks, dtype=np.uint16)
        n, L = ranks.shape
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_solver_from_ranks(device, n, L, _ptr(ranks), tau, kernel_id(kernel), ctypes.byref(h), err,
                                           len(err)), err)
        return cls(h)

    @classmethod
    def from_calls(cls, calls: np.ndarray, tau: int = 0, kernel="auto", device: int = 0):
        """Device encoding of allele calls (n x L u64, 0 = missing), tau <= 0 automatic."""
        calls = np.ascontiguousarray(calls, dtype=np.uint64)
        n, L = calls.shape
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_solver_from_calls(device, n, L, _ptr(calls), tau, kernel_id(kernel), ctypes.byref(h), err,
                                           len(err)), err)
        return cls(h)

    def info(self) -> dict:
        i = Info()
        lib().tch_solver_info(self._h, ctypes.byref(i))
        return i.as_dict()

    def set_schedule(self, sub_rows: int = 0, tile_group: int = 0):
        """Rows per rare-count + tile-pass pair inside a stripe (0 = the whole
        stripe) and 128-row blocks per raster group of the tile pass (0 = the
        library default)."""
        if lib().tch_solver_set_schedule(self._h, sub_rows, tile_group):
            raise TchError("invalid schedule")

    def stripe(self, r0: int, rows: int, d_out: int, ldo: int, stream: int = 0):
        """One stripe into device memory at address d_out (row stride ldo u16)."""
        err = _errbuf()
        _check(lib().tch_solver_stripe(self._h, r0, rows, ctypes.c_void_p(d_out), ldo,
                                       ctypes.c_void_p(stream) if stream else None, err, len(err)), err)

    def rare_counts(self, r0: int, rows: int, d_R: int, ldr: int, stream: int = 0):
        """Dense rare counts of a stripe into device memory at d_R (row stride
        ldr u16, ldr >= up(n - r0, 256)); dense-rare solvers only."""
        err = _errbuf()
        _check(lib().tch_solver_rare_counts(self._h, r0, rows, ctypes.c_void_p(d_R), ldr,
                                            ctypes.c_void_p(stream) if stream else None, err, len(err)), err)

    def stripe_counts(self, r0: int, rows: int, d_out: int, ldo: int, d_R: int, ldr: int, stream: int = 0):
        """The stripe's tile pass with the rare term read from d_R."""
        err = _errbuf()
        _check(lib().tch_solver_stripe_counts(self._h, r0, rows, ctypes.c_void_p(d_out), ldo, ctypes.c_void_p(d_R),
                                              ldr, ctypes.c_void_p(stream) if stream else None, err, len(err)), err)

    def check(self):
        err = _errbuf()
        _check(lib().tch_solver_check(self._h, err, len(err)), err)

    def write_tsv(self, ids, osep: str = "\t", index_name: str = "cgmlst-hamming-gpu", layout: str = "full",
                  cap: int = 0, block_rows: int = 0, sink=None) -> str | None:
        """The reference's TSV matrix, formatted on the GPU; returns the text,
        or hands each chunk (bytes) to sink(chunk) when given."""
        parts = []

        def take(ctx, p, n):
            chunk = ctypes.string_at(p, n)
            if sink is not None:
                sink(chunk)
            else:
                parts.append(chunk)

        cb = TEXT_CB(take)
        arr = (ctypes.c_char_p * max(len(ids), 1))(*[i.encode() for i in ids])
        err = _errbuf()
        _check(lib().tch_solver_write_tsv(self._h, arr, osep.encode(), index_name.encode(), LAYOUTS[layout], cap,
                                          block_rows, cb, None, err, len(err)), err)
        return None if sink is not None else b"".join(parts).decode()

    def mst(self):
        """The minimum spanning tree on the device (edges ordered by distance,
        smaller index, larger index): (u, v, w) of its n - 1 edges, u < v."""
        m = max(self.info()["n"] - 1, 0)
        u, v, w = np.zeros(m, np.uint32), np.zeros(m, np.uint32), np.zeros(m, np.uint16)
        total = ctypes.c_uint64(0)
        err = _errbuf()
        _check(lib().tch_solver_mst(self._h, _ptr(u), _ptr(v), _ptr(w), ctypes.byref(total), err, len(err)), err)
        return u, v, w

    def clusters(self, thresholds) -> np.ndarray:
        """Single-linkage cluster labels (the smallest index of each profile's
        cluster), one row per threshold."""
        thr = np.ascontiguousarray(thresholds, dtype=np.uint32)
        n = self.info()["n"]
        labels = np.zeros((len(thr), n), np.uint32)
        err = _errbuf()
        _check(lib().tch_solver_clusters(self._h, _ptr(thr), len(thr), _ptr(labels), err, len(err)), err)
        return labels

    def neighbors(self, k: int):
        """Every profile's k nearest profiles by (distance, index): (idx, dist), n x k."""
        n = self.info()["n"]
        idx, dist = np.zeros((n, max(k, 0)), np.uint32), np.zeros((n, max(k, 0)), np.uint16)
        err = _errbuf()
        _check(lib().tch_solver_neighbors(self._h, k, _ptr(idx), _ptr(dist), err, len(err)), err)
        return idx, dist

    def run(self, stripe: int = 512, sink: StripeSink | None = None):
        sink = sink or StripeSink(self.info()["n"])
        cb = CB(sink)
        secs = ctypes.c_double(0)
        err = _errbuf()
        _check(lib().tch_solver_run(self._h, stripe, cb, None, ctypes.byref(secs), err, len(err)), err)
        return sink.H, secs.value

    def close(self):
        if self._h:
            lib().tch_solver_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------
# consumers of a matrix already in device memory
# ---------------------------------------------------------------------------------------

def mst_device(d_H: int, ld: int, n: int, stream: int = 0):
    """Minimum spanning tree of a full symmetric n x n u16 matrix at device
    address d_H (row stride ld): (u, v, w)."""
    m = max(n - 1, 0)
    u, v, w = np.zeros(m, np.uint32), np.zeros(m, np.uint32), np.zeros(m, np.uint16)
    total = ctypes.c_uint64(0)
    err = _errbuf()
    _check(lib().tch_mst_device(ctypes.c_void_p(d_H), ld, n, ctypes.c_void_p(stream) if stream else None, _ptr(u),
                                _ptr(v), _ptr(w), ctypes.byref(total), err, len(err)), err)
    return u, v, w


def neighbors_device(d_H: int, ld: int, n: int, k: int, stream: int = 0):
    """The k nearest profiles of every row of a full matrix in device memory."""
    idx, dist = np.zeros((n, max(k, 0)), np.uint32), np.zeros((n, max(k, 0)), np.uint16)
    err = _errbuf()
    _check(lib().tch_neighbors_device(ctypes.c_void_p(d_H), ld, n, k, ctypes.c_void_p(stream) if stream else None,
                                      _ptr(idx), _ptr(dist), err, len(err)), err)
    return idx, dist


def mst_clusters(n: int, u, v, w, thresholds) -> np.ndarray:
    """Single-linkage labels at each threshold from a spanning tree's edges (host)."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    w = np.ascontiguousarray(w, dtype=np.uint16)
    thr = np.ascontiguousarray(thresholds, dtype=np.uint32)
    if not (len(u) == len(v) == len(w)):
        raise TchError(f"u, v and w must have one entry per edge (got {len(u)}, {len(v)}, {len(w)})")
    labels = np.zeros((len(thr), n), np.uint32)
    err = _errbuf()
    _check(lib().tch_mst_clusters(n, _ptr(u), _ptr(v), _ptr(w), len(u), _ptr(thr), len(thr), _ptr(labels), err,
                                  len(err)), err)
    return labels


# ---------------------------------------------------------------------------------------
# serving: resident database, query batches, continuous batching
# ---------------------------------------------------------------------------------------

def pinned_empty(shape, dtype=np.uint16) -> np.ndarray:
    """A numpy array in page-locked host memory (freed with the array)."""
    import weakref

    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    p = lib().tch_host_alloc(nbytes)
    if not p:
        raise TchError(f"could not page-lock {nbytes} bytes")
    buf = (ctypes.c_char * max(nbytes, 1)).from_address(p)
    a = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
    weakref.finalize(buf, lib().tch_host_free, p)
    return a


def _result_buffer(buf, shape, name: str, zero: bool = False) -> np.ndarray:
    """A caller's u16 result buffer checked against the call's shape (the
    library writes shape[0] x shape[1] cells through its pointer), or a new one."""
    if buf is None:
        return np.zeros(shape, np.uint16) if zero else np.empty(shape, np.uint16)
    if buf.shape != shape or buf.dtype != np.uint16 or not buf.flags.c_contiguous:
        raise TchError(f"{name} must be a C-contiguous {shape[0]} x {shape[1]} uint16 array "
                       f"(got {buf.dtype} {buf.shape})")
    return buf


class Database:
    """A profile database resident on the device (tch_db)."""

    def __init__(self, calls: np.ndarray, tau: int = 0, device: int = 0):
        calls = np.ascontiguousarray(calls, dtype=np.uint64)
        self.n, self.L = calls.shape
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_db_create(device, self.n, self.L, _ptr(calls), tau, ctypes.byref(h), err, len(err)), err)
        self._h = h

    def info(self) -> dict:
        n, L, tau, kc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        d, b = ctypes.c_size_t(), ctypes.c_size_t()
        lib().tch_db_info(self._h, ctypes.byref(n), ctypes.byref(L), ctypes.byref(tau), ctypes.byref(d),
                          ctypes.byref(b), ctypes.byref(kc))
        return dict(n=n.value, L=L.value, tau=tau.value, d_onehot=d.value, device_bytes=b.value, k_chunks=kc.value)

    def query_bytes(self, m: int) -> int:
        return lib().tch_db_query_bytes(self._h, m)

    def query(self, q: np.ndarray, want_qq: bool = True, stream: int = 0, out: np.ndarray | None = None,
              out_qq: np.ndarray | None = None):
        """(q x database distances [m x n], q x q upper triangle [m x m] or None);
        out / out_qq: caller buffers (page-locked ones arrive fastest)."""
        q = np.ascontiguousarray(q, dtype=np.uint64)
        m = q.shape[0]
        if q.shape[1] != self.L:
            raise TchError(f"queries have {q.shape[1]} loci, the database {self.L}")
        qdb = _result_buffer(out, (m, self.n), "out")  # every cell is written
        qq = _result_buffer(out_qq, (m, m), "out_qq", zero=True) if want_qq else None
        err = _errbuf()
        _check(lib().tch_db_query(self._h, m, _ptr(q), _ptr(qdb), _ptr(qq) if want_qq else None,
                                  ctypes.c_void_p(stream) if stream else None, err, len(err)), err)
        return qdb, qq

    def close(self):
        if self._h:
            lib().tch_db_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Continuous batching over a Database (tch_server): submit() returns at
    once; wait() blocks until that request's results are in its buffers."""

    def __init__(self, db: Database, slots: int = 4, budget: int = 0):
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_server_create(db._h, slots, budget, ctypes.byref(h), err, len(err)), err)
        self._h = h
        self.db = db
        self._live = {}

    def submit(self, q: np.ndarray, want_qq: bool = True, out: np.ndarray | None = None,
               out_qq: np.ndarray | None = None) -> int:
        """out / out_qq: caller buffers for the results (m x n and m x m u16;
        page-locked ones, see pinned_empty, arrive fastest)."""
        q = np.ascontiguousarray(q, dtype=np.uint64)
        m = q.shape[0]
        if q.ndim != 2 or q.shape[1] != self.db.L:
            raise TchError(f"queries must be m x {self.db.L} (the database's loci), got shape {q.shape}")
        qdb = _result_buffer(out, (m, self.db.n), "out")  # every cell is written
        qq = _result_buffer(out_qq, (m, m), "out_qq", zero=True) if want_qq else None
        rid = lib().tch_server_submit(self._h, m, _ptr(q), _ptr(qdb), _ptr(qq) if want_qq else None)
        if rid < 0:
            raise TchError("request rejected")
        self._live[rid] = (q, qdb, qq)  # buffers live until wait()
        return rid

    def wait(self, rid: int):
        """(qdb, qq, queued seconds, latency seconds)."""
        qs, ls = ctypes.c_double(), ctypes.c_double()
        err = _errbuf()
        rc = lib().tch_server_wait(self._h, rid, ctypes.byref(qs), ctypes.byref(ls), err, len(err))
        q, qdb, qq = self._live.pop(rid, (None, None, None))  # each id is waited for once
        _check(rc, err)
        return qdb, qq, qs.value, ls.value

    def close(self):
        if self._h:
            lib().tch_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---------------------------------------------------------------------------------------
# batched solves under a CUDA graph
# ---------------------------------------------------------------------------------------

class Batch:
    """Many profile sets solved together (tch_batch): every set's upper
    triangle into one device buffer, launches captured as one CUDA graph."""

    def __init__(self, sets=(), taus=None, device: int = 0):
        h = ctypes.c_void_p()
        err = _errbuf()
        _check(lib().tch_batch_create(device, 0, None, None, None, None, ctypes.byref(h), err, len(err)), err)
        self._h = h
        self.shapes = []
        for k, A in enumerate(sets):
            self.add(A, 0 if taus is None else taus[k])

    def add(self, calls: np.ndarray, tau: int = 0):
        calls = np.ascontiguousarray(calls, dtype=np.uint64)
        n, L = calls.shape
        err = _errbuf()
        _check(lib().tch_batch_add(self._h, n, L, _ptr(calls), tau, err, len(err)), err)
        self.shapes.append((n, L))

    def layout(self):
        c = len(self.shapes)
        off = np.zeros(c + 1, np.uint64)
        ld = np.zeros(max(c, 1), np.uint64)
        lib().tch_batch_layout(self._h, _ptr(off), _ptr(ld))
        return off.astype(np.int64), ld[:c].astype(np.int64)

    def run(self, d_out: int, stream: int = 0):
        err = _errbuf()
        _check(lib().tch_batch_run(self._h, ctypes.c_void_p(d_out), ctypes.c_void_p(stream) if stream else None,
                                   err, len(err)), err)

    def check(self):
        err = _errbuf()
        _check(lib().tch_batch_check(self._h, err, len(err)), err)

    def tune(self, d_out: int, stream: int = 0, reps: int = 3) -> dict:
        ms = ctypes.c_double()
        nb = ctypes.c_int()
        err = _errbuf()
        _check(lib().tch_batch_tune(self._h, ctypes.c_void_p(d_out), ctypes.c_void_p(stream) if stream else None,
                                    reps, ctypes.byref(ms), ctypes.byref(nb), err, len(err)), err)
        return dict(ms=ms.value, branches=nb.value)

    def set_schedule(self, branches: int):
        if lib().tch_batch_set_schedule(self._h, branches):
            raise TchError("invalid schedule")

    def info(self) -> dict:
        c = ctypes.c_int()
        taus = np.zeros(max(len(self.shapes), 1), np.int32)
        nb = ctypes.c_int()
        lib().tch_batch_info(self._h, ctypes.byref(c), _ptr(taus), ctypes.byref(nb))
        return dict(count=c.value, taus=taus[:c.value].tolist(), branches=nb.value)

    def close(self):
        if self._h:
            lib().tch_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---------------------------------------------------------------------------------------
# ranks files (tensorcore/to_ranks.py: int32 n, int32 L, then n x L u16, 0 = missing)
# ---------------------------------------------------------------------------------------

def write_ranks(path: str, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x, dtype="<u2")
    with open(path, "wb") as f:
        np.array(x.shape, dtype="<i4").tofile(f)
        x.tofile(f)


def read_ranks(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        n, L = np.fromfile(f, dtype="<i4", count=2)
        x = np.fromfile(f, dtype="<u2", count=int(n) * int(L))
    if x.size != int(n) * int(L):
        raise TchError(f"{path}: truncated ranks file")
    return x.reshape(int(n), int(L))
