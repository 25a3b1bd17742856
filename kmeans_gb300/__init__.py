"""kmeans_gb300: GB300-native (sm_103a) K-means Lloyd hot path.

Python mirror of the reference's interfaces (PaulMullowney/kmeans):

* ``computeKmeansF`` / ``computeKmeansD`` -- the reference driver entry points
  (main/cpp/kmeans.hpp:102-132) with the same arguments, return codes and D x K result layout;
* ``ClosestCentersF``, ``rowTransformMinimumF/D``, ``ClusterCentersF/D``, ``CompactnessF/D``,
  ``rowNormalizeF/D``, ``colNormalizeF/D``, ``MatMatMultF/D`` -- the per-kernel entry points
  (main/cuda/KmeansCudaKernels.h:198-474) on device pointers;
* ``lloyd`` / ``Handle`` -- the extension: explicit initial centers, labels, per-iteration SSE,
  precision tier, resident data.

Everything calls the in-tree C-ABI library ``libkmeans_gb300.so`` through ctypes. There is no
CPU fallback: if the library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkmeans_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "kmeans_gb300.h")

KMEANS_SUCCESS = 0
KMEANS_ERROR_BUILDDATA = 1
KMEANS_ERROR_INITIALIZE = 2
KMEANS_ERROR_CLOSEST_CENTERS = 3
KMEANS_ERROR_CLUSTER_CENTERS = 4
KMEANS_ERROR_COMPACTNESS = 5
KMEANS_ERROR_RESET = 7
KMEANS_ERROR_COMPUTE = 8
KMEANS_ERROR_GET_CENTERS = 9
KMEANS_NONCONVERGENCE = 13
ASSIGN_FP32 = 0
ASSIGN_BF16 = 1
ASSIGN_BF16X3 = 2
ASSIGN_FP8 = 3
ASSIGN_AUTO = 4  # kmgb_lloyd_batched_f32: per dimension from the tuned cost table
EMPTY_NAN = 0
EMPTY_KEEP = 1
INIT_REFERENCE = 0
INIT_KMEANSPP = 1

ERROR_STRINGS = {
    1: "error in building the data",
    2: "error in the initialization",
    3: "error in computing the closest centers",
    4: "error in computing the cluster centers",
    5: "error in computing the compactness",
    6: "error in transpose",
    7: "error in reset",
    8: "error in compute",
    9: "error in copying the data back to the host",
    10: "error in the tiling",
    11: "error in copy tile",
    12: "error in constructing the minibatch",
    13: "algorithm did not converge",
}


class KmeansError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"kmeans_gb300 error {code}: {ERROR_STRINGS.get(code, 'no error')}"
                         + (f" ({msg})" if msg else ""))
        self.code = code


class kmgb_options(C.Structure):
    _fields_ = [("assign_tier", C.c_int), ("certify", C.c_int), ("empty_policy", C.c_int),
                ("max_iters", C.c_int), ("criterion", C.c_double),
                ("mini_batch_fraction", C.c_float), ("stream_tile_rows", C.c_int),
                ("init_algorithm", C.c_int), ("num_retries", C.c_int),
                ("seed", C.c_ulonglong), ("router", C.c_int), ("router_groups", C.c_int),
                ("router_retrain", C.c_int), ("router_hidden", C.c_int)]


class kmgb_problem(C.Structure):
    _fields_ = [("X", C.c_void_p), ("n", C.c_longlong), ("d", C.c_int), ("k", C.c_int),
                ("init", C.c_void_p), ("centers", C.c_void_p), ("labels", C.c_void_p),
                ("sse", C.c_void_p), ("iterations", C.c_int), ("status", C.c_int),
                ("reserved", C.c_longlong * 4)]


class kmgb_router_stats(C.Structure):
    _fields_ = [("trainings", C.c_longlong), ("train_ms", C.c_double), ("group_ms", C.c_double),
                ("last_loss", C.c_double), ("last_accuracy", C.c_double),
                ("groups_nonempty", C.c_int), ("components", C.c_int),
                ("max_group", C.c_int), ("max_component", C.c_int),
                ("scan_chunks", C.c_ulonglong),
                ("routed", C.c_ulonglong), ("flagged", C.c_ulonglong),
                ("certified", C.c_ulonglong), ("fallback", C.c_ulonglong),
                ("routed_iterations", C.c_longlong), ("device_bytes", C.c_longlong),
                ("stage_ms", C.c_double * 7), ("reserved", C.c_longlong * 4)]

    STAGES = ("permute_centers", "separation", "inference", "sort", "group_scan",
              "near_ties", "certificate")

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in ("reserved", "stage_ms")}
        d["stage_ms"] = dict(zip(self.STAGES, list(self.stage_ms)))
        return d


class kmgb_stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("reranked", C.c_ulonglong),
                ("reranked_fp64", C.c_ulonglong), ("empty_clusters", C.c_longlong),
                ("ms_total", C.c_double), ("reserved", C.c_longlong * 8)]


_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the CUDA library for sm_103a (nvcc) if needed."""
    return _build.build(force=force)


def lib():
    """Load libkmeans_gb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run kmeans_gb300.build() (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        P, i32, i64, f32, f64 = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_double
        b = C.c_bool
        sig = {
            "kmeansGetErrorString": (C.c_char_p, [i32]),
            "computeKmeansF": (i32, [P, i32, i32, i32, f32, i32, i32, i32, i32, i32, P, f32]),
            "computeKmeansD": (i32, [P, i32, i32, i32, f64, i32, i32, i32, i32, i32, P, f64]),
            "ClosestCentersF": (i32, [i32, i32, i32, P, i32, P, P, P, P, i32, P, P, P]),
            "ClosestCentersD": (i32, [i32, i32, i32, P, i32, P, P, P, P, i32, P, P, P]),
            "rowTransformMinimumF": (i32, [i32, i32, i32, P, P, P, P]),
            "rowTransformMinimumD": (i32, [i32, i32, i32, P, P, P, P]),
            "ClusterCentersF": (i32, [i32, i32, i32, i32, b, P, P, P, P, P, P]),
            "ClusterCentersD": (i32, [i32, i32, i32, i32, b, P, P, P, P, P, P]),
            "ClusterCentersF_noalloc": (i32, [i32, i32, i32, i32, b, P, P, P, P, P, P]),
            "CompactnessF": (i32, [i32, i32, b, i32, i32, P, P, P, P]),
            "CompactnessD": (i32, [i32, i32, b, i32, i32, P, P, P, P]),
            "MatMatMultF": (i32, [i32, i32, P, i32, P, P]),
            "MatMatMultD": (i32, [i32, i32, P, i32, P, P]),
            "rowNormalizeF": (i32, [i32, i32, i32, P, P]),
            "rowNormalizeD": (i32, [i32, i32, i32, P, P]),
            "colNormalizeF": (i32, [i32, i32, P, P]),
            "colNormalizeD": (i32, [i32, i32, P, P]),
            "kmgb_default_options": (None, [P]),
            "kmgb_lloyd_f32": (i32, [P, i64, i32, i32, P, P, P, P, P, P]),
            "kmgb_create": (i32, [P, i64, i32, i32, P]),
            "kmgb_set_data": (i32, [P, P, i32]),
            "kmgb_set_centers": (i32, [P, P, i32]),
            "kmgb_run": (i32, [P, i32, f64]),
            "kmgb_synchronize": (i32, [P]),
            "kmgb_get_centers": (i32, [P, P, i32]),
            "kmgb_get_labels": (i32, [P, P, i32]),
            "kmgb_get_sse": (i32, [P, P, i32]),
            "kmgb_get_stats": (i32, [P, P]),
            "kmgb_stream": (P, [P]),
            "kmgb_destroy": (i32, [P]),
            "kmgb_last_error": (C.c_char_p, []),
            "kmgb_set_profiling": (i32, [P, i32]),
            "kmgb_get_phase_ms": (i32, [P, P, P]),
            "kmgb_launch_count": (i64, []),
            "kmgb_release_cached_memory": (i32, []),
            "kmgb_sum_piece": (i32, []),
            "kmgb_reference_init": (i32, [P, i32, i32, i32, P, P, P]),
            "kmgb_tc_accumulators": (i32, [P, i64, i32, P, i32, i32, P]),
            "kmgb_version": (C.c_char_p, []),
            "kmgb_kmeanspp_f32": (i32, [P, i64, i32, i32, C.c_ulonglong, P, P]),
            "kmgb_kmeanspp_f64": (i32, [P, i64, i32, i32, C.c_ulonglong, P, P]),
            "kmgb_init_kmeanspp": (i32, [P, C.c_ulonglong, P]),
            "kmgb_lloyd_batched_f32": (i32, [P, i32, P, P]),
            "kmgb_get_router_stats": (i32, [P, P]),
            "kmgb_shard_partials": (i32, [P, P, P, P, i32]),
            "kmgb_shard_update": (i32, [P, P, P, P, P, i32]),
            "kmgb_router_mlp_train": (i32, [P, i32, i32, P, i32, i32, P, i32, i32, f32, P, P]),
            "kmgb_debug_fail_nth": (None, [i32, i64]),
            "kmgb_debug_withhold_stage": (None, [i64, C.c_ulonglong]),
            "kmgb_debug_pool_used_bytes": (i64, []),
            "kmgb_debug_audit": (i32, [P, i64, i32, i64, P, i32, i64, P, i32, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def launch_count() -> int:
    return int(lib().kmgb_launch_count())


def release_cached_memory() -> None:
    """Return the device memory that destroyed handles left in the library's pool (handles
    reuse it otherwise; KMGB_POOL=0 returns it at every destroy)."""
    if lib().kmgb_release_cached_memory() != 0:
        raise KmeansError(KMEANS_ERROR_BUILDDATA, last_error())


FAULT_ALLOC, FAULT_COPY, FAULT_LAUNCH = 1, 2, 3


def debug_fail_nth(kind: int, nth: int) -> None:
    """Test hook: the nth later event of `kind` (FAULT_ALLOC / FAULT_COPY / FAULT_LAUNCH) fails
    once, as the CUDA call would have failed; nth <= 0 disarms it."""
    lib().kmgb_debug_fail_nth(int(kind), int(nth))


def debug_withhold_stage(stage: int, wait_cycles: int = 0) -> None:
    """Test hook: FP32-tier assignment launches withhold their TMA loads from pipeline step
    `stage` on (0 disarms) and bound every wait by `wait_cycles` SM cycles."""
    lib().kmgb_debug_withhold_stage(int(stage), int(wait_cycles))


def router_mlp_train(X: np.ndarray, y: np.ndarray, params: np.ndarray, hidden: int, groups: int,
                     batch: int, steps: int, lr: float = 1e-3):
    """The router's network alone (kmgb_router_mlp_train): steps == 0 returns (loss, gradients)
    of one forward/backward pass over the first batch; otherwise trains `params` in place with
    Adam and returns (loss of the last batch, None)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.int32)
    assert params.dtype == np.float32 and params.flags.c_contiguous
    rows, d = X.shape
    loss = C.c_double()
    grads = np.empty_like(params) if steps == 0 else None
    rc = lib().kmgb_router_mlp_train(_ptr(X), rows, d, _ptr(y), hidden, groups, _ptr(params),
                                     batch, steps, lr, C.byref(loss), _ptr(grads))
    if rc:
        raise KmeansError(rc, last_error())
    return loss.value, grads


def debug_audit(X, C, labels, rows: int = 64):
    """Test hook: one audit of `rows` sampled rows (device tensors X n x d, C k x d float32,
    labels int32) against the FP64 arg-min. Returns (rows audited, violations, 1 + the last
    violating row or 0)."""
    n, d = X.shape
    k = C.shape[0]
    out = np.zeros(3, dtype=np.uint64)
    rc = lib().kmgb_debug_audit(X.data_ptr(), n, d, X.stride(0), C.data_ptr(), k, C.stride(0),
                                labels.data_ptr(), rows, _ptr(out))
    if rc:
        raise KmeansError(rc, last_error())
    return int(out[0]), int(out[1]), int(out[2])


def debug_pool_used_bytes() -> int:
    """Bytes of the current device's library pool handed out and not yet given back."""
    return int(lib().kmgb_debug_pool_used_bytes())


def last_error() -> str:
    return lib().kmgb_last_error().decode()


def default_options(**kw) -> kmgb_options:
    o = kmgb_options()
    lib().kmgb_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _ptr(a) -> Optional[int]:
    """Address of a numpy array (host) or a torch tensor (device or host)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())


# ----------------------------------------------------------------------------------------
# reference driver API
# ----------------------------------------------------------------------------------------

def computeKmeansF(data: np.ndarray, m: int, n: int, k: int, criterion: float, maxIters: int,
                   numRetries: int, initAlgorithm: int, doFullSGEMM: int, matrixFormat: int,
                   result: np.ndarray, miniBatchFraction: float = 1.0) -> int:
    """Same arguments and return code as the reference (kmeans.hpp:102-107); `result` (n*k
    float32, K fastest) receives the final centers."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    assert result.dtype == np.float32 and result.flags.c_contiguous and result.size >= n * k
    return int(lib().computeKmeansF(_ptr(data), m, n, k, criterion, maxIters, numRetries,
                                    initAlgorithm, doFullSGEMM, matrixFormat, _ptr(result),
                                    miniBatchFraction))


def computeKmeansD(data: np.ndarray, m: int, n: int, k: int, criterion: float, maxIters: int,
                   numRetries: int, initAlgorithm: int, doFullSGEMM: int, matrixFormat: int,
                   result: np.ndarray, miniBatchFraction: float = 1.0) -> int:
    data = np.ascontiguousarray(data, dtype=np.float64)
    assert result.dtype == np.float64 and result.flags.c_contiguous and result.size >= n * k
    return int(lib().computeKmeansD(_ptr(data), m, n, k, criterion, maxIters, numRetries,
                                    initAlgorithm, doFullSGEMM, matrixFormat, _ptr(result),
                                    miniBatchFraction))


def reference_init(data: np.ndarray, k: int):
    """The reference's initial centers (host only): returns (centers k x d, perm, picks)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    m, d = data.shape
    cen = np.empty((k, d), np.float32)
    perm = np.empty(m, np.int32)
    picks = np.empty(k, np.int32)
    rc = lib().kmgb_reference_init(_ptr(data), m, d, k, _ptr(cen), _ptr(perm), _ptr(picks))
    if rc:
        raise KmeansError(rc, last_error())
    return cen, perm, picks


def kmeanspp(X, k: int, seed: int = 0):
    """k-means++ initial centers through kmgb_kmeanspp_f32/_f64. X: numpy (host) or torch (device)
    n x d, float32 or float64. Returns (centers k x d numpy, picks int32[k])."""
    dbl = str(getattr(X, "dtype", "")).endswith("float64")
    if isinstance(X, np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float64 if dbl else np.float32)
    n, d = X.shape
    cen = np.empty((k, d), np.float64 if dbl else np.float32)
    picks = np.empty(k, np.int32)
    fn = lib().kmgb_kmeanspp_f64 if dbl else lib().kmgb_kmeanspp_f32
    rc = fn(_ptr(X), n, d, k, seed, _ptr(cen), _ptr(picks))
    if rc:
        raise KmeansError(rc, last_error())
    return cen, picks


def tc_accumulators(X: np.ndarray, C: np.ndarray, split) -> np.ndarray:
    """Raw tcgen05 accumulators x.c_j - ||c_j||^2/2 (n x k) of the BF16 (split 0), split BF16
    (1) or two-product split kernel for BF16-valued X (2)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    C = np.ascontiguousarray(C, dtype=np.float32)
    n, d = X.shape
    k = C.shape[0]
    out = np.empty((n, k), np.float32)
    rc = lib().kmgb_tc_accumulators(_ptr(X), n, d, _ptr(C), k, int(split), _ptr(out))
    if rc:
        raise KmeansError(rc, last_error())
    return out


def kmeansGetErrorString(err: int) -> str:
    return lib().kmeansGetErrorString(err).decode()


# ----------------------------------------------------------------------------------------
# per-kernel API (device tensors; torch is used only as device memory)
# ----------------------------------------------------------------------------------------

def ClosestCentersF(m0, nRowsA, nColsA, A, nColsB, B, Bpadded, normRowsOfA_squared,
                    normColsOfB_squared, nColsC, Cpart, Cindices, CindicesFinal) -> int:
    return int(lib().ClosestCentersF(m0, nRowsA, nColsA, _ptr(A), nColsB, _ptr(B), _ptr(Bpadded),
                                     _ptr(normRowsOfA_squared), _ptr(normColsOfB_squared),
                                     nColsC, _ptr(Cpart), _ptr(Cindices), _ptr(CindicesFinal)))


def ClosestCentersD(m0, nRowsA, nColsA, A, nColsB, B, Bpadded, normRowsOfA_squared,
                    normColsOfB_squared, nColsC, Cpart, Cindices, CindicesFinal) -> int:
    return int(lib().ClosestCentersD(m0, nRowsA, nColsA, _ptr(A), nColsB, _ptr(B), _ptr(Bpadded),
                                     _ptr(normRowsOfA_squared), _ptr(normColsOfB_squared),
                                     nColsC, _ptr(Cpart), _ptr(Cindices), _ptr(CindicesFinal)))


def rowTransformMinimumF(m0, m, n, normA, normB, inp, out) -> int:
    return int(lib().rowTransformMinimumF(m0, m, n, _ptr(normA), _ptr(normB), _ptr(inp), _ptr(out)))


def rowTransformMinimumD(m0, m, n, normA, normB, inp, out) -> int:
    return int(lib().rowTransformMinimumD(m0, m, n, _ptr(normA), _ptr(normB), _ptr(inp), _ptr(out)))


def ClusterCentersF(m0, m, n, k, lastTile, data, indices, centers_large, counts_large, centers,
                    counts) -> int:
    return int(lib().ClusterCentersF(m0, m, n, k, bool(lastTile), _ptr(data), _ptr(indices),
                                     _ptr(centers_large), _ptr(counts_large), _ptr(centers),
                                     _ptr(counts)))


def ClusterCentersD(m0, m, n, k, lastTile, data, indices, centers_large, counts_large, centers,
                    counts) -> int:
    return int(lib().ClusterCentersD(m0, m, n, k, bool(lastTile), _ptr(data), _ptr(indices),
                                     _ptr(centers_large), _ptr(counts_large), _ptr(centers),
                                     _ptr(counts)))


def ClusterCentersF_noalloc(m0, m, n, k, lastTile, data, indices, centers_large, counts_large,
                            centers, counts) -> int:
    """ClusterCentersF without any device allocation (working memory in the library's static
    8 MiB device array); for callers that cannot allocate."""
    return int(lib().ClusterCentersF_noalloc(m0, m, n, k, bool(lastTile), _ptr(data),
                                             _ptr(indices), _ptr(centers_large),
                                             _ptr(counts_large), _ptr(centers), _ptr(counts)))


def CompactnessF(m0, m, lastTile, n, k, data, indices, centers, compactness) -> int:
    return int(lib().CompactnessF(m0, m, bool(lastTile), n, k, _ptr(data), _ptr(indices),
                                  _ptr(centers), _ptr(compactness)))


def CompactnessD(m0, m, lastTile, n, k, data, indices, centers, compactness) -> int:
    return int(lib().CompactnessD(m0, m, bool(lastTile), n, k, _ptr(data), _ptr(indices),
                                  _ptr(centers), _ptr(compactness)))


def MatMatMultF(nRowsA, nColsA, A, nColsB, B, C) -> int:
    return int(lib().MatMatMultF(nRowsA, nColsA, _ptr(A), nColsB, _ptr(B), _ptr(C)))


def MatMatMultD(nRowsA, nColsA, A, nColsB, B, C) -> int:
    return int(lib().MatMatMultD(nRowsA, nColsA, _ptr(A), nColsB, _ptr(B), _ptr(C)))


def rowNormalizeF(m0, m, n, inp, out) -> int:
    return int(lib().rowNormalizeF(m0, m, n, _ptr(inp), _ptr(out)))


def rowNormalizeD(m0, m, n, inp, out) -> int:
    return int(lib().rowNormalizeD(m0, m, n, _ptr(inp), _ptr(out)))


def colNormalizeF(m, n, inp, out) -> int:
    return int(lib().colNormalizeF(m, n, _ptr(inp), _ptr(out)))


def colNormalizeD(m, n, inp, out) -> int:
    return int(lib().colNormalizeD(m, n, _ptr(inp), _ptr(out)))


# ----------------------------------------------------------------------------------------
# extension
# ----------------------------------------------------------------------------------------

@dataclass
class LloydResult:
    status: int
    centers: np.ndarray
    labels: np.ndarray
    sse: np.ndarray
    iterations: int
    reranked: int
    reranked_fp64: int
    empty_clusters: int
    ms_total: float
    audited: int = 0           # rows checked against the FP64 arg-min (sampled per iteration)
    audit_violations: int = 0  # of those, labels farther than the nearest center


def lloyd(X, k: int, init=None, max_iters: int = 20, criterion: float = -1.0,
          assign_tier: int = ASSIGN_FP32, certify: bool = True, empty_policy: int = EMPTY_NAN,
          mini_batch_fraction: float = 1.0, stream_tile_rows: int = 0,
          init_algorithm: int = INIT_REFERENCE, num_retries: int = 1,
          seed: int = 0, router: bool = False, router_groups: int = 0,
          router_retrain: int = 0) -> LloydResult:
    """One-shot Lloyd run through kmgb_lloyd_f32. X: numpy (host) or torch (device) n x d
    float32; init: k x d float32, or None for init_algorithm (the reference initialisation, or
    k-means++ with num_retries seeded runs keeping the lowest final SSE). stream_tile_rows > 0
    keeps a host X in host memory and streams it through the GPU in tiles of that many rows."""
    if isinstance(X, np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
    n, d = X.shape
    if init is not None and isinstance(init, np.ndarray):
        init = np.ascontiguousarray(init, dtype=np.float32)
    opt = default_options(assign_tier=assign_tier, certify=int(certify),
                          empty_policy=empty_policy, max_iters=max_iters, criterion=criterion,
                          mini_batch_fraction=mini_batch_fraction,
                          stream_tile_rows=stream_tile_rows, init_algorithm=init_algorithm,
                          num_retries=num_retries, seed=seed, router=int(router),
                          router_groups=router_groups, router_retrain=router_retrain)
    cen = np.empty((k, d), dtype=np.float32)
    lab = np.empty(n, dtype=np.int32)
    sse = np.zeros(max(max_iters, 1), dtype=np.float64)
    st = kmgb_stats()
    rc = lib().kmgb_lloyd_f32(_ptr(X), n, d, k, _ptr(init), C.byref(opt), _ptr(cen), _ptr(lab),
                              _ptr(sse), C.byref(st))
    if rc not in (KMEANS_SUCCESS, KMEANS_NONCONVERGENCE):
        raise KmeansError(rc, last_error())
    return LloydResult(rc, cen, lab, sse[:st.iterations], st.iterations, st.reranked,
                       st.reranked_fp64, st.empty_clusters, st.ms_total, int(st.reserved[6]),
                       int(st.reserved[7]))


def lloyd_batched(problems, max_iters: int = 20, criterion: float = -1.0,
                  empty_policy: int = EMPTY_NAN, certify: bool = True,
                  assign_tier: int = ASSIGN_FP32):
    """Many independent Lloyd runs in one kmgb_lloyd_batched_f32 call. problems: sequence of
    (X, k) or (X, k, init) with X numpy (host) or a contiguous torch tensor (device), n x d
    float32 (init k x d, or None for the reference initialisation). Returns (list of
    LloydResult, kmgb_stats)."""
    arr = (kmgb_problem * len(problems))()
    keep = []
    outs = []
    for i, p in enumerate(problems):
        X, k = p[0], int(p[1])
        init = p[2] if len(p) > 2 else None
        if isinstance(X, np.ndarray):
            X = np.ascontiguousarray(X, dtype=np.float32)
        if init is not None:
            init = np.ascontiguousarray(init, dtype=np.float32)
        n, d = X.shape
        cen = np.empty((k, d), np.float32)
        lab = np.empty(n, np.int32)
        sse = np.zeros(max(max_iters, 1), np.float64)
        keep += [X, init]
        outs.append((cen, lab, sse))
        arr[i].X, arr[i].n, arr[i].d, arr[i].k = _ptr(X), n, d, k
        arr[i].init = _ptr(init)
        arr[i].centers, arr[i].labels, arr[i].sse = _ptr(cen), _ptr(lab), _ptr(sse)
    opt = default_options(max_iters=max_iters, criterion=criterion, empty_policy=empty_policy,
                          certify=int(certify), assign_tier=assign_tier)
    st = kmgb_stats()
    rc = lib().kmgb_lloyd_batched_f32(arr, len(problems), C.byref(opt), C.byref(st))
    if rc:
        raise KmeansError(rc, last_error())
    res = []
    for i, (cen, lab, sse) in enumerate(outs):
        it = arr[i].iterations
        res.append(LloydResult(arr[i].status, cen, lab, sse[:it], it, 0, 0, 0, 0.0))
    return res, st


class Handle:
    """Resident data set + centers; iterations run on the handle's own CUDA stream."""

    def __init__(self, n: int, d: int, k: int, **opts):
        self._h = C.c_void_p()
        o = default_options(**opts)
        rc = lib().kmgb_create(C.byref(self._h), n, d, k, C.byref(o))
        if rc:
            raise KmeansError(rc, last_error())
        self.n, self.d, self.k = n, d, k

    def _chk(self, rc):
        if rc not in (KMEANS_SUCCESS,):
            raise KmeansError(rc, last_error())

    def set_data(self, X, on_device: bool):
        self._chk(lib().kmgb_set_data(self._h, _ptr(X), int(on_device)))

    def set_centers(self, Cn=None, on_device: bool = False):
        self._chk(lib().kmgb_set_centers(self._h, _ptr(Cn), int(on_device)))

    def init_kmeanspp(self, seed: int = 0) -> np.ndarray:
        """k-means++ centers from the resident data; returns the picked rows."""
        picks = np.empty(self.k, np.int32)
        self._chk(lib().kmgb_init_kmeanspp(self._h, seed, _ptr(picks)))
        return picks

    def run(self, iters: int, criterion: float = -1.0):
        self._chk(lib().kmgb_run(self._h, iters, criterion))

    def synchronize(self):
        self._chk(lib().kmgb_synchronize(self._h))

    @property
    def stream(self) -> int:
        return int(lib().kmgb_stream(self._h) or 0)

    def centers(self) -> np.ndarray:
        out = np.empty((self.k, self.d), dtype=np.float32)
        self._chk(lib().kmgb_get_centers(self._h, _ptr(out), 0))
        return out

    def labels(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.int32)
        self._chk(lib().kmgb_get_labels(self._h, _ptr(out), 0))
        return out

    def sse(self, count: int) -> np.ndarray:
        out = np.zeros(max(count, 1), dtype=np.float64)
        c = lib().kmgb_get_sse(self._h, _ptr(out), count)
        return out[:c]

    def stats(self) -> kmgb_stats:
        st = kmgb_stats()
        self._chk(lib().kmgb_get_stats(self._h, C.byref(st)))
        return st

    def shard_partials(self, S=None, counts=None, Q=None):
        """Assign the handle's rows to its centers; canonical FP64 sums per cluster. With torch
        device tensors given (S k*d float64, counts k int32, Q k float64) they are filled on the
        device; otherwise host numpy arrays are returned."""
        on_dev = S is not None and not isinstance(S, np.ndarray)
        if S is None:
            S = np.empty(self.k * self.d, np.float64)
            counts = np.empty(self.k, np.int32)
            Q = np.empty(self.k, np.float64)
        self._chk(lib().kmgb_shard_partials(self._h, _ptr(S), _ptr(counts), _ptr(Q),
                                            int(on_dev)))
        return S, counts, Q

    def shard_update(self, S, counts, Q) -> float:
        """New centers from the summed partials of all shards; returns the iteration's SSE."""
        on_dev = not isinstance(S, np.ndarray)
        sse = C.c_double()
        self._chk(lib().kmgb_shard_update(self._h, _ptr(S), _ptr(counts), _ptr(Q),
                                          C.byref(sse), int(on_dev)))
        return sse.value

    def router_stats(self) -> kmgb_router_stats:
        st = kmgb_router_stats()
        self._chk(lib().kmgb_get_router_stats(self._h, C.byref(st)))
        return st

    def set_profiling(self, on: bool = True):
        self._chk(lib().kmgb_set_profiling(self._h, int(on)))

    def phase_ms(self):
        """(ms[prep, assign, rerank, update] summed, iterations covered)."""
        ms = (C.c_double * 4)()
        it = C.c_int(0)
        self._chk(lib().kmgb_get_phase_ms(self._h, ms, C.byref(it)))
        return list(ms), it.value

    def close(self):
        if self._h:
            lib().kmgb_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
