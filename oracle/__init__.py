"""CPU oracle for the Lloyd hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference-arm leg may
import this package, and only as the checker (or as the timed CPU stand-in for the
reference, which has no CPU path of its own). The product library never imports it.

`build()` compiles oracle.cpp with g++ (OpenMP, -ffp-contract=off so FP64 results are the
same on x86-64 and aarch64) into oracle/liboracle.so; `lib()` loads it with ctypes
signatures; the numpy helpers below wrap the calls.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.cpp")
_SO = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

# Canonical FP64 center-sum piece size; must equal the product's (checked by a test).
PIECE = 128


def build(force: bool = False) -> str:
    """Compile the oracle shared library if it is missing or older than its source."""
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(_SRC)):
        return _SO
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           _SRC, "-o", _SO + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(_SO + ".tmp", _SO)
    return _SO


_REF = os.path.join(_HERE, "_ref")
_REF_CUBIN = os.path.join(_REF, "closest_centers.cubin")
_REF_CC_CUBIN = os.path.join(_REF, "cluster_centers.cubin")
_REF_CP_CUBIN = os.path.join(_REF, "compactness.cubin")
_REF_SO = os.path.join(_REF, "libref_kernels.so")
_REF_LOADER_SRC = os.path.join(_HERE, "ref_kernels.cpp")
_REF_SHIM = os.path.join(_HERE, "ref_shfl_shim.h")


def _reference_cuda_dir() -> str:
    """main/cuda of the reference checkout: $KMGB_REFERENCE_DIR when set, else a checkout named
    `reference` beside this repository. Present only where the reference's sources are (the
    development machine), never on the GPU host, which uses the prebuilt cubins in oracle/_ref."""
    root = os.environ.get("KMGB_REFERENCE_DIR") or os.path.join(
        os.path.dirname(os.path.dirname(_HERE)), "reference")
    return os.path.join(root, "main", "cuda")


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isdir(os.path.join(cand, "include")):
            return cand
    return "/usr/local/cuda"


def build_ref() -> bool:
    """Recipe for oracle/_ref (git-ignored, test infrastructure).

    1. Where the reference's sources are present, compile its main/cuda/ClosestCenters.cu,
       ClusterCenters.cu and Compactness.cu, as they lie, into cubins for sm_103a with
       ref_shfl_shim.h force-included (the reference's pre-Volta shuffles). Device code does not
       depend on the host architecture, so the cubins built here run on the Arm GPU host.
    2. Wherever a CUDA toolkit is present, compile ref_kernels.cpp, the loader that plays the
       reference's host side (host code built from the reference's sources, which exist only in
       the x86 development container, could not run on the Arm GPU host).

    Returns True when both the cubin and the loader exist.
    """
    os.makedirs(_REF, exist_ok=True)
    ref_dir = _reference_cuda_dir()
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    for name, out in (("ClosestCenters.cu", _REF_CUBIN), ("ClusterCenters.cu", _REF_CC_CUBIN),
                      ("Compactness.cu", _REF_CP_CUBIN)):
        src = os.path.join(ref_dir, name)
        if os.path.exists(src) and not os.path.exists(out):
            subprocess.check_call([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                                   "-O3", "-w", "-include", _REF_SHIM, "-I", ref_dir,
                                   src, "-o", out + ".tmp"])
            os.replace(out + ".tmp", out)
    if os.path.isdir(os.path.join(cuda, "include")) and (
            not os.path.exists(_REF_SO)
            or os.path.getmtime(_REF_SO) < os.path.getmtime(_REF_LOADER_SRC)):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I",
                               os.path.join(cuda, "include"), _REF_LOADER_SRC, "-o",
                               _REF_SO + ".tmp", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                               "-Wl,-rpath," + os.path.join(cuda, "lib64")])
        os.replace(_REF_SO + ".tmp", _REF_SO)
    return os.path.exists(_REF_CUBIN) and os.path.exists(_REF_SO)


_ref_lib = None


def ref_kernels():
    """The reference's assignment kernels (cubin + loader), or None when oracle/_ref is absent.
    When its center and compactness cubins are present too, `has_update` is True and
    refk_cluster_centers_f / refk_compactness_f are bound."""
    global _ref_lib
    with _lock:
        if _ref_lib is not None:
            return _ref_lib
        if not (os.path.exists(_REF_CUBIN) and os.path.exists(_REF_SO)):
            return None
        L = C.CDLL(_REF_SO)
        P = C.c_void_p
        L.refk_load.argtypes = [C.c_char_p]
        L.refk_load.restype = C.c_int
        L.refk_last_error.restype = C.c_char_p
        L.refk_closest_centers_f.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int, P, P, C.c_int,
                                             P, P, P]
        L.refk_closest_centers_f.restype = C.c_int
        found = L.refk_load(_REF_CUBIN.encode())
        if found != 17:
            raise RuntimeError(f"reference cubin: found {found} of 17 kernels "
                               f"({L.refk_last_error().decode()})")
        L.has_update = False
        if os.path.exists(_REF_CC_CUBIN) and os.path.exists(_REF_CP_CUBIN):
            L.refk_load_update.argtypes = [C.c_char_p, C.c_char_p]
            L.refk_load_update.restype = C.c_int
            L.refk_cluster_centers_f.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P]
            L.refk_cluster_centers_f.restype = C.c_int
            L.refk_compactness_f.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P]
            L.refk_compactness_f.restype = C.c_int
            got = L.refk_load_update(_REF_CC_CUBIN.encode(), _REF_CP_CUBIN.encode())
            if got != 4:
                raise RuntimeError(f"reference update cubins: found {got} of 4 kernels "
                                   f"({L.refk_last_error().decode()})")
            L.has_update = True
        _ref_lib = L
        return L


def lib():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        L = C.CDLL(_SO)
        P = C.c_void_p
        i32, i64, f32, f64 = C.c_int, C.c_longlong, C.c_float, C.c_double
        L.orc_shuffle_perm.argtypes = [i32, P]
        L.orc_init_picks.argtypes = [i32, i32, P]
        L.orc_init_picks.restype = i32
        L.orc_reference_init.argtypes = [P, i32, i32, i32, P]
        L.orc_reference_init.restype = i32
        L.orc_assign.argtypes = [P, i64, i32, P, i32, P, P]
        L.orc_update.argtypes = [P, i64, i32, P, i32, i32, P, i32, P, P, P]
        L.orc_sse.argtypes = [P, i64, i32, P, P]
        L.orc_sse.restype = f64
        L.orc_lloyd.argtypes = [P, i64, i32, i32, P, i32, f64, f32, i32, i32, P, P, P, P]
        L.orc_lloyd.restype = i32
        L.orc_assign_d.argtypes = [P, i64, i32, P, i32, P, P]
        L.orc_update_d.argtypes = [P, i64, i32, P, i32, i32, P, i32, P, P, P]
        L.orc_sse_d.argtypes = [P, i64, i32, P, P]
        L.orc_sse_d.restype = f64
        L.orc_lloyd_d.argtypes = [P, i64, i32, i32, P, i32, f64, f32, i32, i32, P, P, P, P]
        L.orc_lloyd_d.restype = i32
        L.orc_lloyd_tiled.argtypes = [P, i64, i32, i32, P, i32, f64, i32, i32, i64, P, P, P, P]
        L.orc_lloyd_tiled.restype = i32
        L.orc_closest_expansion.argtypes = [P, i32, i32, P, i32, P, P]
        L.orc_closest_expansion_d.argtypes = [P, i32, i32, P, i32, P, P]
        L.orc_row_transform_min_f.argtypes = [i32, i32, i32, P, P, P, P]
        L.orc_row_transform_min_d.argtypes = [i32, i32, i32, P, P, P, P]
        L.orc_port_lloyd.argtypes = [P, i64, i32, i32, P, i32, i32, P, P, P]
        L.orc_port_lloyd.restype = i32
        L.orc_num_threads.restype = i32
        L.orc_kmeanspp.argtypes = [P, i64, i32, i32, C.c_ulonglong, P, P]
        L.orc_kmeanspp.restype = i32
        L.orc_kmeanspp_d.argtypes = [P, i64, i32, i32, C.c_ulonglong, P, P]
        L.orc_kmeanspp_d.restype = i32
        _lib = L
        return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def shuffle_perm(m: int) -> np.ndarray:
    out = np.empty(m, dtype=np.int32)
    lib().orc_shuffle_perm(m, _p(out))
    return out


def init_picks(m: int, k: int) -> np.ndarray:
    out = np.empty(k, dtype=np.int32)
    rc = lib().orc_init_picks(m, k, _p(out))
    if rc:
        raise ValueError(f"init picks failed ({rc})")
    return out


def reference_init(X: np.ndarray, k: int) -> np.ndarray:
    X = _f32(X)
    m, d = X.shape
    out = np.empty((k, d), dtype=np.float32)
    rc = lib().orc_reference_init(_p(X), m, d, k, _p(out))
    if rc:
        raise ValueError(f"reference init failed ({rc})")
    return out


def assign(X: np.ndarray, Cn: np.ndarray, with_dist: bool = False):
    X, Cn = _f32(X), _f32(Cn)
    m, d = X.shape
    k = Cn.shape[0]
    lab = np.empty(m, dtype=np.int32)
    dist = np.empty(m, dtype=np.float64) if with_dist else None
    lib().orc_assign(_p(X), m, d, _p(Cn), k, _p(lab), _p(dist) if with_dist else None)
    return (lab, dist) if with_dist else lab


def update(X, labels, k, old_centers=None, empty_policy=0, piece=PIECE):
    X = _f32(X)
    m, d = X.shape
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    oc = _f32(old_centers) if old_centers is not None else None
    newc = np.empty((k, d), dtype=np.float32)
    cnt = np.empty(k, dtype=np.int64)
    sums = np.empty((k, d), dtype=np.float64)
    lib().orc_update(_p(X), m, d, _p(labels), k, piece, _p(oc) if oc is not None else None,
                     empty_policy, _p(newc), _p(cnt), _p(sums))
    return newc, cnt, sums


def sse(X, labels, centers) -> float:
    X, centers = _f32(X), _f32(centers)
    m, d = X.shape
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    return float(lib().orc_sse(_p(X), m, d, _p(labels), _p(centers)))


def lloyd_tiled(X, init, max_iters, tile_rows, criterion=-1.0, empty_policy=0, piece=PIECE):
    """Full-batch loop with the host-streamed tiles' update order (tiles of `tile_rows` rows).
    Returns (status, centers KxD, labels, sse[iters], iters)."""
    X, init = _f32(X), _f32(init)
    m, d = X.shape
    k = init.shape[0]
    cen = np.empty((k, d), dtype=np.float32)
    lab = np.empty(m, dtype=np.int32)
    sse_ = np.zeros(max(max_iters, 1), dtype=np.float64)
    its = C.c_int(0)
    st = lib().orc_lloyd_tiled(_p(X), m, d, k, _p(init), max_iters, float(criterion),
                               empty_policy, piece, int(tile_rows), _p(cen), _p(lab), _p(sse_),
                               C.byref(its))
    return st, cen, lab, sse_[:its.value], its.value


def lloyd(X, init, max_iters, criterion=-1.0, mb_fraction=1.0, empty_policy=0, piece=PIECE):
    """Returns (status, centers KxD, labels, sse[iters], iters)."""
    X, init = _f32(X), _f32(init)
    m, d = X.shape
    k = init.shape[0]
    cen = np.empty((k, d), dtype=np.float32)
    lab = np.empty(m, dtype=np.int32)
    sse_ = np.zeros(max(max_iters, 1), dtype=np.float64)
    its = C.c_int(0)
    st = lib().orc_lloyd(_p(X), m, d, k, _p(init), max_iters, float(criterion),
                         float(mb_fraction), empty_policy, piece, _p(cen), _p(lab), _p(sse_),
                         C.byref(its))
    return st, cen, lab, sse_[:its.value], its.value


def lloyd_d(X, init, max_iters, criterion=-1.0, mb_fraction=1.0, empty_policy=0, piece=PIECE):
    """FP64-data Lloyd loop. Returns (status, centers KxD float64, labels, sse, iters)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    init = np.ascontiguousarray(init, dtype=np.float64)
    m, d = X.shape
    k = init.shape[0]
    cen = np.empty((k, d), dtype=np.float64)
    lab = np.empty(m, dtype=np.int32)
    sse_ = np.zeros(max(max_iters, 1), dtype=np.float64)
    its = C.c_int(0)
    st = lib().orc_lloyd_d(_p(X), m, d, k, _p(init), max_iters, float(criterion),
                           float(mb_fraction), empty_policy, piece, _p(cen), _p(lab), _p(sse_),
                           C.byref(its))
    return st, cen, lab, sse_[:its.value], its.value


def closest_expansion(A, B, nb):
    """FP64 arg-min_j nb_j - 2 A_i.B_j (B is d x k), the per-kernel ClosestCenters semantics."""
    f64 = A.dtype == np.float64
    dt = np.float64 if f64 else np.float32
    A = np.ascontiguousarray(A, dtype=dt)
    B = np.ascontiguousarray(B, dtype=dt)
    nb = np.ascontiguousarray(nb, dtype=dt)
    m, d = A.shape
    k = B.shape[1]
    out = np.empty(m, dtype=np.int32)
    fn = lib().orc_closest_expansion_d if f64 else lib().orc_closest_expansion
    fn(_p(A), m, d, _p(B), k, _p(nb), _p(out))
    return out


def row_transform_min_f(m0, normA, normB, G, out_len):
    normA, normB, G = _f32(normA), _f32(normB), _f32(G)
    m, n = G.shape
    out = np.zeros(out_len, dtype=np.int32)
    lib().orc_row_transform_min_f(m0, m, n, _p(normA), _p(normB), _p(G), _p(out))
    return out


def row_transform_min_d(m0, normA, normB, G, out_len):
    normA = np.ascontiguousarray(normA, dtype=np.float64)
    normB = np.ascontiguousarray(normB, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64)
    m, n = G.shape
    out = np.zeros(out_len, dtype=np.int32)
    lib().orc_row_transform_min_d(m0, m, n, _p(normA), _p(normB), _p(G), _p(out))
    return out


def port_lloyd(X, init, iters, piece=PIECE):
    """FP32 port of the loop (CPU baseline). Returns (centers, labels, sse[iters])."""
    X, init = _f32(X), _f32(init)
    m, d = X.shape
    k = init.shape[0]
    cen = np.empty((k, d), dtype=np.float32)
    lab = np.empty(m, dtype=np.int32)
    s = np.zeros(max(iters, 1), dtype=np.float64)
    lib().orc_port_lloyd(_p(X), m, d, k, _p(init), iters, piece, _p(cen), _p(lab), _p(s))
    return cen, lab, s[:iters]


def kmeanspp(X: np.ndarray, k: int, seed: int = 0):
    """k-means++ picks (k row indices) and centers (k x d) of X (float32 or float64)."""
    dbl = X.dtype == np.float64
    X = np.ascontiguousarray(X, dtype=np.float64 if dbl else np.float32)
    n, d = X.shape
    picks = np.empty(k, np.int32)
    cen = np.empty((k, d), X.dtype)
    fn = lib().orc_kmeanspp_d if dbl else lib().orc_kmeanspp
    rc = fn(_p(X), n, d, k, seed, _p(picks), _p(cen))
    if rc != 0:
        raise ValueError("kmeanspp: needs 0 < k <= n")
    return picks, cen


def num_threads() -> int:
    return int(lib().orc_num_threads())
