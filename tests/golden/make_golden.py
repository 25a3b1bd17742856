"""Generates the golden fixtures that pin the oracle (run from the repository root):

    python tests/golden/make_golden.py

Every fixture comes from a restatement that is independent of oracle/oracle.cpp:

* picks.json      -- the reference's initial picks (kmeans.cpp:876-883) drawn from glibc's own
                     srand(42)/rand() through ctypes, with the reference's binary_search over the
                     unsorted pick list restated as a lower_bound in Python.
* shuffle.json    -- the reference's shuffle (kmeans.cpp:554-557), std::shuffle with
                     std::default_random_engine(0), restated in Python from libstdc++'s published
                     algorithm: minstd_rand0 (x <- 16807 x mod 2^31-1, seed 0 -> state 1),
                     uniform_int_distribution by rejection + division, and std::shuffle's
                     two-swaps-per-draw path when (2^31-3) / n >= n.
* distance.npz    -- the reference's known-answer procedure of test/python/distance.py.in:32-79:
                     np.random.seed(42) uniform data, labels = argmin(||a||^2 + ||b||^2 - 2 a.b),
                     here evaluated in FP64 with numpy (smaller m than the reference's 899946).
* lloyd_small.npz -- a Lloyd run restated in numpy (FP64 distances, FP64 means rounded to FP32,
                     SSE against the new centers, reference initialisation).
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

OUT = os.path.dirname(os.path.abspath(__file__))


# ---------------- glibc picks ----------------
def glibc_picks(m: int, k: int) -> list[int]:
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(42)

    def found(v, x):  # std::binary_search == lower_bound + !(x < *it), on an unsorted vector
        lo, hi = 0, len(v)
        while lo < hi:
            mid = (lo + hi) // 2
            if v[mid] < x:
                lo = mid + 1
            else:
                hi = mid
        return lo < len(v) and not (x < v[lo])

    pts: list[int] = []
    for _ in range(k):
        idx = libc.rand() % m
        while found(pts, idx):
            idx = libc.rand() % m
        pts.append(idx)
    return pts


# ---------------- libstdc++ std::shuffle with minstd_rand0(0) ----------------
class MinstdRand0:
    A, M = 16807, 2147483647

    def __init__(self, seed: int = 0):
        s = seed % self.M
        self.x = 1 if s == 0 else s

    def __call__(self) -> int:
        self.x = (self.A * self.x) % self.M
        return self.x

    min, max = 1, 2147483646


def uniform_int(g: MinstdRand0, a: int, b: int) -> int:
    urngrange = g.max - g.min
    urange = b - a
    if urngrange > urange:
        uerange = urange + 1
        scaling = urngrange // uerange
        past = uerange * scaling
        while True:
            ret = g() - g.min
            if ret < past:
                break
        return a + ret // scaling
    if urngrange == urange:
        return a + g() - g.min
    raise NotImplementedError("range wider than the generator")


def gen_two_uniform_ints(b0: int, b1: int, g: MinstdRand0):
    x = uniform_int(g, 0, b0 * b1 - 1)
    return x // b1, x % b1


def std_shuffle(n: int) -> list[int]:
    v = list(range(n))
    if n == 0:
        return v
    g = MinstdRand0(0)
    urngrange = g.max - g.min
    urange = n
    if urngrange // urange >= urange:
        i = 1
        if urange % 2 == 0:
            j = uniform_int(g, 0, 1)
            v[i], v[j] = v[j], v[i]
            i += 1
        while i != n:
            swap_range = i + 1
            p1, p2 = gen_two_uniform_ints(swap_range, swap_range + 1, g)
            v[i], v[p1] = v[p1], v[i]
            i += 1
            v[i], v[p2] = v[p2], v[i]
            i += 1
        return v
    for i in range(1, n):
        j = uniform_int(g, 0, i)
        v[i], v[j] = v[j], v[i]
    return v


# ---------------- numpy Lloyd (reference semantics) ----------------
def numpy_lloyd(X: np.ndarray, init: np.ndarray, iters: int):
    C = init.astype(np.float32).copy()
    X64 = X.astype(np.float64)
    sse_hist, labels = [], None
    for _ in range(iters):
        d2 = ((X64[:, None, :] - C.astype(np.float64)[None, :, :]) ** 2).sum(-1)
        labels = np.argmin(d2, axis=1)  # first minimum = lowest index on ties
        k = C.shape[0]
        newC = np.full_like(C, np.nan)
        for j in range(k):
            mem = X64[labels == j]
            if len(mem):
                newC[j] = (mem.sum(0) / len(mem)).astype(np.float32)
        diff = X64 - newC.astype(np.float64)[labels]
        sse_hist.append(float((diff ** 2).sum()))
        C = newC
    return C, labels.astype(np.int32), np.array(sse_hist)


def main():
    picks = {f"{m}_{k}": glibc_picks(m, k) for (m, k) in
             [(50, 40), (100, 64), (1000, 64), (100000, 64), (4000000, 1024), (7, 7)]}
    with open(os.path.join(OUT, "picks.json"), "w") as f:
        json.dump(picks, f)

    sh = {}
    for n in (1, 2, 3, 10, 11, 1000, 46340, 46341, 100000):
        p = std_shuffle(n)
        sh[str(n)] = p if n <= 1000 else {"head": p[:64], "tail": p[-64:],
                                         "sum_i_p": int(sum(i * x for i, x in enumerate(p)) % (1 << 61))}
    with open(os.path.join(OUT, "shuffle.json"), "w") as f:
        json.dump(sh, f)

    # distance.py.in:32-79 procedure (seed 42, uniform data, FP64 arg-min of the expansion)
    np.random.seed(seed=42)
    m, n, k = 1024, 129, 256
    a = np.asarray(np.random.rand(m, n), np.float32)
    b = np.asarray(np.random.rand(n, k), np.float32)
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    anorm = (a64 ** 2).sum(1)
    bnorm = (b64 ** 2).sum(0)
    lab = np.argmin(anorm[:, None] + bnorm[None, :] - 2.0 * (a64 @ b64), axis=1).astype(np.int32)
    np.savez_compressed(os.path.join(OUT, "distance.npz"), a=a, b=b, labels=lab)

    # small Lloyd run with the reference initialisation
    rng = np.random.default_rng(7)
    N, D, K, IT = 3000, 8, 12, 10
    means = rng.uniform(-10, 10, size=(K, D))
    comp = rng.integers(0, K, size=N)
    X = (rng.standard_normal((N, D)) + means[comp]).astype(np.float32)
    perm = std_shuffle(N)
    pk = glibc_picks(N, K)
    init = X[[perm[p] for p in pk]]
    Cf, lab, sse = numpy_lloyd(X, init, IT)
    np.savez_compressed(os.path.join(OUT, "lloyd_small.npz"), X=X, init=init, centers=Cf,
                        labels=lab, sse=sse)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
