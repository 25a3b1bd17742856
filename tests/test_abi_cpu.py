"""CPU checks of the C-ABI library: it builds for sm_103a, loads, and exports every entry point
that include/kmeans_gb300.h declares; host-only calls behave as the reference's."""
import ctypes
import os
import re
import subprocess

import pytest


def declared_symbols(km):
    src = open(km.HEADER_PATH).read()
    return sorted(set(re.findall(r"KMGB_EXPORT\s+[\w\s\*]+?\b(\w+)\(", src)))


def test_library_exports_every_declared_symbol(km):
    km.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", km.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    decl = declared_symbols(km)
    assert len(decl) >= 30
    missing = [s for s in decl if s not in exported]
    assert not missing, missing
    lib = km.lib()
    for s in decl:
        assert getattr(lib, s) is not None


def test_reference_entry_points_present(km):
    names = ["computeKmeansF", "computeKmeansD", "kmeansGetErrorString", "ClosestCentersF",
             "ClosestCentersD", "rowTransformMinimumF", "rowTransformMinimumD",
             "ClusterCentersF", "ClusterCentersD", "CompactnessF", "CompactnessD",
             "rowNormalizeF", "rowNormalizeD", "colNormalizeF", "colNormalizeD",
             "MatMatMultF", "MatMatMultD"]
    decl = declared_symbols(km)
    for n in names:
        assert n in decl


def test_error_strings_match_reference(km):
    for code, s in km.ERROR_STRINGS.items():
        assert km.kmeansGetErrorString(code) == s
    assert km.kmeansGetErrorString(0) == "no error"


def test_piece_size_matches_oracle(km, orc):
    assert km.lib().kmgb_sum_piece() == orc.PIECE


def test_default_options(km):
    o = km.default_options()
    assert (o.assign_tier, o.certify, o.empty_policy, o.max_iters) == (0, 1, 0, 20)
    assert o.criterion < 0 and o.mini_batch_fraction == 1.0


def test_mat_mat_mult_rejects_negative_sizes_without_gpu(km):
    # ERROR_MATMATMULT (1) before any device call
    assert km.MatMatMultF(-1, 2, None, 2, None, None) == 1
    assert km.MatMatMultD(2, -2, None, 2, None, None) == 1


def test_invalid_arguments_rejected_without_gpu(km):
    import numpy as np
    res = np.zeros(16, np.float32)
    data = np.zeros((2, 2), np.float32)
    # argument validation happens before any device call
    assert km.computeKmeansF(data, 2, 2, 0, -1.0, 1, 1, 0, 0, 0, res, 1.0) == 1
    assert km.computeKmeansF(data, 2, 2, 3, -1.0, 1, 1, 0, 0, 0, res, 1.0) == 2
    assert km.computeKmeansF(data, 2, 2, 1, -1.0, 1, 1, 0, 3, 0, res, 1.0) == 1


def test_reference_init_matches_oracle_and_fixtures(km, orc):
    import json
    import numpy as np
    from kmeans_gb300.synthetic import mixture_numpy
    X, _, _ = mixture_numpy(50_000, 24, 40, seed=7)
    cen, perm, picks = km.reference_init(X, 40)
    assert np.array_equal(perm, orc.shuffle_perm(50_000))
    assert np.array_equal(picks, orc.init_picks(50_000, 40))
    assert np.array_equal(cen, orc.reference_init(X, 40))
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "picks.json")))
    for key, v in gold.items():
        m, k = map(int, key.split("_"))
        Z = np.zeros((m, 1), np.float32) if m <= 100_000 else None
        if Z is None:
            continue
        _, _, p = km.reference_init(Z, k)
        assert p.tolist() == v, key


def test_header_compiles_as_c_and_cpp_with_reference_default(km, tmp_path):
    """A C++ caller of the reference passes 11 arguments to computeKmeansF/D (miniBatchFraction
    defaults to 1.0 in kmeans.hpp:102-132); the header keeps that default for C++ and stays valid
    C."""
    inc = os.path.dirname(km.HEADER_PATH)
    cpp = tmp_path / "caller.cpp"
    cpp.write_text('#include "kmeans_gb300.h"\n'
                   "int f(const float* d, float* r, const double* dd, double* rd) {\n"
                   "  return computeKmeansF(d, 4, 2, 2, -1.0f, 1, 1, 0, 0, 0, r) +\n"
                   "         computeKmeansD(dd, 4, 2, 2, -1.0, 1, 1, 0, 0, 0, rd);\n}\n")
    c = tmp_path / "caller.c"
    c.write_text('#include "kmeans_gb300.h"\n'
                 "int f(const float* d, float* r) {\n"
                 "  return computeKmeansF(d, 4, 2, 2, -1.0f, 1, 1, 0, 0, 0, r, 1.0f);\n}\n")
    subprocess.run(["g++", "-std=c++17", "-c", "-I", inc, str(cpp), "-o", str(tmp_path / "a.o")],
                   check=True)
    subprocess.run(["gcc", "-std=c99", "-c", "-I", inc, str(c), "-o", str(tmp_path / "b.o")],
                   check=True)


def test_debug_hooks_exported_and_inert_without_gpu(km):
    lib = km.lib()
    # arming and disarming touches no device
    km.debug_fail_nth(km.FAULT_LAUNCH, 3)
    km.debug_fail_nth(km.FAULT_LAUNCH, 0)
    km.debug_withhold_stage(0, 0)
    for s in ("kmgb_debug_fail_nth", "kmgb_debug_withhold_stage", "kmgb_debug_pool_used_bytes"):
        assert getattr(lib, s) is not None
