"""The batched autotuner's header writer (kmeans_gb300/autotune.py, no GPU): the cost table that
KMGB_ASSIGN_AUTO reads holds, per family and (d, k) bucket, the measured GPU time per row and
iteration, in the layout batch.cu indexes (family, dimension bucket, center bucket)."""
import re

import numpy as np

from kmeans_gb300 import autotune


def test_header_holds_cost_per_row(tmp_path):
    rec = {"gpu": "test GPU", "date": "2026-01-01", "iters": 5, "buckets": {}}
    for d in autotune.DIMS:
        for k in autotune.KMAX:
            rows = max(256, 2 * k * k)
            rec["buckets"][f"d{d}_k{k}"] = {"problems": 10, "rows_each": rows,
                                            "fp32_ms_per_iter": 1e-6 * 10 * rows * (d + k),
                                            "bf16x3_ms_per_iter": 1e-6 * 10 * rows * d}
    out = tmp_path / "tuned.h"
    autotune.write_header(rec, str(out))
    text = out.read_text()
    assert "kTunedNsPerRow[2][%d][%d]" % (len(autotune.DIMS), len(autotune.KMAX)) in text
    body = text[text.index("kTunedNsPerRow"):]
    vals = [float(v) for v in re.findall(r"([0-9.eE+-]+)f", body)]
    table = np.array(vals).reshape(2, len(autotune.DIMS), len(autotune.KMAX))
    for i, d in enumerate(autotune.DIMS):
        for j, k in enumerate(autotune.KMAX):
            # ms per iteration * 1e6 / (problems * rows) = ns per row and iteration
            assert np.isclose(table[0, i, j], d + k, rtol=1e-4)
            assert np.isclose(table[1, i, j], d, rtol=1e-4)


def test_committed_header_matches_the_tuned_buckets():
    import os
    path = os.path.join(os.path.dirname(autotune.__file__), "csrc", "tuned_batched.h")
    text = open(path).read()
    dims = re.search(r"kTunedDims\[\] = \{([^}]*)\}", text).group(1)
    kmax = re.search(r"kTunedKMax\[\] = \{([^}]*)\}", text).group(1)
    assert [int(v) for v in dims.split(",")] == list(autotune.DIMS)
    assert [int(v) for v in kmax.split(",")] == list(autotune.KMAX)
