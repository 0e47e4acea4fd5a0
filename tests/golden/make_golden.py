"""Generate the committed golden fixtures for the block conversion.

Runs the reference's own CPU conversion (``blockProcess_fp16_balance`` /
``blockProcess_tf32_balance``, gcn/Block_gcn/example.cpp:48-348, built from the
reference tree by ``oracle/build_ref.py`` into ``oracle/_ref/``) on

* the 32-row known-answer CSR that every reference test uses
  (gcn/Block_gcn/test.py:4-6, Block/test.py:4-6), and
* a few seeded random graphs with empty windows, hub rows, duplicate columns
  and a ragged last window,

for the window/wide/partSize triples the reference uses, and stores inputs and
outputs in ``tests/golden/blocks_golden.npz``.  The tests check both the C
oracle and the CUDA conversion against this file, so it pins the oracle to the
reference's actual output without needing the reference at test time.

Usage (needs the reference tree; run from the repo root):
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

FIXTURE_ROW = [0, 6, 7, 8, 10, 10, 11, 13, 15, 18, 19, 19, 19, 20, 20, 20, 20, 24,
               25, 26, 28, 28, 29, 31, 33, 36, 37, 37, 37, 38, 38, 38, 38]
FIXTURE_COL = [1, 2, 3, 11, 16, 21, 1, 1, 2, 24, 25, 16, 22, 0, 27, 0, 4, 25, 9, 27, 1, 3,
               11, 21, 1, 1, 2, 24, 25, 16, 22, 0, 27, 0, 4, 25, 9, 27]
CONFIGS = [(8, 8, 32), (8, 4, 32), (16, 8, 32), (8, 8, 1), (8, 4, 1), (8, 16, 2), (16, 16, 3)]


def random_graphs():
    rng = np.random.default_rng(20240611)
    graphs = []
    for g in range(4):
        n = [61, 203, 150, 517][g]
        lens = rng.integers(0, 10, size=n)
        if g == 1:
            lens[rng.integers(0, n)] = 700          # hub row -> many parts
        if g == 2:
            lens[8:40] = 0                          # empty windows
        if g == 3:
            lens[rng.integers(0, n, size=3)] = rng.integers(200, 400, size=3)
        rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
        col = rng.integers(0, n, size=int(rowptr[-1])).astype(np.int32)
        if g == 0:
            col[::7] = col[1::7][: col[::7].shape[0]]   # duplicates within rows
        graphs.append((rowptr, col))
    return graphs


def main():
    import torch
    from oracle import build_ref
    ref = build_ref.build()
    if ref is None:
        raise SystemExit("reference tree not present; cannot regenerate golden fixtures")
    out = {}
    graphs = [(np.array(FIXTURE_ROW, np.int32), np.array(FIXTURE_COL, np.int32))] + random_graphs()
    for gi, (rowptr, col) in enumerate(graphs):
        n = rowptr.shape[0] - 1
        lens = np.diff(rowptr).astype(np.float32)
        if gi == 0:
            d32 = np.ones(n, np.float32)
        else:
            d32 = torch.rsqrt(torch.from_numpy(np.maximum(lens, 1.0))).numpy()
        d16 = torch.from_numpy(d32).half().numpy()
        out["g%d_rowptr" % gi] = rowptr
        out["g%d_col" % gi] = col
        out["g%d_deg16" % gi] = d16
        out["g%d_deg32" % gi] = d32
        for (W, w, P) in CONFIGS:
            for kind, deg in (("fp16", d16), ("tf32", d32)):
                fn = ref.blockProcess_fp16_balance if kind == "fp16" else ref.blockProcess_tf32_balance
                res = fn(torch.from_numpy(rowptr), torch.from_numpy(col), torch.from_numpy(deg), W, w, P)
                key = "g%d_%s_%d_%d_%d" % (gi, kind, W, w, P)
                for name, t in zip(("rowptr", "col", "val", "window", "atomic"), res):
                    out[key + "_" + name] = t.numpy().copy()
    path = os.path.join(ROOT, "tests", "golden", "blocks_golden.npz")
    np.savez_compressed(path, n_graphs=np.int32(len(graphs)),
                        configs=np.array(CONFIGS, np.int32), **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
