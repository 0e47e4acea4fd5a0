"""The 32-row known-answer CSR copied into every reference test
(gcn/Block_gcn/test.py:4-6, Block/test.py:4-6,
benchmark-v3/spmm-benchmark/test/spmm_fp16/test_spmm_h_m.py:20-22)."""
import numpy as np

ROW = np.array([0, 6, 7, 8, 10, 10, 11, 13, 15, 18, 19, 19, 19, 20, 20, 20, 20, 24,
                25, 26, 28, 28, 29, 31, 33, 36, 37, 37, 37, 38, 38, 38, 38], np.int32)
COL = np.array([1, 2, 3, 11, 16, 21, 1, 1, 2, 24, 25, 16, 22, 0, 27, 0, 4, 25, 9, 27, 1, 3,
                11, 21, 1, 1, 2, 24, 25, 16, 22, 0, 27, 0, 4, 25, 9, 27], np.int32)
