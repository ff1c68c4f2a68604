"""Correctly rounded block-CSR products for the SpMV parity tests: every product
a x split into exact FP64 parts and each row summed by math.fsum, with the
bounds the device results are held to."""
import math

import numpy as np


def split(v):
    """Dekker's split: v = hi + lo with at most 26 significant bits in each, so
    that products of parts are exact in FP64."""
    c = v * 134217729.0          # 2^27 + 1
    hi = c - (c - v)
    return hi, v - hi


def exact_apply(row, col, vals, dim, x):
    """A x with every product split exactly and each row summed by math.fsum
    (correctly rounded), and the rows' sums of |a x|."""
    N = len(row) - 1
    a = vals.reshape(-1, dim, dim)
    xc = x.reshape(-1, dim)[col - 1][:, None, :]           # (nnz, 1, dim)
    ah, al = split(a)
    xh, xl = split(xc)
    parts = np.stack([ah * xh, ah * xl, al * xh, al * xl], axis=-1)   # (nnz, dim, dim, 4)
    mag = np.abs(a * xc).sum(axis=2)                        # (nnz, dim)
    y = np.empty((N, dim))
    m = np.empty((N, dim))
    for r in range(N):
        seg = parts[row[r]:row[r + 1]]
        for i in range(dim):
            y[r, i] = math.fsum(seg[:, i].ravel().tolist())
        m[r] = mag[row[r]:row[r + 1]].sum(axis=0)
    return y.reshape(-1), m.reshape(-1)


# Bounds relative to the row's sum of |a x|: FP64 values, the FMA chain of at
# most 81 products and the lane merges (each rounding within 2^-53 of that sum);
# FP32 values, the double-float sums (measured within 15 x 2^-48 on random rows
# by tests/spmv_df_check.cc).
BOUND = {"fp64": 2.0 ** -46, "fp32": 2.0 ** -44}
