"""Error metrics between two assemblies of the same CSR pattern.

The reference checks an assembly only through two Frobenius norms
(src/FEM.cc:59-98).  The FP32 path is measured against an FP64 assembly per
matrix with:

* max entry error relative to the diagonal scale, |dA_ij,ab| / sqrt(|A_ii,aa| |A_jj,bb|)
  (a plain relative error is meaningless for entries that cancel to ~0);
* the raw relative error |dA_ij,ab| / |A_ij,ab| over the values whose magnitude
  is at least tau times their diagonal scale, for several floors tau, with the
  count of values above 1e-6 and the share of values the floor keeps (an entry
  that cancels to 1e-4 of its scale carries the FP32 contributions' relative
  error times 1e4, whatever the summation);
* max entry error relative to max |A|;
* relative Frobenius error ||dA|| / ||A||;
* relative error of the preconditioned operator P A applied to seeded random
  vectors, ||P' A' x - P A x|| / ||P A x||.
"""
from __future__ import annotations

import numpy as np


def _diag_index(row, col):
    N = len(row) - 1
    r = np.repeat(np.arange(N), np.diff(row))
    pos = np.full(N, -1, np.int64)
    m = (col - 1) == r
    pos[r[m]] = np.nonzero(m)[0]
    return r, pos


def entry_errors(row, col, ref, test, dim: int, raw: bool = True) -> dict:
    R = np.asarray(ref, np.float64).reshape(-1, dim)
    T = np.asarray(test, np.float64).reshape(-1, dim)
    d = np.abs(T - R)
    r, dpos = _diag_index(row, col)
    c = col - 1
    if dim == 1:
        dg = np.abs(R[dpos, 0])
        scale = np.sqrt(dg[r] * dg[c])[:, None]
    else:
        dg = np.abs(R[dpos][:, [0, 4, 8]])                     # (N, 3)
        scale = np.sqrt(dg[r][:, :, None] * dg[c][:, None, :]).reshape(-1, 9)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(scale > 0, d / scale, 0.0)
    out = {"max_rel_diag_scaled": float(rel.max()),
           "max_rel_to_max": float(d.max() / np.abs(R).max()),
           "frobenius_rel": float(np.linalg.norm(T - R) / np.linalg.norm(R))}
    if raw:
        out["raw"] = raw_errors(R, d, scale)
    return out


def raw_errors(R, d, scale, floors=(0.1, 0.01, 0.001), bound: float = 1e-6) -> dict:
    """Raw relative errors |dA| / |A| per value, over the values with |A| >= tau *
    (diagonal scale) for each floor tau, and over every non-zero value."""
    A = np.abs(R)
    with np.errstate(divide="ignore", invalid="ignore"):
        raw = np.where(A > 0, d / A, 0.0)
        ratio = np.where(scale > 0, A / scale, np.inf)
    out = {}
    for tau in floors:
        sel = ratio >= tau
        r = raw[sel]
        out[f"tau_{tau:g}"] = {"max": float(r.max()) if r.size else 0.0,
                               "values_above_%g" % bound: int((r > bound).sum()),
                               "share_of_values": round(float(sel.mean()), 4)}
    nz = A > 0
    out["all_nonzero"] = {"max": float(raw[nz].max()), "values_above_%g" % bound: int((raw[nz] > bound).sum()),
                          "values": int(nz.sum())}
    return out


def _apply(row, col, vals, prec, dim, x):
    from scipy.sparse import bsr_matrix, csr_matrix
    N = len(row) - 1
    if dim == 1:
        A = csr_matrix((vals, col - 1, row), shape=(N, N))
        return prec * (A @ x)
    A = bsr_matrix((vals.reshape(-1, 3, 3), col - 1, row), shape=(3 * N, 3 * N))
    y = (A @ x).reshape(N, 3)
    P = prec.reshape(N, 3, 3)
    return np.einsum("nij,nj->ni", P, y).reshape(-1)


def operator_error(row, col, ref_vals, ref_prec, vals, prec, dim: int, seed: int = 7,
                   nvec: int = 3) -> float:
    rng = np.random.default_rng(seed)
    N = len(row) - 1
    bs = 1 if dim == 1 else 3
    worst = 0.0
    for _ in range(nvec):
        x = rng.standard_normal(N * bs)
        y0 = _apply(row, col, np.asarray(ref_vals, np.float64), ref_prec, dim, x)
        y1 = _apply(row, col, np.asarray(vals, np.float64), prec, dim, x)
        worst = max(worst, float(np.linalg.norm(y1 - y0) / np.linalg.norm(y0)))
    return worst
