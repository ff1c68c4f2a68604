import numpy as np

import pyoracle as O
from minifem import metrics
from minifem.meshgen import cube_mesh


def test_metrics_zero_for_identical_and_positive_for_perturbed():
    m = cube_mesh(5, seed=1, op="ela")
    r = O.full(m, op="ela")
    e = metrics.entry_errors(r["row"], r["col"], r["values"], r["values"], 9)
    assert e["max_rel_diag_scaled"] == 0 and e["frobenius_rel"] == 0
    assert metrics.operator_error(r["row"], r["col"], r["values"], r["prec"], r["values"], r["prec"], 9) == 0
    v = r["values"] * (1 + 1e-7 * np.cos(np.arange(r["values"].size)))
    e = metrics.entry_errors(r["row"], r["col"], r["values"], v, 9)
    assert 0 < e["frobenius_rel"] < 2e-7 and 0 < e["max_rel_diag_scaled"] < 1e-6
    op = metrics.operator_error(r["row"], r["col"], r["values"], r["prec"], v, r["prec"], 9)
    assert 0 < op < 1e-6


def test_metrics_lap():
    m = cube_mesh(5, seed=2, op="lap")
    r = O.full(m, op="lap")
    v = r["values"].astype(np.float32).astype(np.float64)
    e = metrics.entry_errors(r["row"], r["col"], r["values"], v, 1)
    assert e["max_rel_diag_scaled"] < 1e-6
    assert metrics.operator_error(r["row"], r["col"], r["values"], r["prec"], v, r["prec"], 1) < 1e-6
