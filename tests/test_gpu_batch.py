"""The batched form with tuned tile sizes (many uneven lap/ela meshes, several
coefficient sets each, one graph replay per iteration) against the oracle, and
the accuracy-targeted sliver threshold of the tuner."""
import numpy as np
import pytest

import pyoracle as O
from minifem import metrics
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-6   # max entry error relative to the diagonal scale


def test_tuned_batch_fp64_bit_exact_and_fp32_within_tolerance(gpu):
    import minifem
    from minifem import autotune
    specs = [(6, "lap", 3), (13, "ela", 2), (9, "ela", 3), (15, "lap", 2), (11, "ela", 1)]
    b = minifem.Batch(0)
    items, pending = [], []
    for n, op, k in specs:
        meshes = [cube_mesh(n, seed=7 * n + s, op=op) for s in range(k)]
        m = meshes[0]
        a = gpu(0)
        a.set_mesh(m.coord, m.elemToNode)
        row, col = a.create_nodeToNode("reference")       # the oracle's column order
        a.set_check_bounds(O.checkbounds(m.boundNodesCode))
        a.set_coefficients(op, m.coef)
        cs = np.stack([mm.coef for mm in meshes])
        items.append((a, op, m, cs, row, col))
        pending.append((a, op, cs))
    tuned = autotune.tune_batch(pending, repeats=1)
    assert tuned["choice"]["fp32_kernel"] == 1 and len(tuned["timings"]) >= 2
    for a, op, m, cs, _, _ in items:
        b.add(a, op, cs)
    b.assemble("fp64", prec=True)
    b.synchronize()
    v64 = {(i, s): (b.values(i, s, "fp64"), b.prec(i, s)) for i, it in enumerate(items)
           for s in range(it[3].shape[0])}
    b.assemble("fp32", prec=True)
    b.synchronize()
    for i, (a, op, m, cs, row, col) in enumerate(items):
        for s in range(cs.shape[0]):
            ref = O.full(m, op=op, coef=cs[s])
            assert np.array_equal(ref["col"], col)
            got_v, got_p = v64[(i, s)]
            assert got_v.tobytes() == ref["values"].tobytes(), (i, s)
            assert got_p.tobytes() == ref["prec"].tobytes(), (i, s)
            e = metrics.entry_errors(row, col, ref["values"], b.values(i, s, "fp32"), O.op_dim(op),
                                     raw=False)
            assert e["max_rel_diag_scaled"] < TOL_FP32, (i, s, e)


def test_sliver_threshold_tuned_to_the_error_target(gpu):
    """A small stress mesh (jitter 0.45h, slivers, E jump 1e6, nu up to 0.45):
    the tuner returns the lowest threshold whose FP32 assembly is within 1e-6 of
    the FP64 one, and the assembly at that threshold is."""
    from minifem import autotune
    m = cube_mesh(16, seed=5, op="ela", jitter=0.45, sliver_fraction=0.05, jump=1e6, nu_max=0.45)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    a.set_coefficients("ela", m.coef)
    r = autotune.tune_sliver_threshold(a, "ela", row, col, target=TOL_FP32, repeats=1)
    assert r["errors"][str(r["choice"])] <= TOL_FP32
    lower = [float(q) for q in r["errors"] if float(q) < r["choice"]]
    assert all(r["errors"][str(q)] > TOL_FP32 for q in lower)
    a.assembly("ela", "fp64", "gather")
    v64 = a.values()
    a.assembly("ela", "fp32", "gather")
    e = metrics.entry_errors(row, col, v64, a.values(), 9)
    assert e["max_rel_diag_scaled"] <= TOL_FP32
